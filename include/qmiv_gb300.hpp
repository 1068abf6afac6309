/* qmiv_gb300.hpp — header-only C++17 processors over the C ABI of qmiv_gb300.h, with the
 * method names and argument meaning of the reference's metric processors, so that host code
 * written against them (apps/QMIV/src/xAppQMIV.cpp) switches by changing the class it
 * instantiates:
 *
 *   xPSNR   (libs/pmbb-ivqm/src/xPSNR.h:33)         -> qmiv_gpu::xPSNR_GPU::calcPicPSNR
 *   xWSPSNR (xWSPSNR.h:20-23, xWeightedSpherically.h:21) -> qmiv_gpu::xWSPSNR_GPU::calcPicWSPSNR
 *   xIVPSNR (xIVPSNR.h:32-35, xCorrespPixelShift.h:42-44, xGlobClrDiff.h:24,41)
 *                                                   -> qmiv_gpu::xIVPSNR_GPU::calcPicIVPSNR
 *   xSSIM   (xSSIM.h:40-44)                         -> qmiv_gpu::xSSIM_GPU::calcPicSSIM / calcPicMSSSIM
 *   xIVSSIM (xSSIM.h:74-78)                         -> qmiv_gpu::xIVSSIM_GPU::calcPicIVSSIM
 *   xShftCompPicProc::GenShftCompPics (xShftCompPic.h:33-44) -> qmiv_gpu::xIVPSNR_GPU::GenShftCompPics
 *
 * Pictures are qmiv_pic descriptors (see make_pic_planar for the xPicP mapping). "Tst" is
 * the application's picture 0 and "Ref" its picture 1, as in xAppQMIV. Failures throw
 * qmiv_gpu::Error with the library's message; the reference asserts instead. */
#ifndef QMIV_GB300_HPP
#define QMIV_GB300_HPP

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "qmiv_gb300.h"

namespace qmiv_gpu {

using int32V4 = std::array<int32_t, 4>;
using flt32V4 = std::array<float, 4>;
using flt64V4 = std::array<double, 4>;

struct Error : std::runtime_error {
  qmiv_status status;
  Error(qmiv_status s, const char* where)
    : std::runtime_error(std::string(where) + ": " + qmiv_status_str(s) + " (" + qmiv_last_error() + ")"), status(s) {}
};

inline void check(qmiv_status s, const char* where) { if(s != QMIV_OK) throw Error(s, where); }

/* A planar picture: origin pointers of the three planes (xPicP::getAddr(eCmp), i.e. past the
 * margin), row stride in samples (xPicP::getStride()), luma size and bit depth. The margin
 * is ignored: borders are handled by clamping, which equals the reference's edge replication.
 * chroma_format QMIV_CF444 for xPicP's 4:4:4 planes, QMIV_CF420 for native 4:2:0 planes. */
template <typename T>
inline qmiv_pic make_pic_planar(const T* y, const T* cb, const T* cr, int32_t stride, int32_t chroma_stride,
                                int32_t width, int32_t height, int32_t bitdepth, int32_t chroma_format, bool on_device)
{
  qmiv_pic p{};
  p.plane[0] = y; p.plane[1] = cb; p.plane[2] = cr;
  p.stride[0] = stride; p.stride[1] = chroma_stride; p.stride[2] = chroma_stride;
  p.width = width; p.height = height; p.bitdepth = bitdepth;
  p.sample_bytes = (int32_t)sizeof(T);
  p.chroma_format = chroma_format;
  p.is_device = on_device ? 1 : 0;
  return p;
}

/* Shared processor state: the options of the reference's setters and one handle, created on
 * first use (or by create) for the largest picture seen so far. */
class xMetricProcGPU {
public:
  xMetricProcGPU() { qmiv_default_options(&m_Opt); }
  virtual ~xMetricProcGPU() { destroy(); }
  xMetricProcGPU(const xMetricProcGPU&) = delete;
  xMetricProcGPU& operator=(const xMetricProcGPU&) = delete;

  /* xCorrespPixelShift.h:42-44 */
  void setSearchRange(int32_t SearchRange) { m_Opt.search_range = SearchRange; xUpdate(); }
  void setCmpWeightsSearch(const int32V4& W) { for(int c = 0; c < 4; c++) m_Opt.cmp_w_search[c] = W[c]; xUpdate(); }
  void setCmpWeightsAverage(const int32V4& W) { for(int c = 0; c < 4; c++) m_Opt.cmp_w_avg[c] = W[c]; xUpdate(); }
  /* xGlobClrDiff.h:24 */
  void setUnntcbCoef(const flt32V4& U) { for(int c = 0; c < 4; c++) m_Opt.unnoticeable[c] = U[c]; xUpdate(); }
  /* xPSNR.h:31, xWSPSNR.h:20 */
  void setFakeValsForExact(bool F) { m_Opt.fake_exact = F ? 1 : 0; xUpdate(); }
  void setLegacyWS8bit(bool L) { m_Opt.legacy_ws8 = L ? 1 : 0; xUpdate(); }
  /* xWeightedSpherically.h:21: the reference precomputes row weights here; the GPU library
   * computes and caches them on first use for each picture height. */
  void initWS(bool UseWS, int32_t Width, int32_t Height, int32_t /*BitDepth*/, int32_t LonRangeDeg = 360,
              int32_t LatRangeDeg = 180)
  {
    m_Opt.use_ws = UseWS ? 1 : 0; m_Opt.lon_deg = LonRangeDeg; m_Opt.lat_deg = LatRangeDeg;
    xReserve(Width, Height);
    xUpdate();
  }
  /* choose the SSIM window: QMIV_SSIM_REF10 (the reference's) or QMIV_SSIM_GAUSS11 */
  void setSSIMWindow(int32_t Window) { m_Opt.ssim_window = Window; xUpdate(); }
  void setStream(qmiv_stream S) { m_Stream = S; }

  void create(int32_t MaxWidth, int32_t MaxHeight) { xReserve(MaxWidth, MaxHeight); }
  void destroy() { if(m_H) { qmiv_destroy(m_H); m_H = nullptr; } }
  qmiv_handle* handle(const qmiv_pic& P) { xReserve(P.width, P.height); return m_H; }
  const qmiv_options& options() const { return m_Opt; }

protected:
  void xReserve(int32_t W, int32_t H)
  {
    if(m_H && W <= m_MaxW && H <= m_MaxH) return;
    destroy();
    m_MaxW = W > m_MaxW ? W : m_MaxW;
    m_MaxH = H > m_MaxH ? H : m_MaxH;
    check(qmiv_create(&m_H, &m_Opt, m_MaxW, m_MaxH, 1), "qmiv_create");
  }
  void xUpdate() { if(m_H) check(qmiv_set_options(m_H, &m_Opt), "qmiv_set_options"); }

  qmiv_options m_Opt{};
  qmiv_handle* m_H = nullptr;
  int32_t m_MaxW = 0, m_MaxH = 0;
  qmiv_stream m_Stream = nullptr;
};

class xPSNR_GPU : public xMetricProcGPU {
public:
  /* xPSNR::calcPicPSNR (xPSNR.cpp:17) */
  flt64V4 calcPicPSNR(const qmiv_pic* Tst, const qmiv_pic* Ref)
  {
    flt64V4 r{};
    check(qmiv_psnr(handle(*Tst), Tst, Ref, r.data(), nullptr, m_Stream), "calcPicPSNR");
    return r;
  }
};

class xWSPSNR_GPU : public xMetricProcGPU {
public:
  /* xWSPSNR::calcPicWSPSNR (xWSPSNR.cpp:17); plain PSNR when initWS was given UseWS = false */
  flt64V4 calcPicWSPSNR(const qmiv_pic* Tst, const qmiv_pic* Ref)
  {
    flt64V4 r{};
    check(qmiv_psnr(handle(*Tst), Tst, Ref, nullptr, r.data(), m_Stream), "calcPicWSPSNR");
    return r;
  }
};

class xIVPSNR_GPU : public xMetricProcGPU {
public:
  /* xIVPSNR::calcPicIVPSNR(Tst, Ref) (xIVPSNR.cpp:18-28): GCD computed here */
  double calcPicIVPSNR(const qmiv_pic* Tst, const qmiv_pic* Ref)
  {
    double iv = 0;
    check(qmiv_ivpsnr(handle(*Tst), Tst, Ref, nullptr, &iv, nullptr, nullptr, m_Stream), "calcPicIVPSNR");
    return iv;
  }
  /* xIVPSNR::calcPicIVPSNR(Tst, Ref, GlobalColorDiffRef2Tst) (xIVPSNR.cpp:32-56) */
  double calcPicIVPSNR(const qmiv_pic* Tst, const qmiv_pic* Ref, const int32V4& GlobalColorDiffRef2Tst)
  {
    double iv = 0;
    check(qmiv_ivpsnr(handle(*Tst), Tst, Ref, GlobalColorDiffRef2Tst.data(), &iv, nullptr, nullptr, m_Stream),
          "calcPicIVPSNR");
    return iv;
  }
  /* xGlobClrDiffProc::CalcGlobalColorDiff(Tst, Ref) (xGlobClrDiff.h:41) */
  int32V4 CalcGlobalColorDiff(const qmiv_pic* Tst, const qmiv_pic* Ref)
  {
    int32V4 g{};
    check(qmiv_gcd(handle(*Tst), Tst, Ref, g.data(), m_Stream), "CalcGlobalColorDiff");
    return g;
  }
  /* xShftCompPicProc::GenShftCompPics(DstRef, DstTst, SrcRef, SrcTst, GCD) (xShftCompPic.h:33-44):
   * 4:4:4 uint16 outputs, host or device planes per dst_on_device */
  void GenShftCompPics(uint16_t* DstRef[3], uint16_t* DstTst[3], int32_t DstStride, bool DstOnDevice,
                       const qmiv_pic* SrcRef, const qmiv_pic* SrcTst, const int32V4& GlobalColorDiffRef2Tst)
  { // the library's scp0 is built from picture 0 (Tst), scp1 from picture 1 (Ref)
    check(qmiv_scp(handle(*SrcTst), SrcTst, SrcRef, GlobalColorDiffRef2Tst.data(), DstTst, DstRef, DstStride,
                   DstOnDevice ? 1 : 0, m_Stream), "GenShftCompPics");
  }
};

class xSSIM_GPU : public xMetricProcGPU {
public:
  /* xSSIM::create(Size, BitDepth, Margin, EnableMS) (xSSIM.h:40) */
  void create(int32_t Width, int32_t Height, int32_t /*BitDepth*/, int32_t /*Margin*/, bool /*EnableMS*/)
  {
    xMetricProcGPU::create(Width, Height);
  }
  /* xSSIM::calcPicSSIM(Tst, Ref, CalcL) (xSSIM.cpp:54) */
  flt64V4 calcPicSSIM(const qmiv_pic* Tst, const qmiv_pic* Ref, bool CalcL = true)
  {
    flt64V4 r{};
    check(qmiv_ssim(handle(*Tst), Tst, Ref, CalcL ? 1 : 0, r.data(), m_Stream), "calcPicSSIM");
    return r;
  }
  /* xSSIM::calcPicMSSSIM(Tst, Ref) (xSSIM.cpp:67-87) */
  flt64V4 calcPicMSSSIM(const qmiv_pic* Tst, const qmiv_pic* Ref)
  {
    flt64V4 r{};
    check(qmiv_msssim(handle(*Tst), Tst, Ref, r.data(), m_Stream), "calcPicMSSSIM");
    return r;
  }
};

class xIVSSIM_GPU : public xSSIM_GPU {
public:
  /* xIVSSIM::calcPicIVSSIM(Tst, Ref) (xSSIM.cpp:166-190): GCD and SCPs built here */
  double calcPicIVSSIM(const qmiv_pic* Tst, const qmiv_pic* Ref)
  {
    double iv = 0;
    check(qmiv_ivssim(handle(*Tst), Tst, Ref, nullptr, &iv, nullptr, nullptr, m_Stream), "calcPicIVSSIM");
    return iv;
  }
};

}  // namespace qmiv_gpu

#endif
