// Test-infrastructure harness around the reference QMIV metric library (pmbb-ivqm).
//
// This file is the checker's driver, not product code. It is compiled by
// oracle/build_ref.sh against the reference's own sources (never copied into this
// repository) and writes one JSON line per frame with every value the GPU path
// must reproduce, printed with 17 significant digits. It calls the processors the
// same way the QMIV application does (apps/QMIV/src/xAppQMIV.cpp:593-650 for set-up,
// :661-751 for the per-frame order), including the quirk that WS weights are only
// initialised on the PSNR processor (xAppQMIV.cpp:632).
//
// Usage:
//   qmiv_ref_harness -w W -h H -bd BD -cf 420|444 -i0 pic0.yuv -i1 pic1.yuv
//                    [-im mask.yuv -bdm 8] [-f frames] [-sr 2] [-erp] [-lat 180] [-lon 360]
//                    [-nth 4] [-ssim 0|1] [-dump prefix]
//
// -dump writes, per frame, the CPS argmin map of both directions (int8 index
// dy*(2B+1)+dx, row-major) and the two shift-compensated pictures (uint16 planar
// 4:4:4) so the GPU path can be compared element by element.

#include "xPic.h"
#include "xSeq.h"
#include "xThreadPool.h"
#include "xPixelOps.h"
#include "xIVPSNR.h"
#include "xSSIM.h"
#include "xGlobClrDiff.h"
#include "xShftCompPic.h"
#include "xCorrespPixelShift.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace PMBB_NAMESPACE;

namespace {

struct Args {
  int w = 0, h = 0, bd = 8, cf = 420, bdm = 8, frames = 1, sr = 2, nth = 4, lat = 180, lon = 360;
  bool erp = false, ssim = true;
  std::string i0, i1, im, dump;
};

bool parse(int argc, char** argv, Args& a)
{
  for(int i = 1; i < argc; i++)
  {
    std::string k = argv[i];
    auto next = [&](void) -> const char* { if(i + 1 >= argc) { std::exit(2); } return argv[++i]; };
    if     (k == "-w"   ) a.w      = std::atoi(next());
    else if(k == "-h"   ) a.h      = std::atoi(next());
    else if(k == "-bd"  ) a.bd     = std::atoi(next());
    else if(k == "-bdm" ) a.bdm    = std::atoi(next());
    else if(k == "-cf"  ) a.cf     = std::atoi(next());
    else if(k == "-f"   ) a.frames = std::atoi(next());
    else if(k == "-sr"  ) a.sr     = std::atoi(next());
    else if(k == "-nth" ) a.nth    = std::atoi(next());
    else if(k == "-lat" ) a.lat    = std::atoi(next());
    else if(k == "-lon" ) a.lon    = std::atoi(next());
    else if(k == "-erp" ) a.erp    = true;
    else if(k == "-ssim") a.ssim   = std::atoi(next()) != 0;
    else if(k == "-i0"  ) a.i0     = next();
    else if(k == "-i1"  ) a.i1     = next();
    else if(k == "-im"  ) a.im     = next();
    else if(k == "-dump") a.dump   = next();
    else { std::fprintf(stderr, "unknown arg %s\n", k.c_str()); return false; }
  }
  return a.w > 0 && a.h > 0 && !a.i0.empty() && !a.i1.empty();
}

// FNV-1a over the visible area of the three planes, used as a compact SCP fingerprint.
uint64_t fnv_planes(const xPicP& P)
{
  uint64_t hsh = 1469598103934665603ull;
  for(int c = 0; c < 3; c++)
  {
    const uint16* p = P.getAddr((eCmp)c);
    for(int y = 0; y < P.getHeight(); y++)
    {
      for(int x = 0; x < P.getWidth(); x++)
      {
        uint16 v = p[y * P.getStride() + x];
        hsh ^= (uint64_t)(v & 0xFF); hsh *= 1099511628211ull;
        hsh ^= (uint64_t)(v >> 8  ); hsh *= 1099511628211ull;
      }
    }
  }
  return hsh;
}

void write_planes(const xPicP& P, FILE* f)
{
  for(int c = 0; c < 3; c++)
  {
    const uint16* p = P.getAddr((eCmp)c);
    for(int y = 0; y < P.getHeight(); y++) { std::fwrite(p + y * P.getStride(), sizeof(uint16), P.getWidth(), f); }
  }
}

// CPS argmin map for one direction through the reference's public static search
// (xCorrespPixelShift.cpp:48), returned as the window index dy*(2B+1)+dx.
std::vector<int8_t> cps_map(const xPicP& Tst, const xPicP& Ref, const int32V4& GCD, int32 SR, const int32V4& W)
{
  std::vector<int8_t> Map((size_t)Tst.getWidth() * Tst.getHeight());
  const int32 Stride = Ref.getStride();
  for(int32 y = 0; y < Tst.getHeight(); y++)
  {
    for(int32 x = 0; x < Tst.getWidth(); x++)
    {
      const int32 o = y * Tst.getStride() + x;
      int32V4 T = int32V4((int32)Tst.getAddr(eCmp::LM)[o], (int32)Tst.getAddr(eCmp::CB)[o], (int32)Tst.getAddr(eCmp::CR)[o], 0) + GCD;
      int32 Best = xCorrespPixelShift::xFindBestPixelWithinBlock(T, &Ref, x, y, SR, W);
      // Best = (y+dy)*Stride + (x+dx); recover dy,dx with the margin-safe floor division.
      int32 rel = Best - (y * Stride + x) + SR * Stride + SR;
      int32 dy = rel / Stride, dx = rel % Stride;
      Map[(size_t)y * Tst.getWidth() + x] = (int8_t)(dy * (2 * SR + 1) + dx);
    }
  }
  return Map;
}

} // namespace

int main(int argc, char** argv)
{
  Args a;
  if(!parse(argc, argv, a)) { std::fprintf(stderr, "bad arguments\n"); return 2; }

  const int32V2 Size(a.w, a.h);
  const int32   Margin = xRoundUpToNearestMultiple(a.sr, 2); // xAppQMIV.cpp:330
  const eCrF    CF     = (eCrF)a.cf;
  const bool    UseMask = !a.im.empty();

  xSeq Seq0(Size, a.bd, CF), Seq1(Size, a.bd, CF), SeqM(Size, a.bdm, CF);
  if(!Seq0.openFile(a.i0, xSeqBase::eMode::Read)) { std::fprintf(stderr, "cannot open %s\n", a.i0.c_str()); return 1; }
  if(!Seq1.openFile(a.i1, xSeqBase::eMode::Read)) { std::fprintf(stderr, "cannot open %s\n", a.i1.c_str()); return 1; }
  if(UseMask && !SeqM.openFile(a.im, xSeqBase::eMode::Read)) { std::fprintf(stderr, "cannot open %s\n", a.im.c_str()); return 1; }

  xPicP P0(Size, a.bd, Margin), P1(Size, a.bd, Margin), PM(Size, a.bdm, Margin);
  xPicI I0(Size, a.bd, Margin), I1(Size, a.bd, Margin);
  xPicP SCP0(Size, a.bd, Margin), SCP1(Size, a.bd, Margin);

  xThreadPool Pool; Pool.create(a.nth, a.h + 1);

  const int32V4 W = xCorrespPixelShiftPrms::c_DefaultCmpWeights;
  const flt32V4 Unc = xGlobClrDiffPrms::c_DefaultUnntcbCoef;

  xIVPSNRM ProcPSNR;
  ProcPSNR.setSearchRange(a.sr); ProcPSNR.setCmpWeightsSearch(W); ProcPSNR.setCmpWeightsAverage(W); ProcPSNR.setUnntcbCoef(Unc);
  ProcPSNR.initThreadPool(&Pool, a.h + 1);
  ProcPSNR.initRowBuffers(a.h);
  if(a.erp) { ProcPSNR.initWS(true, a.w, a.h, a.bd, a.lon, a.lat); }
  flt64 LastR2T = 0, LastT2R = 0; int32V4 DbgGCD = { 0, 0, 0, 0 };
  ProcPSNR.setDebugCallbackQAP([&](flt64 R2T, flt64 T2R) { LastR2T = R2T; LastT2R = T2R; });

  xGlobClrDiffProc ProcGCD; ProcGCD.setUnntcbCoef(Unc); ProcGCD.initThreadPool(&Pool, a.h + 1);
  xShftCompPicProc ProcSCP; ProcSCP.setSearchRange(a.sr); ProcSCP.setCmpWeightsSearch(W); ProcSCP.setCmpWeightsAverage(W); ProcSCP.initThreadPool(&Pool, a.h + 1);

  xIVSSIM ProcSSIM;
  flt64 SsimR2T = 0, SsimT2R = 0;
  if(a.ssim && !UseMask)
  {
    ProcSSIM.create(Size, a.bd, Margin, true);
    ProcSSIM.setSearchRange(a.sr); ProcSSIM.setCmpWeightsSearch(W); ProcSSIM.setCmpWeightsAverage(W); ProcSSIM.setUnntcbCoef(Unc);
    ProcSSIM.initThreadPool(&Pool, a.h + 1);
    ProcSSIM.initRowBuffers(a.h);
    ProcSSIM.setDebugCallbackQAP([&](flt64 R2T, flt64 T2R) { SsimR2T = R2T; SsimT2R = T2R; });
  }
  (void)DbgGCD;

  for(int f = 0; f < a.frames; f++)
  {
    if(!Seq0.readFrame(&P0) || !Seq1.readFrame(&P1)) { std::fprintf(stderr, "read error frame %d\n", f); return 1; }
    if(UseMask && !SeqM.readFrame(&PM)) { std::fprintf(stderr, "mask read error frame %d\n", f); return 1; }

    bool Exact[3];
    for(int c = 0; c < 3; c++) { Exact[c] = P0.equalCmp(&P1, (eCmp)c); } // xAppQMIV.cpp:773-776
    P0.extend(); P1.extend(); if(UseMask) { PM.extend(); }
    I0.rearrangeFromPlanar(&P0); I1.rearrangeFromPlanar(&P1);

    std::printf("{\"frame\": %d", f);
    std::printf(", \"exact\": [%d, %d, %d]", (int)Exact[0], (int)Exact[1], (int)Exact[2]);

    if(!UseMask)
    {
      const int32V4 GCD = ProcGCD.CalcGlobalColorDiff(&P0, &P1); // xAppQMIV.cpp:696
      std::printf(", \"gcd\": [%d, %d, %d]", GCD[0], GCD[1], GCD[2]);

      flt64V4 PSNR = ProcPSNR.calcPicPSNR(&P0, &P1);
      flt64V4 WSPSNR = ProcPSNR.calcPicWSPSNR(&P0, &P1);
      for(int c = 0; c < 3; c++) { if(Exact[c]) { PSNR[c] = ProcPSNR.getFakePSNR(P0.getArea(), P0.getBitDepth()); WSPSNR[c] = PSNR[c]; } } // xAppQMIV.cpp:837-844
      std::printf(", \"psnr\": [%.17g, %.17g, %.17g]", PSNR[0], PSNR[1], PSNR[2]);
      std::printf(", \"wspsnr\": [%.17g, %.17g, %.17g]", WSPSNR[0], WSPSNR[1], WSPSNR[2]);

      flt64 IVI = ProcPSNR.calcPicIVPSNR(&I0, &I1, GCD); // interleaved (SSE path on x86)
      std::printf(", \"ivpsnr\": %.17g, \"ivpsnr_r2t\": %.17g, \"ivpsnr_t2r\": %.17g", IVI, LastR2T, LastT2R);
      flt64 IVP = ProcPSNR.calcPicIVPSNR(&P0, &P1, GCD); // planar
      std::printf(", \"ivpsnr_planar\": %.17g", IVP);

      // exact per-component CPS SSE sums for both directions (xCorrespPixelShift.cpp:20)
      const int32V4 NegGCD = -GCD;
      uint64V4 S0 = { 0, 0, 0, 0 }, S1 = { 0, 0, 0, 0 };
      for(int32 y = 0; y < a.h; y++)
      {
        S0 += xCorrespPixelShift::xCalcDistAsymmetricRow(&P0, &P1, y, GCD, a.sr, W);
        S1 += xCorrespPixelShift::xCalcDistAsymmetricRow(&P1, &P0, y, NegGCD, a.sr, W);
      }
      std::printf(", \"sse_r2t\": [%llu, %llu, %llu], \"sse_t2r\": [%llu, %llu, %llu]",
        (unsigned long long)S0[0], (unsigned long long)S0[1], (unsigned long long)S0[2],
        (unsigned long long)S1[0], (unsigned long long)S1[1], (unsigned long long)S1[2]);

      ProcSCP.GenShftCompPics(&SCP1, &SCP0, &P1, &P0, GCD); // xAppQMIV.cpp:703
      std::printf(", \"scp0_fnv\": \"%016llx\", \"scp1_fnv\": \"%016llx\"", (unsigned long long)fnv_planes(SCP0), (unsigned long long)fnv_planes(SCP1));

      if(a.ssim)
      {
        flt64V4 SSIM   = ProcSSIM.calcPicSSIM  (&P0, &P1);
        flt64V4 MSSSIM = ProcSSIM.calcPicMSSSIM(&P0, &P1);
        flt64   IVSSIM = ProcSSIM.calcPicIVSSIM(&P0, &P1, &SCP0, &SCP1);
        std::printf(", \"ssim\": [%.17g, %.17g, %.17g]", SSIM[0], SSIM[1], SSIM[2]);
        std::printf(", \"msssim\": [%.17g, %.17g, %.17g]", MSSSIM[0], MSSSIM[1], MSSSIM[2]);
        std::printf(", \"ivssim\": %.17g, \"ivssim_r2t\": %.17g, \"ivssim_t2r\": %.17g", IVSSIM, SsimR2T, SsimT2R);
      }

      if(!a.dump.empty())
      {
        std::string fn = a.dump + "_f" + std::to_string(f);
        std::vector<int8_t> M0 = cps_map(P0, P1, GCD, a.sr, W);
        std::vector<int8_t> M1 = cps_map(P1, P0, NegGCD, a.sr, W);
        FILE* fm = std::fopen((fn + "_cps.bin").c_str(), "wb");
        std::fwrite(M0.data(), 1, M0.size(), fm); std::fwrite(M1.data(), 1, M1.size(), fm); std::fclose(fm);
        FILE* fs = std::fopen((fn + "_scp.bin").c_str(), "wb");
        write_planes(SCP0, fs); write_planes(SCP1, fs); std::fclose(fs);
      }
    }
    else
    {
      const int32 NNM = xPixelOps::CountNonZero(PM.getAddr(eCmp::LM), PM.getStride(), PM.getWidth(), PM.getHeight());
      const int32V4 GCD = ProcGCD.CalcGlobalColorDiffM(&P0, &P1, &PM, NNM); // xAppQMIV.cpp:695
      std::printf(", \"nnm\": %d, \"gcd\": [%d, %d, %d]", NNM, GCD[0], GCD[1], GCD[2]);
      flt64V4 PSNR = ProcPSNR.calcPicPSNRM(&P0, &P1, &PM, NNM);
      flt64V4 WSPSNR = ProcPSNR.calcPicWSPSNRM(&P0, &P1, &PM, NNM);
      for(int c = 0; c < 3; c++) { if(Exact[c]) { PSNR[c] = ProcPSNR.getFakePSNR(P0.getArea(), P0.getBitDepth()); WSPSNR[c] = PSNR[c]; } }
      std::printf(", \"psnr\": [%.17g, %.17g, %.17g]", PSNR[0], PSNR[1], PSNR[2]);
      std::printf(", \"wspsnr\": [%.17g, %.17g, %.17g]", WSPSNR[0], WSPSNR[1], WSPSNR[2]);
      flt64 IV = ProcPSNR.calcPicIVPSNRM(&I0, &I1, &PM, NNM, GCD); // xAppQMIV.cpp:888
      std::printf(", \"ivpsnr\": %.17g, \"ivpsnr_r2t\": %.17g, \"ivpsnr_t2r\": %.17g", IV, LastR2T, LastT2R);
    }
    std::printf("}\n");
  }

  if(a.ssim && !UseMask) { ProcSSIM.destroy(); }
  ProcPSNR.uninitThreadPool(); ProcGCD.uninitThreadPool(); ProcSCP.uninitThreadPool();
  if(a.ssim && !UseMask) { ProcSSIM.uninitThreadPool(); }
  Pool.destroy();
  return 0;
}
