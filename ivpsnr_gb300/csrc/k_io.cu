// Input-side kernels around the metric path (all HBM bound, one thread per sample or pixel):
//   * 4:2:2 to 4:4:4 horizontal nearest-neighbour upsampling of raw frames
//     (xSeqBase::xUnpackFrame, libs/pmbb-core/src/xSeq.cpp:179-250, UpsampleH semantics);
//   * range check and concealment of out-of-range samples (xPixelOpsSTD::CheckIfInRange /
//     ClipToRange, libs/pmbb-core/src/xPixelOpsSTD.cpp:163-209, as xAppQMIV::validateFrames uses
//     them, apps/QMIV/src/xAppQMIV.cpp:753-770);
//   * fixed-point RGB <-> YCbCr conversion (xColorSpaceSTD::ConvertRGB2YCbCr_I32 /
//     ConvertYCbCr2RGB_I32, libs/pmbb-core/src/xColorSpaceSTD.cpp:195-272), 16-bit fraction.
#include "qmiv_io.h"

namespace qmiv {

namespace {

__device__ __forceinline__ int ld(const void* p, int sb, int64_t o)
{
  return sb == 1 ? (int)__ldg((const uint8_t*)p + o) : (int)__ldg((const uint16_t*)p + o);
}

// plain (coherent) load, for planes the same kernel writes (in-place clipping and conversion)
__device__ __forceinline__ int ld_rw(const void* p, int sb, int64_t o)
{
  return sb == 1 ? (int)((const uint8_t*)p)[o] : (int)((const uint16_t*)p)[o];
}

// dst (W x H, pitch W) from a chroma plane of W/2 x H: dst(x, y) = src(x >> 1, y)
__global__ void k_upsample_h(const void* __restrict__ src, int sbytes, int sstride, void* __restrict__ dst, int W, int H)
{
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if(x >= W || y >= H) return;
  const int v = ld(src, sbytes, (int64_t)y * sstride + (x >> 1));
  if(sbytes == 1) ((uint8_t*)dst)[(int64_t)y * W + x] = (uint8_t)v;
  else            ((uint16_t*)dst)[(int64_t)y * W + x] = (uint16_t)v;
}

// count samples above Max per plane; optionally clip them in place. grid.y is the component; a
// block walks rows (grid-stride over rows, threads over columns), 16-bit rows in 8-sample vectors
// when the row starts on 16 bytes, so no 64-bit division per sample.
__device__ __forceinline__ unsigned range_word(uint32_t& w, int maxv, int conceal)
{ // two 16-bit samples
  const int lo = (int)(w & 0xFFFFu), hi = (int)(w >> 16);
  const unsigned n = (unsigned)(lo > maxv) + (unsigned)(hi > maxv);
  if(conceal && n) w = (uint32_t)min(lo, maxv) | ((uint32_t)min(hi, maxv) << 16);
  return n;
}

__global__ void __launch_bounds__(256) k_range(RangeJob J)
{
  __shared__ unsigned int s_n[8];
  const int c = blockIdx.y;
  // fields of component c by selection: a runtime index into the parameter arrays would copy
  // them to local memory
  void* const plane = c == 0 ? J.plane[0] : (c == 1 ? J.plane[1] : J.plane[2]);
  const int stride = c == 0 ? J.stride[0] : (c == 1 ? J.stride[1] : J.stride[2]);
  const int w = c == 0 ? J.w[0] : (c == 1 ? J.w[1] : J.w[2]);
  const int h = c == 0 ? J.h[0] : (c == 1 ? J.h[1] : J.h[2]);
  const int maxv = J.maxv, conceal = J.conceal, sbytes = J.sbytes;
  unsigned int n = 0;
  const bool vec = sbytes == 2 && ((((uintptr_t)plane) | ((size_t)stride * 2)) & 15) == 0;
  for(int y = blockIdx.x; y < h; y += gridDim.x)
  {
    if(vec)
    {
      uint4* row = reinterpret_cast<uint4*>((uint16_t*)plane + (int64_t)y * stride);
      const int nv = w >> 3;
      for(int i0 = threadIdx.x; i0 < nv; i0 += 4 * blockDim.x)
      { // four independent 16-byte loads in flight per thread
        uint4 v[4];
        #pragma unroll
        for(int k = 0; k < 4; k++)
        {
          const int i = i0 + k * blockDim.x;
          if(i < nv) v[k] = row[i];
        }
        #pragma unroll
        for(int k = 0; k < 4; k++)
        {
          const int i = i0 + k * blockDim.x;
          if(i >= nv) break;
          const unsigned m = range_word(v[k].x, maxv, conceal) + range_word(v[k].y, maxv, conceal) +
                             range_word(v[k].z, maxv, conceal) + range_word(v[k].w, maxv, conceal);
          n += m;
          if(conceal && m) row[i] = v[k];
        }
      }
      for(int x = 8 * nv + threadIdx.x; x < w; x += blockDim.x)
      {
        uint16_t* p = (uint16_t*)plane + (int64_t)y * stride + x;
        if((int)*p > maxv) { n++; if(conceal) *p = (uint16_t)maxv; }
      }
    }
    else
      for(int x = threadIdx.x; x < w; x += blockDim.x)
      {
        const int64_t o = (int64_t)y * stride + x;
        const int v = ld_rw(plane, sbytes, o);
        if(v > maxv)
        {
          n++;
          if(conceal)
          {
            if(sbytes == 1) ((uint8_t*)plane)[o] = (uint8_t)maxv;
            else            ((uint16_t*)plane)[o] = (uint16_t)maxv;
          }
        }
      }
  }
  for(int d = 16; d > 0; d >>= 1) n += __shfl_xor_sync(0xffffffffu, n, d);
  if((threadIdx.x & 31) == 0) s_n[threadIdx.x >> 5] = n;
  __syncthreads();
  if(threadIdx.x == 0)
  {
    unsigned int t = 0;
    for(int k = 0; k < 8; k++) t += s_n[k];
    if(t) atomicAdd(J.count + c, (unsigned long long)t);
  }
}

__device__ __forceinline__ int clipu(int v, int mx) { return v < 0 ? 0 : (v > mx ? mx : v); }

__device__ __forceinline__ void color_px(const ColorJob& J, int a, int b, int c, int& o0, int& o1, int& o2)
{
  const int mid = 1 << (J.bd - 1), mx = (1 << J.bd) - 1;
  if(J.to_ycbcr)
  { // a, b, c = R, G, B (xColorSpaceSTD.cpp:195-232)
    const int ty = (J.m[0][0] * a + J.m[0][1] * b + J.m[0][2] * c + kColorAdd) >> kColorPrec;
    const int tu = (J.m[1][0] * a + J.m[1][1] * b + (c << (kColorPrec - 1)) + kColorAdd) >> kColorPrec;
    const int tv = ((a << (kColorPrec - 1)) + J.m[2][1] * b + J.m[2][2] * c + kColorAdd) >> kColorPrec;
    o0 = clipu(ty, mx); o1 = clipu(tu + mid, mx); o2 = clipu(tv + mid, mx);
  }
  else
  { // a, b, c = Y, Cb, Cr (xColorSpaceSTD.cpp:234-272)
    const int iu = b - mid, iv = c - mid;
    const int sy = (a << kColorPrec) + kColorAdd;
    o0 = clipu((sy + J.m[0][2] * iv) >> kColorPrec, mx);
    o1 = clipu((sy + J.m[1][1] * iu + J.m[1][2] * iv) >> kColorPrec, mx);
    o2 = clipu((sy + J.m[2][1] * iu) >> kColorPrec, mx);
  }
}

// four pixels per thread; 16-bit planes whose rows start on 8 bytes move as 4-sample vectors
__global__ void k_color(ColorJob J)
{
  const int x0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x), y = blockIdx.y;
  if(x0 >= J.W || y >= J.H) return;
  const int64_t so = (int64_t)y * J.sstride + x0, dof = (int64_t)y * J.dstride + x0;
  const bool vec = J.sbytes == 2 && x0 + 4 <= J.W &&
                   (((uintptr_t)J.src[0] | (uintptr_t)J.src[1] | (uintptr_t)J.src[2] | (uintptr_t)J.dst[0] |
                     (uintptr_t)J.dst[1] | (uintptr_t)J.dst[2] | ((size_t)J.sstride * 2) | ((size_t)J.dstride * 2)) & 7) == 0;
  if(vec)
  {
    uint2 in[3], outv[3];
    #pragma unroll
    for(int k = 0; k < 3; k++) in[k] = *reinterpret_cast<const uint2*>((const uint16_t*)J.src[k] + so);
    uint32_t o[3][2];
    #pragma unroll
    for(int h = 0; h < 2; h++)
    {
      const uint32_t a = h ? in[0].y : in[0].x, b = h ? in[1].y : in[1].x, c = h ? in[2].y : in[2].x;
      int p0, p1, p2, q0, q1, q2;
      color_px(J, (int)(a & 0xFFFFu), (int)(b & 0xFFFFu), (int)(c & 0xFFFFu), p0, p1, p2);
      color_px(J, (int)(a >> 16), (int)(b >> 16), (int)(c >> 16), q0, q1, q2);
      o[0][h] = (uint32_t)p0 | ((uint32_t)q0 << 16);
      o[1][h] = (uint32_t)p1 | ((uint32_t)q1 << 16);
      o[2][h] = (uint32_t)p2 | ((uint32_t)q2 << 16);
    }
    #pragma unroll
    for(int k = 0; k < 3; k++) { outv[k] = make_uint2(o[k][0], o[k][1]); *reinterpret_cast<uint2*>(J.dst[k] + dof) = outv[k]; }
    return;
  }
  for(int i = 0; i < 4 && x0 + i < J.W; i++)
  {
    const int a = ld_rw(J.src[0], J.sbytes, so + i), b = ld_rw(J.src[1], J.sbytes, so + i), c = ld_rw(J.src[2], J.sbytes, so + i);
    int o0, o1, o2;
    color_px(J, a, b, c, o0, o1, o2);
    J.dst[0][dof + i] = (uint16_t)o0;
    J.dst[1][dof + i] = (uint16_t)o1;
    J.dst[2][dof + i] = (uint16_t)o2;
  }
}

}  // namespace

void color_matrix(int space, bool to_ycbcr, int32_t m[3][3])
{ // base coefficients (Kr, Kg, Kb) of BT.601, BT.709, SMPTE 240M, BT.2020 (xColorSpaceCoeff.h:36-42)
  static const double base[4][3] = { { 0.299, 0.587, 0.114 }, { 0.2126, 0.7152, 0.0722 },
                                     { 0.2120, 0.7010, 0.0870 }, { 0.2627, 0.6780, 0.0593 } };
  const double kr = base[space][0], kg = base[space][1], kb = base[space][2];
  double d[3][3];
  if(to_ycbcr)
  {
    const double sb = 0.5 / (kb - 1.0), sr = 0.5 / (kr - 1.0);
    const double t[3][3] = { { kr, kg, kb }, { sb * kr, sb * kg, 0.5 }, { 0.5, sr * kg, sr * kb } };
    for(int i = 0; i < 3; i++) for(int j = 0; j < 3; j++) d[i][j] = t[i][j];
  }
  else
  {
    const double t[3][3] = { { 1.0, 0.0, 2 - 2 * kr },
                             { 1.0, 2.0 * (kb * kb - kb) / kg, 2.0 * (kr * kr - kr) / kg },
                             { 1.0, 2 - 2 * kb, 0.0 } };
    for(int i = 0; i < 3; i++) for(int j = 0; j < 3; j++) d[i][j] = t[i][j];
  }
  // 2^16 fraction bits, rounded half away from zero
  for(int i = 0; i < 3; i++)
    for(int j = 0; j < 3; j++)
    {
      const double v = 65536.0 * d[i][j];
      m[i][j] = v >= 0.0 ? (int32_t)(v + 0.5) : -(int32_t)(-v + 0.5);
    }
}

cudaError_t launch_upsample_h(const void* src, int sbytes, int sstride, void* dst, int W, int H, cudaStream_t st)
{
  k_upsample_h<<<dim3((W + 255) / 256, H), 256, 0, st>>>(src, sbytes, sstride, dst, W, H);
  return cudaGetLastError();
}

cudaError_t launch_range(const RangeJob& j, int sms, cudaStream_t st)
{
  const int hmax = std::max(j.h[0], std::max(j.h[1], j.h[2]));
  // about 8 blocks per SM over the three planes together
  const int blocks = std::max(1, std::min(hmax, (std::max(1, sms) * 8 + 2) / 3));
  k_range<<<dim3(blocks, 3), 256, 0, st>>>(j);
  return cudaGetLastError();
}

cudaError_t launch_color(const ColorJob& j, cudaStream_t st)
{
  k_color<<<dim3((j.W + 1023) / 1024, j.H), 256, 0, st>>>(j);
  return cudaGetLastError();
}

}  // namespace qmiv
