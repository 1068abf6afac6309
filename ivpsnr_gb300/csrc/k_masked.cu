// Masked GCD, PSNR, WS-PSNR and IV-PSNR of one picture pair with a per-pixel mask picture:
//   GCD-M    xGlobClrDiff::CalcGlobalColorDiffM   libs/pmbb-ivqm/src/xGlobClrDiff.cpp:52-83
//   PSNR-M   xPSNR::calcPicPSNRM                  xPSNR.cpp:42-121,148-155
//   WS-PSNR-M xWSPSNR::calcPicWSPSNRM             xWSPSNR.cpp:61,150-159
//   IV-PSNR-M xIVPSNRM::calcPicIVPSNRM            xIVPSNR.cpp:138-200 with
//             xCorrespPixelShiftSTD::CalcDistAsymmetricRowM  xCorrespPixelShiftSTD.cpp:80-138
// The mask has luma resolution and weights every component of a 4:4:4 pixel (4:2:0 chroma is
// read at (x>>1, y>>1)). Pixels with mask 0 are skipped as tested pixels and as search
// candidates; errors are weighted by the mask value; the dB step uses the non-masked count
// and the mask's peak: 10 log10(NumNonMasked * Max^2 * MaxMask / SSD). Integer sums are exact
// (64-bit), so results do not depend on the launch shape. The search stages a 32x16 tile of
// both pictures and the mask (halo of the search range, edge samples replicated, which equals
// the reference's clamped reads) in shared memory; its costs are 32-bit when the largest
// possible cost fits, 64-bit otherwise.
#include "qmiv_device.cuh"
#include "qmiv_masked.h"

namespace qmiv {

namespace {

__device__ __forceinline__ int smp(const void* p, int sb, int64_t o)
{
  return sb == 1 ? (int)__ldg((const uint8_t*)p + o) : (int)__ldg((const uint16_t*)p + o);
}

__device__ __forceinline__ int pel(const MaskJob& J, int pic, int c, int x, int y)
{
  const int sh = c ? J.cshift : 0;
  const void* p = pic == 0 ? J.p0[c] : J.p1[c];
  const int s = pic == 0 ? J.s0[c] : J.s1[c];
  return smp(p, J.sbytes, (int64_t)(y >> sh) * s + (x >> sh));
}

__device__ __forceinline__ int msk(const MaskJob& J, int x, int y)
{
  return smp(J.mask, J.msbytes, (int64_t)y * J.mstride + x);
}

__device__ __forceinline__ double psnr_masked(double ssd, int64_t nnm, int bd, int mbd)
{ // CalcPSNRfromMaskedSSD (xPSNR.cpp:148-155)
  const double mp = (double)((1 << bd) - 1), mm = (double)((1 << mbd) - 1);
  const double MAX = __dmul_rn(__dmul_rn((double)nnm, __dmul_rn(mp, mp)), mm);
  return ssd > 0 ? __dmul_rn(10.0, log10(__ddiv_rn(MAX, ssd))) : DBL_MAX;
}

// per-row sums, two rows per block (four warps per row); the last block forms GCD-M, PSNR-M
// and WS-PSNR-M
__global__ void __launch_bounds__(256) k_masked_stats(MaskJob J)
{
  __shared__ bool is_last;
  __shared__ double scratch[16];
  __shared__ long long s_part[2][4][kMaskRowVals];
  const int lane = threadIdx.x & 31, half = threadIdx.x >> 7, tr = threadIdx.x & 127;
  const int y = blockIdx.x * 2 + half;
  {
    long long sd[3] = { 0, 0, 0 };
    unsigned long long ssd[3] = { 0, 0, 0 };
    int nnz = 0, dif[3] = { 0, 0, 0 };
    if(y < J.H)
      for(int x = tr; x < J.W; x += 128)
      {
        const int m = msk(J, x, y);
        nnz += m != 0;
        for(int c = 0; c < 3; c++)
        {
          const int d = pel(J, 1, c, x, y) - pel(J, 0, c, x, y);
          sd[c] += (long long)d * m;
          ssd[c] += (unsigned long long)((long long)d * d) * (unsigned long long)m;
          dif[c] += d != 0;
        }
      }
    long long v[kMaskRowVals];
    for(int c = 0; c < 3; c++) { v[c] = warp_sum(sd[c]); v[3 + c] = (long long)warp_sum(ssd[c]); v[7 + c] = warp_sum(dif[c]); }
    v[6] = warp_sum(nnz);
    if(lane == 0)
      for(int i = 0; i < kMaskRowVals; i++) s_part[half][tr >> 5][i] = v[i];
  }
  __syncthreads();
  if(y < J.H && tr < kMaskRowVals)
    J.rows[(int64_t)y * kMaskRowVals + tr] = s_part[half][0][tr] + s_part[half][1][tr] + s_part[half][2][tr] + s_part[half][3][tr];
  if(y < J.H && tr < 6) J.cps_rows[((int64_t)(tr / 3) * J.H + y) * 3 + tr % 3] = 0ull;
  __threadfence();
  __syncthreads();
  if(threadIdx.x == 0) is_last = atomicAdd(&J.counters[0], 1u) == gridDim.x - 1;
  __syncthreads();
  if(!is_last) return;
  __threadfence();
  // totals over rows: sd, ssd, nnz, any difference (fixed per-thread order, then block sums)
  long long t[10];
  for(int i = 0; i < 10; i++) t[i] = 0;
  for(int r = threadIdx.x; r < J.H; r += blockDim.x)
    for(int i = 0; i < 10; i++) t[i] += __ldcg(J.rows + (int64_t)r * kMaskRowVals + i);
  __shared__ long long s_t[8][10];
  for(int i = 0; i < 10; i++)
  {
    const long long w = warp_sum(t[i]);
    if(lane == 0) s_t[threadIdx.x >> 5][i] = w;
  }
  __syncthreads();
  __shared__ long long tot[10];
  if(threadIdx.x < 10)
  {
    long long s = 0;
    for(int w = 0; w < 8; w++) s += s_t[w][threadIdx.x];
    tot[threadIdx.x] = s;
  }
  __syncthreads();
  double ws[3] = { 0, 0, 0 };
  if(J.use_ws && (J.metrics & QMIV_M_WSPSNR))
    for(int c = 0; c < 3; c++)
    {
      Kbns k = { 0.0, 0.0 };
      for(int r = threadIdx.x; r < J.H; r += blockDim.x)
        k = kbns_add(k, __dmul_rn((double)(unsigned long long)__ldcg(J.rows + (int64_t)r * kMaskRowVals + 3 + c), J.ws[r]));
      ws[c] = block_kbns(k, scratch);
    }
  if(threadIdx.x != 0) return;
  qmiv_frame_result* R = J.result;
  const int64_t nnm = tot[6];
  *J.nnm = nnm;
  const int64_t area = (int64_t)J.W * J.H;
  const double mm = (double)((1 << J.mbd) - 1);
  for(int c = 0; c < 3; c++)
  {
    int g = nnm > 0 ? __double2int_rn(__ddiv_rn((double)tot[c], __dmul_rn((double)nnm, mm))) : 0;
    g = g < -J.maxdiff[c] ? -J.maxdiff[c] : (g > J.maxdiff[c] ? J.maxdiff[c] : g);
    if(!J.gcd_given) J.gcd[c] = g;
    R->gcd_r2t[c] = J.gcd_given ? J.gcd[c] : g;
  }
  R->gcd_r2t[3] = 0;
  double ps[3], wp[3];
  const double fake = psnr_from_ssd(1.0, area, J.bd);
  for(int c = 0; c < 3; c++)
  {
    const bool exact = tot[7 + c] == 0;
    R->exact[c] = exact;
    ps[c] = psnr_masked((double)(unsigned long long)tot[3 + c], nnm, J.bd, J.mbd);
    wp[c] = J.use_ws ? psnr_masked(__dmul_rn(ws[c], J.ws_corr), nnm, J.bd, J.mbd) : ps[c];
    if(exact && J.fake_exact) { ps[c] = fake; wp[c] = fake; }
  }
  R->exact[3] = 0;
  if(J.metrics & QMIV_M_PSNR)   { for(int c = 0; c < 3; c++) R->psnr[c] = ps[c];   R->psnr[3] = 0;   R->psnr_pic = weighted3(ps, J.w_avg); }
  if(J.metrics & QMIV_M_WSPSNR) { for(int c = 0; c < 3; c++) R->wspsnr[c] = wp[c]; R->wspsnr[3] = 0; R->wspsnr_pic = weighted3(wp, J.w_avg); }
  R->status = 0;
  __threadfence();
  J.counters[0] = 0;
}

constexpr int kMTW = 32, kMTH = 16;  // search tile: 32x16 pixels per 256-thread block (two rows per thread)

template <bool W64> struct MCost { using T = int; static constexpr T kNone = INT_MAX; };
template <> struct MCost<true> { using T = long long; static constexpr T kNone = LLONG_MAX; };

// One masked search direction for the pixel at tile index ci: tested values t (with the GCD
// applied) searched among the staged reference picture R[3]; masked candidates cost kNone, so
// they never win, and the first strict minimum in raster order of the window is kept, as the
// reference's loop does. Returns the tile index of the best candidate.
template <int SR_T, bool W64>
__device__ __forceinline__ int masked_best(const uint16_t* __restrict__ R0, const uint16_t* __restrict__ R1,
                                           const uint16_t* __restrict__ R2, const uint16_t* __restrict__ M,
                                           int ci, int TW, int sr, const int t[3], const int w[3])
{
  using C = MCost<W64>;
  const int SR = SR_T >= 0 ? SR_T : sr;
  typename C::T best = C::kNone;
  int bidx = ci;
#pragma unroll
  for(int dy = -SR; dy <= SR; dy++)
  {
    const int rb = ci + dy * TW;
#pragma unroll
    for(int dx = -SR; dx <= SR; dx++)
    {
      const int k = rb + dx;
      const int d0 = t[0] - (int)R0[k], d1 = t[1] - (int)R1[k], d2 = t[2] - (int)R2[k];
      typename C::T e = (typename C::T)d0 * d0 * w[0] + (typename C::T)d1 * d1 * w[1] + (typename C::T)d2 * d2 * w[2];
      e = M[k] ? e : C::kNone;
      if(e < best) { best = e; bidx = k; }
    }
  }
  return bidx;
}

// Both directions per pixel (the application passes (P0, P1) as (Tst, Ref): R2T = Q(P1, P0, -GCD),
// T2R = Q(P0, P1, +GCD), xIVPSNR.cpp:153-200); per-row sums by warp and 64-bit atomics; the last
// block forms IV-PSNR-M. SR_T < 0: search range taken from the job.
template <int SR_T, bool W64>
__global__ void __launch_bounds__(256) k_masked_cps(MaskJob J)
{
  extern __shared__ uint16_t s_mem[];  // [2 pictures][3 components][N], then the mask [N]
  __shared__ bool is_last;
  __shared__ double scratch[16];
  const int SR = SR_T >= 0 ? SR_T : J.sr;
  const int TW = kMTW + 2 * SR, N = TW * (kMTH + 2 * SR);
  const int x0 = blockIdx.x * kMTW, y0 = blockIdx.y * kMTH;
  uint16_t* s_m = s_mem + 6 * N;
  for(int i = threadIdx.x; i < N; i += blockDim.x)
  {
    const int ly = i / TW, lx = i - ly * TW;
    const int gx = min(max(x0 + lx - SR, 0), J.W - 1), gy = min(max(y0 + ly - SR, 0), J.H - 1);
    s_m[i] = (uint16_t)msk(J, gx, gy);
    for(int c = 0; c < 3; c++)
    {
      s_mem[c * N + i] = (uint16_t)pel(J, 0, c, gx, gy);
      s_mem[(3 + c) * N + i] = (uint16_t)pel(J, 1, c, gx, gy);
    }
  }
  const int g[3] = { J.gcd[0], J.gcd[1], J.gcd[2] };
  __syncthreads();
  const int lane = threadIdx.x & 31, ty = threadIdx.x >> 5;
#pragma unroll 1
  for(int r = 0; r < 2; r++)
  {
    const int ly = ty + 8 * r, y = y0 + ly, x = x0 + lane;
    unsigned long long q[2][3] = { { 0, 0, 0 }, { 0, 0, 0 } };
    if(x < J.W && y < J.H)
    {
      const int ci = (ly + SR) * TW + lane + SR;
      const int m = s_m[ci];
      if(m != 0)
#pragma unroll
        for(int d = 0; d < 2; d++)
        {
          const int tp = d ? 0 : 1, rp = 1 - tp, sgn = d ? 1 : -1;
          const uint16_t* T = s_mem + tp * 3 * N;
          const uint16_t* R = s_mem + rp * 3 * N;
          const int t[3] = { T[ci] + sgn * g[0], T[N + ci] + sgn * g[1], T[2 * N + ci] + sgn * g[2] };
          const int b = masked_best<SR_T, W64>(R, R + N, R + 2 * N, s_m, ci, TW, SR, t, J.w_search);
#pragma unroll
          for(int c = 0; c < 3; c++)
          {
            const long long e = t[c] - (int)R[c * N + b];
            q[d][c] = (unsigned long long)(e * e) * (unsigned long long)m;
          }
        }
    }
    if(y < J.H)
#pragma unroll
      for(int d = 0; d < 2; d++)
#pragma unroll
        for(int c = 0; c < 3; c++)
        {
          const unsigned long long v = warp_sum(q[d][c]);
          if(lane == 0 && v) atomicAdd(&J.cps_rows[((int64_t)d * J.H + y) * 3 + c], v);
        }
  }
  __threadfence();
  __syncthreads();
  if(threadIdx.x == 0) is_last = atomicAdd(&J.counters[1], 1u) == gridDim.x * gridDim.y - 1;
  __syncthreads();
  if(!is_last) return;
  __threadfence();
  // one pass over the rows, six sums (direction x component) per thread in a fixed order
  double q[2][3];
  if(J.use_ws)
  { // weighted rows without the H / sum(w) correction (xIVPSNR.cpp:117-118)
    Kbns k[6];
#pragma unroll
    for(int i = 0; i < 6; i++) k[i] = Kbns{ 0.0, 0.0 };
    for(int r = threadIdx.x; r < J.H; r += blockDim.x)
    {
      const double wr = J.ws[r];
#pragma unroll
      for(int i = 0; i < 6; i++)
        k[i] = kbns_add(k[i], __dmul_rn((double)__ldcg(J.cps_rows + ((int64_t)(i / 3) * J.H + r) * 3 + i % 3), wr));
    }
#pragma unroll
    for(int i = 0; i < 6; i++) q[i / 3][i % 3] = block_kbns(k[i], scratch);
  }
  else
  {
    unsigned long long u[6] = { 0, 0, 0, 0, 0, 0 };
    for(int r = threadIdx.x; r < J.H; r += blockDim.x)
#pragma unroll
      for(int i = 0; i < 6; i++) u[i] += __ldcg(J.cps_rows + ((int64_t)(i / 3) * J.H + r) * 3 + i % 3);
    __shared__ unsigned long long s_u[8][6];
#pragma unroll
    for(int i = 0; i < 6; i++)
    {
      const unsigned long long w = warp_sum(u[i]);
      if(lane == 0) s_u[threadIdx.x >> 5][i] = w;
    }
    __syncthreads();
#pragma unroll
    for(int i = 0; i < 6; i++)
    {
      unsigned long long tsum = 0;
      for(int w = 0; w < 8; w++) tsum += s_u[w][i];
      q[i / 3][i % 3] = (double)tsum;
    }
  }
  if(threadIdx.x != 0) return;
#pragma unroll
  for(int d = 0; d < 2; d++)
#pragma unroll
    for(int c = 0; c < 3; c++) q[d][c] = psnr_masked(q[d][c] > 0 ? q[d][c] : 1.0, *J.nnm, J.bd, J.mbd);
  const double a = weighted3(q[0], J.w_avg), b = weighted3(q[1], J.w_avg);
  J.result->ivpsnr_r2t = a;
  J.result->ivpsnr_t2r = b;
  J.result->ivpsnr = b < a ? b : a;
  __threadfence();
  J.counters[1] = 0;
}

template <int SR_T>
cudaError_t launch_masked_cps(const MaskJob& j, cudaStream_t st)
{
  const int sr = SR_T >= 0 ? SR_T : j.sr;
  const size_t smem = (size_t)7 * (kMTW + 2 * sr) * (kMTH + 2 * sr) * sizeof(uint16_t);
  const dim3 grid((j.W + kMTW - 1) / kMTW, (j.H + kMTH - 1) / kMTH);
  if(j.fits32) k_masked_cps<SR_T, false><<<grid, 256, smem, st>>>(j);
  else k_masked_cps<SR_T, true><<<grid, 256, smem, st>>>(j);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_masked(const MaskJob& j, cudaStream_t st)
{
  // the search tile at the largest range, 7 x 64 x 48 x 2 bytes, stays below the 48 KB default
  static_assert(7 * (kMTW + 2 * kMaxSR) * (kMTH + 2 * kMaxSR) * 2 <= 48 * 1024, "masked search tile");
  k_masked_stats<<<(j.H + 1) / 2, 256, 0, st>>>(j);
  cudaError_t e = cudaGetLastError();
  if(e != cudaSuccess || !(j.metrics & QMIV_M_IVPSNR)) return e;
  switch(j.sr)
  {
    case 1: return launch_masked_cps<1>(j, st);
    case 2: return launch_masked_cps<2>(j, st);
    case 3: return launch_masked_cps<3>(j, st);
    case 4: return launch_masked_cps<4>(j, st);
    default: return launch_masked_cps<-1>(j, st);
  }
}

}  // namespace qmiv
