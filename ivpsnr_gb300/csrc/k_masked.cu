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
// (64-bit), so results do not depend on the launch shape. Not a throughput path: one thread
// per pixel with plain cached loads.
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

// per-row sums, one warp per row; the last block forms GCD-M, PSNR-M and WS-PSNR-M
__global__ void __launch_bounds__(256) k_masked_stats(MaskJob J)
{
  __shared__ bool is_last;
  __shared__ double scratch[16];
  const int lane = threadIdx.x & 31, y = blockIdx.x * 8 + (threadIdx.x >> 5);
  if(y < J.H)
  {
    long long sd[3] = { 0, 0, 0 };
    unsigned long long ssd[3] = { 0, 0, 0 };
    int nnz = 0, dif[3] = { 0, 0, 0 };
    for(int x = lane; x < J.W; x += 32)
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
    int64_t v[10];
    for(int c = 0; c < 3; c++) { v[c] = warp_sum(sd[c]); v[3 + c] = (int64_t)warp_sum(ssd[c]); v[7 + c] = warp_sum(dif[c]); }
    v[6] = warp_sum(nnz);
    if(lane < 10) J.rows[(int64_t)y * kMaskRowVals + lane] = v[lane];
    if(lane < 6) J.cps_rows[((int64_t)(lane / 3) * J.H + y) * 3 + lane % 3] = 0ull;
  }
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

// One masked search direction for pixel (x, y): tested picture `tp` (+ g) searched in `rp`.
__device__ __forceinline__ void masked_search(const MaskJob& J, int tp, int rp, int sgn, int x, int y, int m,
                                              unsigned long long sse[3])
{
  int t[3];
  for(int c = 0; c < 3; c++) t[c] = pel(J, tp, c, x, y) + sgn * J.gcd[c];
  long long best = LLONG_MAX;
  int bx = x, by = y;
  for(int dy = -J.sr; dy <= J.sr; dy++)
  {
    const int yy = min(max(y + dy, 0), J.H - 1);
    for(int dx = -J.sr; dx <= J.sr; dx++)
    {
      const int xx = min(max(x + dx, 0), J.W - 1);
      if(msk(J, xx, yy) == 0) continue;
      long long e = 0;
      for(int c = 0; c < 3; c++) { const long long d = t[c] - pel(J, rp, c, xx, yy); e += d * d * J.w_search[c]; }
      if(e < best) { best = e; bx = xx; by = yy; }
    }
  }
  for(int c = 0; c < 3; c++)
  {
    const long long d = t[c] - pel(J, rp, c, bx, by);
    sse[c] = (unsigned long long)(d * d) * (unsigned long long)m;
  }
}

// Both directions per pixel (the application passes (P0, P1) as (Tst, Ref): R2T = Q(P1, P0, -GCD),
// T2R = Q(P0, P1, +GCD), xIVPSNR.cpp:153-200); per-row sums by warp; the last block forms IV-PSNR-M.
__global__ void __launch_bounds__(256) k_masked_cps(MaskJob J)
{
  __shared__ bool is_last;
  __shared__ double scratch[16];
  const int lane = threadIdx.x & 31;
  const int tiles_x = (J.W + 31) / 32;
  const int x = (blockIdx.x % tiles_x) * 32 + lane;
  const int y = (blockIdx.x / tiles_x) * 8 + (threadIdx.x >> 5);
  unsigned long long r2t[3] = { 0, 0, 0 }, t2r[3] = { 0, 0, 0 };
  if(x < J.W && y < J.H)
  {
    const int m = msk(J, x, y);
    if(m != 0)
    {
      masked_search(J, 1, 0, -1, x, y, m, r2t);
      masked_search(J, 0, 1, +1, x, y, m, t2r);
    }
  }
  if(y < J.H)
    for(int c = 0; c < 3; c++)
    {
      const unsigned long long a = warp_sum(r2t[c]), b = warp_sum(t2r[c]);
      if(lane == 0)
      {
        if(a) atomicAdd(&J.cps_rows[((int64_t)0 * J.H + y) * 3 + c], a);
        if(b) atomicAdd(&J.cps_rows[((int64_t)1 * J.H + y) * 3 + c], b);
      }
    }
  __threadfence();
  __syncthreads();
  if(threadIdx.x == 0) is_last = atomicAdd(&J.counters[1], 1u) == gridDim.x - 1;
  __syncthreads();
  if(!is_last) return;
  __threadfence();
  double q[2][3];
  for(int d = 0; d < 2; d++)
    for(int c = 0; c < 3; c++)
    {
      double err;
      if(J.use_ws)
      { // weighted rows without the H / sum(w) correction (xIVPSNR.cpp:117-118)
        Kbns k = { 0.0, 0.0 };
        for(int r = threadIdx.x; r < J.H; r += blockDim.x)
          k = kbns_add(k, __dmul_rn((double)__ldcg(J.cps_rows + ((int64_t)d * J.H + r) * 3 + c), J.ws[r]));
        err = block_kbns(k, scratch);
      }
      else
      {
        unsigned long long s = 0;
        for(int r = threadIdx.x; r < J.H; r += blockDim.x) s += __ldcg(J.cps_rows + ((int64_t)d * J.H + r) * 3 + c);
        s = warp_sum(s);
        __shared__ unsigned long long s_u[8];
        if(lane == 0) s_u[threadIdx.x >> 5] = s;
        __syncthreads();
        unsigned long long tsum = 0;
        for(int w = 0; w < 8; w++) tsum += s_u[w];
        __syncthreads();
        err = (double)tsum;
      }
      q[d][c] = psnr_masked(err > 0 ? err : 1.0, *J.nnm, J.bd, J.mbd);
    }
  if(threadIdx.x != 0) return;
  const double a = weighted3(q[0], J.w_avg), b = weighted3(q[1], J.w_avg);
  J.result->ivpsnr_r2t = a;
  J.result->ivpsnr_t2r = b;
  J.result->ivpsnr = b < a ? b : a;
  __threadfence();
  J.counters[1] = 0;
}

}  // namespace

cudaError_t launch_masked(const MaskJob& j, cudaStream_t st)
{
  k_masked_stats<<<(j.H + 7) / 8, 256, 0, st>>>(j);
  cudaError_t e = cudaGetLastError();
  if(e != cudaSuccess || !(j.metrics & QMIV_M_IVPSNR)) return e;
  k_masked_cps<<<((j.W + 31) / 32) * ((j.H + 7) / 8), 256, 0, st>>>(j);
  return cudaGetLastError();
}

}  // namespace qmiv
