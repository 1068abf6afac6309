// Shared pieces of the CPS kernels: the last-block IV-PSNR finalisation (libs/pmbb-ivqm/
// src/xIVPSNR.cpp:18-56,100-133) and small index helpers.
#pragma once
#include "qmiv_device.cuh"

namespace qmiv {
namespace {

__host__ __device__ constexpr int fdiv2(int v) { return v >= 0 ? v / 2 : -((-v + 1) / 2); } // floor(v/2)
__host__ __device__ constexpr int ceil2(int v) { return (v + 1) / 2; }

// ------------------------------------------------------------------------------------
// Last block of a job: IV-PSNR from the per-row CPS sums.
// ------------------------------------------------------------------------------------
__device__ void finalize_cps(const DevJob& J, const Params& p, double* scratch)
{
  __shared__ unsigned long long s_tot[2][3];
  __shared__ double s_ws[2][3];
  const int64_t area = (int64_t)J.W * J.H;
  for(int d = 0; d < 2; d++)
    for(int c = 0; c < 3; c++)
    {
      unsigned long long t = 0;
      Kbns k = { 0.0, 0.0 };
      for(int y = threadIdx.x; y < J.H; y += blockDim.x)
      {
        const unsigned long long v = __ldcg(J.cps_rows + ((int64_t)d * J.H + y) * 3 + c);
        t += v;
        if(J.use_ws) k = kbns_add(k, __dmul_rn((double)v, J.ws[y]));
      }
      t = warp_sum(t);
      __syncthreads();
      if((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = __longlong_as_double((long long)t);
      __syncthreads();
      if(threadIdx.x == 0)
      {
        unsigned long long a = 0;
        for(int w = 0; w < (int)(blockDim.x >> 5); w++) a += (unsigned long long)__double_as_longlong(scratch[w]);
        s_tot[d][c] = a;
      }
      __syncthreads();
      if(J.use_ws) { const double r = block_kbns(k, scratch); if(threadIdx.x == 0) s_ws[d][c] = r; }
    }
  if(threadIdx.x == 0)
  {
    qmiv_frame_result* R = J.result;
    double q[2];
    for(int d = 0; d < 2; d++)
    {
      double qc[3];
      for(int c = 0; c < 3; c++)
      { // xIVPSNR.cpp:117-126: ERP uses the weighted sum without the H/sum(w) correction
        const double e = J.use_ws ? s_ws[d][c] : (double)s_tot[d][c];
        qc[c] = psnr_from_ssd(e > 0 ? e : 1.0, area, J.bd);
      }
      q[d] = weighted3(qc, p.w_avg);
    }
    R->status = J.sc->status;
    for(int c = 0; c < 3; c++) { R->sse_r2t[c] = s_tot[0][c]; R->sse_t2r[c] = s_tot[1][c]; }
    R->sse_r2t[3] = 0; R->sse_t2r[3] = 0;
    if(J.metrics & QMIV_M_IVPSNR)
    {
      R->ivpsnr_r2t = q[0];
      R->ivpsnr_t2r = q[1];
      R->ivpsnr = q[1] < q[0] ? q[1] : q[0]; // std::min(R2T, T2R) (xIVPSNR.cpp:55)
    }
    __threadfence();
    J.sc->cps_done = 0;
  }
}

__device__ __forceinline__ bool cps_last_block(const DevJob& J)
{
  __shared__ bool is_last;
  __threadfence();
  __syncthreads();
  if(threadIdx.x == 0) is_last = atomicAdd(&J.sc->cps_done, 1u) == (unsigned)(J.cps_strips * J.cps_segs - 1);
  __syncthreads();
  return is_last;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

}  // namespace
}  // namespace qmiv
