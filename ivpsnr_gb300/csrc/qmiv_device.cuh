// Device helpers shared by the kernels: job lookup, sample loads, exact/compensated
// reductions and the FP64 dB step.
#pragma once
#include <cfloat>
#include <cstdint>

#include "qmiv_internal.h"

namespace qmiv {

// Block -> job by binary search over the jobs' first-block offsets (jobs sorted by base).
template <int Which>
__device__ __forceinline__ int find_job(const DevJob* __restrict__ jobs, int n, int b)
{
  int lo = 0, hi = n - 1;
  while(lo < hi)
  {
    const int mid = (lo + hi + 1) >> 1;
    const int base = Which == 0 ? jobs[mid].stat_base : jobs[mid].cps_base;
    if(base <= b) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int ld_sample(const void* p, int sbytes, int64_t idx)
{
  return sbytes == 1 ? (int)__ldg((const uint8_t*)p + idx) : (int)__ldg((const uint16_t*)p + idx);
}

// Neumaier (Kahan-Babuska) compensated sum, the FP64 reduction the reference uses for row
// sums (xKBNS, libs/pmbb-core/src/xMathUtils.h:16). Products are formed with __dmul_rn so
// no multiply is contracted into the additions.
struct Kbns { double s, c; };
__device__ __forceinline__ Kbns kbns_add(Kbns a, double v)
{
  const double t = __dadd_rn(a.s, v);
  if(fabs(a.s) >= fabs(v)) a.c = __dadd_rn(a.c, __dadd_rn(__dsub_rn(a.s, t), v));
  else                     a.c = __dadd_rn(a.c, __dadd_rn(__dsub_rn(v, t), a.s));
  a.s = t;
  return a;
}
__device__ __forceinline__ Kbns kbns_merge(Kbns a, Kbns b) { a = kbns_add(a, b.s); a.c = __dadd_rn(a.c, b.c); return a; }
__device__ __forceinline__ double kbns_result(Kbns a) { return __dadd_rn(a.s, a.c); }

__device__ __forceinline__ Kbns warp_kbns(Kbns v)
{
  for(int o = 16; o > 0; o >>= 1)
  {
    Kbns w; w.s = __shfl_xor_sync(0xffffffffu, v.s, o); w.c = __shfl_xor_sync(0xffffffffu, v.c, o);
    v = kbns_merge(v, w);
  }
  return v;
}

// Block-wide compensated sum; every thread passes its partial, thread 0 gets the result.
// scratch: >= 2*(blockDim/32) doubles of shared memory.
__device__ __forceinline__ double block_kbns(Kbns v, double* scratch)
{
  v = warp_kbns(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if(l == 0) { scratch[2 * w] = v.s; scratch[2 * w + 1] = v.c; }
  __syncthreads();
  double r = 0.0;
  if(threadIdx.x == 0)
  {
    Kbns a = { scratch[0], scratch[1] };
    for(int i = 1; i < nw; i++) { Kbns b = { scratch[2 * i], scratch[2 * i + 1] }; a = kbns_merge(a, b); }
    r = kbns_result(a);
  }
  __syncthreads();
  return r;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
  for(int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// CalcPSNRfromSSD (libs/pmbb-ivqm/src/xPSNR.cpp:139-146) in FP64
__device__ __forceinline__ double psnr_from_ssd(double ssd, int64_t area, int bd)
{
  const uint64_t mx = (uint64_t)((1 << bd) - 1);
  const uint64_t MAX = (uint64_t)area * (mx * mx);
  return ssd > 0 ? __dmul_rn(10.0, log10(__ddiv_rn((double)MAX, ssd))) : DBL_MAX;
}

// 4:1:1-style weighted mean (xAppQMIV.h:245-251, xIVPSNR.cpp:128-132)
__device__ __forceinline__ double weighted3(const double v[3], const int32_t w[3])
{
  const double a0 = __dmul_rn(v[0], (double)w[0]), a1 = __dmul_rn(v[1], (double)w[1]), a2 = __dmul_rn(v[2], (double)w[2]);
  const double inv = __ddiv_rn(1.0, (double)(w[0] + w[1] + w[2]));
  return __dmul_rn(__dadd_rn(__dadd_rn(__dadd_rn(a0, a1), a2), 0.0), inv);
}

}  // namespace qmiv
