// Device descriptor of one masked picture pair (k_masked.cu) and its launcher.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "qmiv_internal.h"

namespace qmiv {

constexpr int kMaskRowVals = 10;  // per row: sum d*m [3], sum d^2*m [3], non-masked count, differing samples [3]

struct MaskJob {
  const void* p0[3];
  const void* p1[3];
  int32_t s0[3], s1[3];
  int32_t W, H, bd, sbytes, cshift;
  const void* mask;                 // luma-resolution mask samples
  int32_t mstride, msbytes, mbd;
  uint32_t metrics;
  int32_t use_ws;
  const double* ws;
  double ws_corr;
  int32_t fake_exact, sr;
  int32_t w_search[3], w_avg[3], maxdiff[3];
  int32_t gcd_given;
  int32_t fits32;                   // the largest search cost, sum of w (2^bd - 1 + maxdiff)^2, is below 2^31 - 1
  int32_t* gcd;                     // [3] device: masked GCD_R2T (written unless given)
  long long* nnm;                   // [1] device: non-masked pixel count
  int64_t* rows;                    // [H][kMaskRowVals]
  unsigned long long* cps_rows;     // [2][H][3]: R2T then T2R
  uint32_t* counters;               // [2] last-block counters (self-resetting)
  qmiv_frame_result* result;
};

cudaError_t launch_masked(const MaskJob& j, cudaStream_t st);

}  // namespace qmiv
