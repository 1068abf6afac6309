// Internal device-side descriptors shared by the kernels and the host launcher.
#pragma once
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/qmiv_gb300.h"

namespace qmiv {

constexpr int kMaxSR = 16;

// Per-job scalars produced on the device and consumed by later kernels of the same job.
struct JobScalars {
  int32_t  gcd[4];          // GCD_R2T after the stats kernel (or supplied by the caller)
  uint32_t stats_done;      // last-block counters (self-resetting)
  uint32_t cps_done;
  uint32_t ssim_done;
  int32_t  status;
  double   ssim_acc[8][3];  // SSIM plane sums for the current job: [pass][cmp] (see k_ssim)
};

// One picture pair as the kernels see it.
struct DevJob {
  const void* p0[3];
  const void* p1[3];
  int32_t stride0[3], stride1[3];
  int32_t W, H, bd, sbytes, cshift;   // cshift 1: 4:2:0 chroma, 0: 4:4:4
  uint32_t metrics;
  int32_t use_ws;
  const double* ws;                   // row weights (H) when use_ws
  double ws_corr;                     // H / sum(w)
  uint16_t* scp0[3];                  // built from picture 0 (T2R argmin), may be null
  uint16_t* scp1[3];                  // built from picture 1 (R2T argmin), may be null
  int32_t scp_stride;
  int16_t* cps_map[2];                // argmin window index per pixel, R2T then T2R; may be null
  int32_t map_stride;
  int32_t gcd_given;                  // 1: sc->gcd preset by the host, stats kernel leaves it
  int32_t slot;                       // the handle's scratch slot (host bookkeeping)
  const void* tmaps;                  // 6 tensor maps (picture 0 Y,Cb,Cr then picture 1) or null
  int64_t* stat_rows;                 // [H][6]: sum(P1-P0)[3], sum((P1-P0)^2)[3]
  unsigned long long* cps_rows;       // [2][H][3]: per-row CPS SSE, direction R2T then T2R
  JobScalars* sc;
  qmiv_frame_result* result;
  // grid decomposition
  int32_t stat_blocks, stat_base;     // row pairs
  int32_t cps_strips, cps_segs, cps_seg_chunks, cps_base;
};

// Launch-wide parameters (the handle's options, pre-digested on the host).
struct Params {
  int32_t sr;
  int32_t w_search[3];
  int32_t w_avg[3];
  int32_t maxdiff_for_bd[15][3];      // rne_f32(unc * Max) per bit depth (index bd) and component
  int32_t fake_exact;
  int32_t legacy_ws8;
  // CPS key construction: E * M + k with (s*dY)^2 = M*w0*dY^2
  uint32_t key_m;                     // M
  int32_t key_m_log2;                 // log2(M) if M is a power of two, else -1
  int32_t luma_scale;                 // s
  int32_t luma_scale_log2;            // log2(s) if s is a power of two, else -1
  uint32_t one;                       // 1, opaque to the compiler (keeps index adds on the multiply-add pipe)
  uint32_t first_wait_test_polls;     // test hook: > 0 makes each block's first bulk-copy wait poll an idle
                                      // barrier this many times and give up (0: normal waits)
};

// Host-side launchers (defined in the .cu files).
cudaError_t launch_init_results(const DevJob* d_jobs, int n, cudaStream_t st);
cudaError_t launch_copy_table(const void* src, void* dst, size_t bytes, cudaStream_t st);  // bytes: a multiple of 16
cudaError_t launch_stats(const DevJob* d_jobs, const DevJob* h_jobs, int n, const Params& p, cudaStream_t st);

// Statistics of one picture pair in a static device array (k_stats.cu): no allocation.
constexpr int kStaticMaxRows = 8192;     // tallest picture the static row sums hold
// widest picture of the static path: a row's sum of differences is kept in an int32, and
// 65536 samples x (2^14 - 1) stays below 2^31 at every supported bit depth
constexpr int kStaticMaxWidth = 65536;
constexpr int kStaticMaxDevices = 64;

// Launch attributes (cudaFuncSetAttribute, occupancy) belong to the current device, so the
// launchers keep their one-time set-up per device ordinal.
inline int device_slot()
{
  int d = 0;
  if(cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= kStaticMaxDevices) d = 0;
  return d;
}
struct StaticStatsScratch {
  int64_t* stat_rows;                    // [kStaticMaxRows][6]
  JobScalars* sc;                        // stats_done must be 0 when the kernel starts
  qmiv_frame_result* result;
};
// The array's address on the current device (looked up on the first call per device).
cudaError_t stats_static_scratch(StaticStatsScratch* out);
cudaError_t launch_stats_static(const DevJob& j, const Params& p, cudaStream_t st);

// One compiled form of the CPS kernel.
struct CpsVariant {
  const char* name;
  cudaError_t (*launch)(const DevJob* d_jobs, int n, int blocks, const Params& p, cudaStream_t st);
  // the same search for launches where some job writes argmin maps (DevJob::cps_map)
  cudaError_t (*launch_map)(const DevJob* d_jobs, int n, int blocks, const Params& p, cudaStream_t st);
  int sr;        // search range it is specialised for (0: any)
  int rows;      // strip rows per block (generic: tile rows)
  int cols;      // columns per chunk (generic: tile columns)
  bool key64;    // 64-bit packed keys (high bit depths)
  int kind;      // 0 generic, 1 staged loads, 2 TMA double-buffered
  int sbytes;    // sample size it requires (0: any)
};
const CpsVariant* cps_variants_staged(int* n);  // k_cps.cu
const CpsVariant* cps_variants_tma(int* n);     // k_cps_tma.cu

}  // namespace qmiv
