// Device descriptors of the SSIM-family kernels (k_ssim.cu) and their host launchers.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "qmiv_internal.h"

namespace qmiv {

// A plane read as sample(x, y) = ptr[(y >> shift) * stride + (x >> shift)]: shift 1 reads a 4:2:0
// chroma plane at luma resolution (nearest-neighbour upsampling, xPixelOpsSTD.cpp:30-49).
struct SsimPlane {
  const void* ptr;
  int32_t stride;
  int8_t sbytes;
  int8_t shift;
  int16_t pad;
};

// One SSIM evaluation of a plane pair (xSSIM::xCalcCmpSSIM, xSSIM.cpp:91-112).
struct SsimJob {
  SsimPlane a, b;        // a = "Tst", b = "Ref" of calcPicSSIM; b also gives the centring offset
  int32_t W, H;
  int32_t calc_l;        // 0: contrast-structure only (MS-SSIM scales 0 and 4)
  float c1, c2;          // (0.01 Max)^2, (0.03 Max)^2
  int32_t tiles_x, tiles_y, tile_base;
  float* partial;        // [(H-10)][tiles_x] per-tile row sums
  double* out;           // picture mean
};

// The full-resolution SSIM family of one component of one frame in a single pass over its
// four planes: picture 0, picture 1 and the two shift-compensated pictures. Outputs (bits of
// `outs`): 0 SSIM(P0, P1) (L*CS), 1 CS(P0, P1) (MS-SSIM scale 0), 2 SSIM(P0, SCP1) (IV-SSIM T2R),
// 3 SSIM(P1, SCP0) (IV-SSIM R2T). Each output's per-tile row sums go to partial[k] in the
// layout of an SsimJob with the same picture size.
struct SsimQuadJob {
  SsimPlane p0, p1, scp1, scp0;
  int32_t W, H;
  float c1, c2;
  int32_t tiles_x, tiles_y, tile_base;
  uint32_t outs;
  float* partial[4];
  const void* tmaps;     // 4 tensor maps (p0, p1, scp1, scp0 boxes) or null: staged by plain loads
  int32_t* status;       // the frame's result status (a bulk load that never arrived), or null
};
int ssim_quad_tiles_y(int H);
// Box of one plane of a fused-kernel tile: width (samples) for `sb`-byte samples at full (shift 0)
// or half resolution, and height for the window (QMIV_SSIM_*).
__host__ __device__ constexpr int quad_box_w(int sb, int shift) { return (shift ? 32 : 64) + 16 / sb; }
int quad_box_h(int window, int shift);
cudaError_t launch_ssim_quad(const SsimQuadJob* d_jobs, const SsimQuadJob* h_jobs, int n, int window,
                             uint32_t first_wait_test_polls, cudaStream_t st);

// One DownsampleHV step of the MS-SSIM pyramid.
struct PyrStep {
  SsimPlane src;
  uint16_t* dst;
  int32_t dst_stride, dw, dh;
};

// Per frame: where the SSIM-job values are and which metrics to combine.
// vals: [0..2] SSIM, [3..17] MS-SSIM scale i component c at 3+3i+c, [18..20] IV-SSIM T2R
// (picture 0 vs SCP1), [21..23] IV-SSIM R2T (picture 1 vs SCP0).
struct SsimFrame {
  uint32_t metrics;
  int32_t pad;
  qmiv_frame_result* result;
  const double* vals;
};

constexpr int kSsimVals = 24;

// One SSIM backward evaluation: gradients of g * SSIM(a, b) (the picture mean of the SSIM map,
// L*CS) with respect to every sample of a and of b, over the whole picture. Planes are FP32.
struct SsimBwdJob {
  SsimPlane a, b;
  int32_t W, H;
  float c1, c2;
  int32_t tiles_x, tiles_y, tile_base;
  const double* g;       // upstream gradient of this SSIM value
  float* outx;           // d/da, W x H with row pitch W (null: not needed)
  float* outy;           // d/db (null: not needed)
};
int ssim_bwd_tiles(int dim);        // 32-column strips of a row of width dim
int ssim_bwd_segments(int H);       // row segments a strip is cut into
cudaError_t launch_ssim_bwd(const SsimBwdJob* d_jobs, const SsimBwdJob* h_jobs, int n, int window, cudaStream_t st);

cudaError_t ssim_set_window_constants(const float g[11], const double w0[2]);
int ssim_tiles_x(int W, int window);
int ssim_tiles_y(int H);
cudaError_t launch_ssim(const SsimJob* d_jobs, const SsimJob* h_jobs, int n, int window, cudaStream_t st);
cudaError_t launch_downsample(const PyrStep* d_steps, const PyrStep* h_steps, int n, cudaStream_t st);
cudaError_t launch_ssim_combine(const SsimFrame* d_frames, int n, const Params& p, cudaStream_t st);

}  // namespace qmiv
