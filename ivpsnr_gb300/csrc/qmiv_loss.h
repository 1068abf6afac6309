// Differentiable IV-PSNR error and IV-SSIM on FP32 4:4:4 pictures (k_loss.cu): workspace
// layout and host launchers.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "qmiv_ssim.h"

namespace qmiv {

constexpr int kLossGcdChunks = 64;   // partial sums per plane for the global colour difference
constexpr int kLossMaxSR = 4;

// Byte offsets of the caller-provided workspace (each 256-aligned). Per image b, component c,
// direction d (0 = R2T: tested pixels searched in the reference, 1 = T2R).
struct LossLayout {
  int n, W, H, window, tiles_x, tiles_y, cps_blocks;
  int gg_blocks;     // blocks of the GCD-gradient reduction per picture (kLossGgPx pixels each)
  int grad_blocks;   // blocks of the gradient gather per picture (32x16 tiles)
  size_t gcd_part;   // double [n*3][kLossGcdChunks]
  size_t gcd;        // float [n*3] clipped GCD_R2T, then int [n*3] 1 = not clipped
  size_t maps;       // uint16 [2][n][H][W]: argmin index (bits 0-7) + unclipped-SCP bits 8-10
  size_t scp;        // float [2][n][3][H][W]: SCP1 (from the reference), SCP0 (from the tested)
  size_t sse_part;   // double [2][n][2][3][cps_blocks]: squared errors, then errors
  size_t esum;       // double [n][2][3]: per-direction sums of the errors (forward, kept for backward)
  size_t sjobs;      // SsimJob [n*6]
  size_t partial;    // float [n*6][H-10][tiles_x]
  size_t dy;         // float [2][n][3][H][W]: d SSIM / d (second picture), T2R then R2T
  size_t g_part;     // double [n*3][gg_blocks], then [n*3]: d loss / d GCD partial sums and totals
  size_t bytes;
};

LossLayout loss_layout(int n, int W, int H, int window);

struct LossArgs {
  const float* tst;
  const float* ref;
  int n, W, H, sr;
  float w_search[3];
  float unc[3];
  int window;
  uint8_t* ws;
  LossLayout L;
};

cudaError_t loss_forward(const LossArgs& a, double* sse, double* ssim, cudaStream_t st);
cudaError_t loss_backward(const LossArgs& a, const double* g_sse, const double* g_ssim, float* g_tst, cudaStream_t st);

}  // namespace qmiv
