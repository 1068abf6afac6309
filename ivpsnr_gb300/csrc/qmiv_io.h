// Input-side kernels (k_io.cu): 4:2:2 upsampling, range check / concealment, RGB <-> YCbCr.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

namespace qmiv {

// xColorSpaceCoeff<int32>: 16 fraction bits, rounding offset 2^15 (xColorSpaceCoeff.h:166-169)
constexpr int kColorPrec = 16;
constexpr int kColorAdd = 1 << (kColorPrec - 1);

struct ColorJob {
  const void* src[3];
  int32_t sbytes, sstride;
  uint16_t* dst[3];
  int32_t dstride;
  int32_t W, H, bd;
  int32_t to_ycbcr;       // 1: R,G,B -> Y,Cb,Cr; 0: Y,Cb,Cr -> R,G,B
  int32_t m[3][3];        // fixed-point matrix of the colour space
};

// The fixed-point matrices of the four YCbCr colour spaces (BT.601, BT.709, SMPTE 240M,
// BT.2020), derived as xColorSpaceCoeffYCbCr / xColorSpaceCoeff do (xColorSpaceCoeff.h:36-203).
void color_matrix(int space, bool to_ycbcr, int32_t m[3][3]);

cudaError_t launch_upsample_h(const void* src, int sbytes, int sstride, void* dst, int W, int H, cudaStream_t st);
// The three planes of one range check / concealment (one launch, grid.y = component).
struct RangeJob {
  void* plane[3];
  int32_t stride[3], w[3], h[3];
  int32_t sbytes, maxv, conceal;
  unsigned long long* count;  // [3] device counters
};
cudaError_t launch_range(const RangeJob& j, int sms, cudaStream_t st);
cudaError_t launch_color(const ColorJob& j, cudaStream_t st);

}  // namespace qmiv
