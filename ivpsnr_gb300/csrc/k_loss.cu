// Differentiable IV-PSNR error and IV-SSIM of FP32 4:4:4 pictures with values in [0, 1]
// (Max = 1), batched over n picture pairs laid out [n][3][H][W]. The reference takes integer
// samples only; its definitions carry over without the integer rounding:
//   GCD_c   = clip(mean(R_c - T_c), -u_c, u_c)                  (xGlobClrDiff.cpp:15-48)
//   R2T:  s1(p) = argmin_s sum_c w_c (T_c(p) + GCD_c - R_c(p+s))^2, first strict minimum in
//         row-major order over the (2B+1)^2 window, coordinates clamped at the borders
//         (xCorrespPixelShift.cpp:48-85); e1_c(p) = T_c(p) + GCD_c - R_c(p+s1(p))
//   T2R:  s0(p) = argmin_s sum_c w_c (R_c(p) - GCD_c - T_c(p+s))^2;  e0_c = R_c(p) - GCD_c - T_c(p+s0)
//   SSE_c(R2T) = sum e1_c^2, SSE_c(T2R) = sum e0_c^2                 (xIVPSNR.cpp:62-95)
//   SCP1_c = clip(R_c(p+s1) - GCD_c, 0, 1), SCP0_c = clip(T_c(p+s0) + GCD_c, 0, 1)  (xShftCompPic.cpp:69-96)
//   SSIM_c(T2R) = SSIM(T_c, SCP1_c), SSIM_c(R2T) = SSIM(R_c, SCP0_c)   (xSSIM.cpp:166-190)
// Gradients with respect to T: the argmin is piecewise constant (no gradient), the error at
// the argmin routes to the pixel it was read from (gather for R2T, scatter for T2R, done here
// as a gather over the window so that it is deterministic), clips pass gradient inside
// [lo, hi] inclusive, and GCD contributes -1/Area per pixel while it is not clipped.
#include <algorithm>
#include <cstring>
#include <type_traits>
#include <vector>

#include "qmiv_device.cuh"

#include "qmiv_loss.h"

namespace qmiv {

namespace {

constexpr int kCpsTX = 32, kCpsTY = 8;
constexpr int kLossGgPx = 1024;               // pixels per block of the GCD-gradient reduction (4 per thread)
constexpr int kGradTX = 32, kGradTY = 16;     // gradient gather tile (two rows per thread)

struct Geo {
  const float* tst;
  const float* ref;
  int n, W, H;
  int64_t plane;       // W*H
};

// ---- global colour difference ---------------------------------------------------------------
// Knuth's TwoSum: a + b = s + e exactly in round-to-nearest FP32.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__global__ void __launch_bounds__(256) k_loss_gcd_part(Geo g, double* __restrict__ part)
{
  __shared__ double scratch[16];
  const int pc = blockIdx.y;                         // image*3 + component
  const int64_t per = (g.plane + kLossGcdChunks - 1) / kLossGcdChunks;
  const int64_t b0 = (int64_t)blockIdx.x * per, b1 = min(g.plane, b0 + per);
  const float* r = g.ref + (int64_t)pc * g.plane;
  const float* t = g.tst + (int64_t)pc * g.plane;
  // Each difference r - t is taken exactly as an unevaluated FP32 pair (TwoSum) and added to a
  // running (hi, lo) pair: hi by TwoSum, lo collects the exact errors. FP32 only, since FP64
  // arithmetic per element runs far below the memory rate here; the thread's pair goes to FP64
  // once, for the block's compensated sum.
  float hi = 0.0f, lo = 0.0f;
  for(int64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x)
  {
    float d, de, e;
    two_sum(__ldg(r + i), -__ldg(t + i), d, de);
    two_sum(hi, d, hi, e);
    lo = __fadd_rn(lo, __fadd_rn(e, de));
  }
  Kbns k = { (double)hi, (double)lo };
  const double s = block_kbns(k, scratch);
  if(threadIdx.x == 0) part[pc * kLossGcdChunks + blockIdx.x] = s;
}

__global__ void k_loss_gcd_final(Geo g, const double* __restrict__ part, float unc0, float unc1, float unc2,
                                 float* __restrict__ gcd, int* __restrict__ ok)
{
  const int pc = blockIdx.x * blockDim.x + threadIdx.x;
  if(pc >= g.n * 3) return;
  Kbns k = { 0.0, 0.0 };
  for(int i = 0; i < kLossGcdChunks; i++) k = kbns_add(k, part[pc * kLossGcdChunks + i]);
  const float m = (float)(kbns_result(k) / (double)g.plane);
  const int c = pc % 3;
  const float u = c == 0 ? unc0 : (c == 1 ? unc1 : unc2);
  gcd[pc] = fminf(fmaxf(m, -u), u);
  ok[pc] = (m >= -u && m <= u) ? 1 : 0;  // clip passes gradient on [-u, u] inclusive
}

// ---- corresponding-pixel search, both directions ----------------------------------------------
template <int SR>
__global__ void __launch_bounds__(kCpsTX * kCpsTY) k_loss_cps(Geo g, float w0, float w1, float w2,
                                                              const float* __restrict__ gcd, uint16_t* __restrict__ maps,
                                                              float* __restrict__ scp, double* __restrict__ sse_part,
                                                              int blocks_per_image)
{
  constexpr int SWX = kCpsTX + 2 * SR, SWY = kCpsTY + 2 * SR;
  __shared__ float2 s_rt[3][SWY][SWX];   // (ref, tst) sample pairs: one load feeds both directions
  __shared__ float s_red[8][12];
  const int b = blockIdx.y;
  const int bx = blockIdx.x % ((g.W + kCpsTX - 1) / kCpsTX), by = blockIdx.x / ((g.W + kCpsTX - 1) / kCpsTX);
  const int x0 = bx * kCpsTX, y0 = by * kCpsTY;
  const float* T = g.tst + (int64_t)b * 3 * g.plane;
  const float* R = g.ref + (int64_t)b * 3 * g.plane;
  { // all loads of the tile are issued before the first store
    constexpr int N = 3 * SWY * SWX, NI = (N + kCpsTX * kCpsTY - 1) / (kCpsTX * kCpsTY);
    float vt[NI], vr[NI];
    #pragma unroll
    for(int k = 0; k < NI; k++)
    {
      const int i = min((int)threadIdx.x + kCpsTX * kCpsTY * k, N - 1);
      const int c = i / (SWY * SWX), rr = (i / SWX) % SWY, q = i % SWX;
      const int gx = min(max(x0 - SR + q, 0), g.W - 1), gy = min(max(y0 - SR + rr, 0), g.H - 1);
      const int64_t o = (int64_t)c * g.plane + (int64_t)gy * g.W + gx;
      vt[k] = __ldg(T + o);
      vr[k] = __ldg(R + o);
    }
    #pragma unroll
    for(int k = 0; k < NI; k++)
    {
      const int i = threadIdx.x + kCpsTX * kCpsTY * k;
      if(i >= N) break;
      (&s_rt[0][0][0])[i] = make_float2(vr[k], vt[k]);
    }
  }
  __syncthreads();
  const int lx = threadIdx.x % kCpsTX, ly = threadIdx.x / kCpsTX;
  const int x = x0 + lx, y = y0 + ly;
  const bool inside = x < g.W && y < g.H;
  float e1[3] = { 0.f, 0.f, 0.f }, e0[3] = { 0.f, 0.f, 0.f };
  // tiles whose windows stay inside the picture read their candidates without clamping
  const bool interior = x0 >= SR && y0 >= SR && x0 + kCpsTX + SR <= g.W && y0 + kCpsTY + SR <= g.H;
  auto search = [&](auto in_tag) {
  constexpr bool IN = decltype(in_tag)::value;
    float gc[3], tg[3], rg[3];
    for(int c = 0; c < 3; c++)
    {
      gc[c] = gcd[b * 3 + c];
      tg[c] = __fadd_rn(s_rt[c][ly + SR][lx + SR].y, gc[c]);
      rg[c] = __fsub_rn(s_rt[c][ly + SR][lx + SR].x, gc[c]);
    }
    const float2 ntg[3] = { make_float2(-tg[0], -rg[0]), make_float2(-tg[1], -rg[1]), make_float2(-tg[2], -rg[2]) };
    const float2 wp0 = make_float2(w0, w0), wp1 = make_float2(w1, w1), wp2 = make_float2(w2, w2);
    float best1 = INFINITY, best0 = INFINITY;
    int k1 = 0, k0 = 0;
    #pragma unroll
    for(int dy = 0; dy <= 2 * SR; dy++)
      #pragma unroll
      for(int dx = 0; dx <= 2 * SR; dx++)
      {
        // clamped candidate (x+dx-SR, y+dy-SR) in staged coordinates
        const int cx = IN ? lx + dx : min(max(x + dx - SR, 0), g.W - 1) - x0 + SR;
        const int cy = IN ? ly + dy : min(max(y + dy - SR, 0), g.H - 1) - y0 + SR;
        // both directions in packed FP32: (ref - tg, tst - rg) per component, the negated
        // differences (their squares are the same), then the weighted error
        // ((w0 d0^2) + (w1 d1^2)) + (w2 d2^2) lane by lane, without contraction: the same
        // rounding as separate tensor ops
        const float2 d0 = __fadd2_rn(s_rt[0][cy][cx], ntg[0]);
        const float2 d1 = __fadd2_rn(s_rt[1][cy][cx], ntg[1]);
        const float2 d2 = __fadd2_rn(s_rt[2][cy][cx], ntg[2]);
        const float2 E = __fadd2_rn(__fadd2_rn(__fmul2_rn(wp0, __fmul2_rn(d0, d0)), __fmul2_rn(wp1, __fmul2_rn(d1, d1))),
                                    __fmul2_rn(wp2, __fmul2_rn(d2, d2)));
        const float E1 = E.x, E0 = E.y;
        const int k = dy * (2 * SR + 1) + dx;
        if(E1 < best1) { best1 = E1; k1 = k; }
        if(E0 < best0) { best0 = E0; k0 = k; }
      }
    const int c1x = min(max(x + k1 % (2 * SR + 1) - SR, 0), g.W - 1) - x0 + SR, c1y = min(max(y + k1 / (2 * SR + 1) - SR, 0), g.H - 1) - y0 + SR;
    const int c0x = min(max(x + k0 % (2 * SR + 1) - SR, 0), g.W - 1) - x0 + SR, c0y = min(max(y + k0 / (2 * SR + 1) - SR, 0), g.H - 1) - y0 + SR;
    // stored index: the clamped displacement's position in the window, so that a pixel's
    // target is p + (k % side - SR, k / side - SR) without clamping and the gradient gather can
    // test "does p map to q" with one comparison
    int m1 = (c1y - ly) * (2 * SR + 1) + (c1x - lx), m0 = (c0y - ly) * (2 * SR + 1) + (c0x - lx);
    const int64_t pix = (int64_t)y * g.W + x;
    float* scp1 = scp + (int64_t)b * 3 * g.plane;
    float* scp0 = scp + ((int64_t)g.n + b) * 3 * g.plane;
    for(int c = 0; c < 3; c++)
    {
      const float rv = s_rt[c][c1y][c1x].x, tv = s_rt[c][c0y][c0x].y;
      e1[c] = __fsub_rn(tg[c], rv);
      e0[c] = __fsub_rn(rg[c], tv);
      const float a1 = __fsub_rn(rv, gc[c]), a0 = __fadd_rn(tv, gc[c]);
      if(a1 >= 0.f && a1 <= 1.f) m1 |= 256 << c;
      if(a0 >= 0.f && a0 <= 1.f) m0 |= 256 << c;
      scp1[(int64_t)c * g.plane + pix] = fminf(fmaxf(a1, 0.f), 1.f);
      scp0[(int64_t)c * g.plane + pix] = fminf(fmaxf(a0, 0.f), 1.f);
    }
    maps[(int64_t)b * g.plane + pix] = (uint16_t)m1;
    maps[((int64_t)g.n + b) * g.plane + pix] = (uint16_t)m0;
  };
  if(inside)
  {
    if(interior) search(std::true_type{});
    else         search(std::false_type{});
  }
  // per-block partials: squared errors [R2T c0..2, T2R c0..2], then the errors themselves (the
  // backward's d loss / d GCD takes 2 g_sse sum(e) per direction and component from them)
  const float v[12] = { e1[0] * e1[0], e1[1] * e1[1], e1[2] * e1[2], e0[0] * e0[0], e0[1] * e0[1], e0[2] * e0[2],
                        e1[0], e1[1], e1[2], e0[0], e0[1], e0[2] };
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  #pragma unroll
  for(int i = 0; i < 12; i++)
  {
    const float s = warp_sum(v[i]);
    if(lane == 0) s_red[warp][i] = s;
  }
  __syncthreads();
  if(threadIdx.x < 12)
  {
    double s = 0.0;
    for(int w = 0; w < 8; w++) s += (double)s_red[w][threadIdx.x];
    const int half = threadIdx.x / 6, d = (threadIdx.x % 6) / 3, c = threadIdx.x % 3;
    sse_part[((int64_t)half * g.n * 6 + ((int64_t)b * 2 + d) * 3 + c) * blocks_per_image + blockIdx.x] = s;
  }
}

// sum of per-block partials: out[i] = sum_k part[i][k] (compensated, fixed order), one
// 256-thread block per output: FP64 adds are slow on this part, so they are spread wide
constexpr int kSumThreads = 256;
__global__ void __launch_bounds__(kSumThreads) k_loss_sum_parts(const double* __restrict__ part, int nparts, int nout,
                                                                double* __restrict__ out, double scale)
{
  __shared__ double scratch[2 * (kSumThreads / 32)];
  const int i = blockIdx.x;
  if(i >= nout) return;
  Kbns k = { 0.0, 0.0 };
  for(int j = threadIdx.x; j < nparts; j += kSumThreads) k = kbns_add(k, part[(int64_t)i * nparts + j]);
  const double t = block_kbns(k, scratch);
  if(threadIdx.x == 0) out[i] = t * scale;
}

// ---- backward -------------------------------------------------------------------------------
struct BwdArgs {
  Geo g;
  int sr;
  const float* gcd;
  const int* gcd_ok;
  const uint16_t* maps;      // [2][n][H][W]: argmin index (bits 0-7), unclipped SCP (bits 8-10)
  const float* dy;           // [2][n][3][H][W]: T2R then R2T
  const double* g_sse;       // [n][2][3]
  const double* esum;        // [n][2][3]: sums of the errors (forward)
  double* g_part;            // [n*3][blocks]: SCP terms of d loss / d GCD
  const double* g_gcd;       // [n*3] (combine pass)
  float* g_tst;
  int blocks_per_image;
};

// d loss / d GCD_c = sum over pixels of 2 g_sse(R2T) e1 - 2 g_sse(T2R) e0 (the errors move
// with +GCD and -GCD) plus the SCP terms: -dSCP1 where SCP1 = clip(R - GCD) is not clipped,
// +dSCP0 where SCP0 = clip(T + GCD) is not. The error terms factor into 2 g_sse sum(e), whose
// sums the forward kept; this kernel sums the SCP terms, kLossGgPx pixels per block (four per
// thread, vector loads when the plane size allows), FP32 within the block, FP64 across blocks.
__global__ void __launch_bounds__(256) k_loss_gcd_grad_part(BwdArgs a)
{
  __shared__ float s_red[8][3];
  const Geo& g = a.g;
  const int b = blockIdx.y;
  const int64_t p0 = (int64_t)blockIdx.x * kLossGgPx + 4 * threadIdx.x;
  const uint16_t* M1 = a.maps + (int64_t)b * g.plane;
  const uint16_t* M0 = a.maps + ((int64_t)g.n + b) * g.plane;
  const float* D1 = a.dy + (int64_t)b * 3 * g.plane;             // d/dSCP1 (T2R)
  const float* D0 = a.dy + ((int64_t)g.n + b) * 3 * g.plane;     // d/dSCP0 (R2T)
  float v[3] = { 0.f, 0.f, 0.f };
  if((g.plane & 3) == 0 && p0 + 3 < g.plane)
  {
    const ushort4 m1 = *reinterpret_cast<const ushort4*>(M1 + p0);
    const ushort4 m0 = *reinterpret_cast<const ushort4*>(M0 + p0);
    float4 d1[3], d0[3];
    #pragma unroll
    for(int c = 0; c < 3; c++)
    {
      d1[c] = *reinterpret_cast<const float4*>(D1 + (int64_t)c * g.plane + p0);
      d0[c] = *reinterpret_cast<const float4*>(D0 + (int64_t)c * g.plane + p0);
    }
    #pragma unroll
    for(int c = 0; c < 3; c++)
    {
      const int bit = 256 << c;
      float t = 0.f;
      if(m1.x & bit) t -= d1[c].x;
      if(m0.x & bit) t += d0[c].x;
      if(m1.y & bit) t -= d1[c].y;
      if(m0.y & bit) t += d0[c].y;
      if(m1.z & bit) t -= d1[c].z;
      if(m0.z & bit) t += d0[c].z;
      if(m1.w & bit) t -= d1[c].w;
      if(m0.w & bit) t += d0[c].w;
      v[c] = t;
    }
  }
  else
    for(int64_t p = p0; p < min(p0 + 4, g.plane); p++)
    {
      const int m1 = M1[p], m0 = M0[p];
      #pragma unroll
      for(int c = 0; c < 3; c++)
      {
        if(m1 & (256 << c)) v[c] -= D1[(int64_t)c * g.plane + p];
        if(m0 & (256 << c)) v[c] += D0[(int64_t)c * g.plane + p];
      }
    }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  #pragma unroll
  for(int c = 0; c < 3; c++)
  {
    const float s = warp_sum(v[c]);
    if(lane == 0) s_red[warp][c] = s;
  }
  __syncthreads();
  if(threadIdx.x < 3)
  {
    double s = 0.0;
    for(int w = 0; w < 8; w++) s += (double)s_red[w][threadIdx.x];
    a.g_part[((int64_t)b * 3 + threadIdx.x) * a.blocks_per_image + blockIdx.x] = s;
  }
}

// d loss / d T(q): the SSIM T2R term already in g_tst, plus the R2T error at q, plus every T2R
// error and R2T SCP sample read from q (gathered over the window), plus the GCD term. A block
// stages a 32x16 tile plus the search-range halo of the T2R argmin indices, the reference and
// d/dSCP0 in shared memory, so the R2T target and every gathered neighbour are shared-memory
// reads; each thread takes two pixels (rows ly and ly + 8).
template <int SR>
__global__ void __launch_bounds__(256) k_loss_grad(BwdArgs a)
{
  constexpr int side = 2 * SR + 1;
  constexpr int HW = kGradTX + 2 * SR, HH = kGradTY + 2 * SR, HN = HW * HH;
  __shared__ uint16_t s_m0[HN];
  __shared__ float s_r[3][HN];
  __shared__ float s_d[3][HN];
  __shared__ float s_f[4][3];   // 2 g_sse(R2T), -2 g_sse(T2R), -g_gcd/area (or 0 when clipped), GCD
  const Geo& g = a.g;
  const int b = blockIdx.y;
  const int tiles_x = (g.W + kGradTX - 1) / kGradTX;
  const int x0 = (blockIdx.x % tiles_x) * kGradTX, y0 = (blockIdx.x / tiles_x) * kGradTY;
  const uint16_t* m0map = a.maps + ((int64_t)g.n + b) * g.plane;
  const float* R = g.ref + (int64_t)b * 3 * g.plane;
  const float* D0 = a.dy + ((int64_t)g.n + b) * 3 * g.plane;
  for(int i = threadIdx.x; i < HN; i += blockDim.x)
  {
    const int r = i / HW, q = i - r * HW;
    const int px = x0 - SR + q, py = y0 - SR + r;
    const bool in = px >= 0 && px < g.W && py >= 0 && py < g.H;
    const int64_t o = (int64_t)py * g.W + px;
    // outside the picture: an index that never maps back into the tile
    s_m0[i] = in ? m0map[o] : (uint16_t)0xffffu;
    #pragma unroll
    for(int c = 0; c < 3; c++)
    {
      s_r[c][i] = in ? R[(int64_t)c * g.plane + o] : 0.f;
      s_d[c][i] = in ? D0[(int64_t)c * g.plane + o] : 0.f;
    }
  }
  if(threadIdx.x < 3)
  {
    const int c = threadIdx.x;
    const double gs1 = a.g_sse[(b * 2 + 0) * 3 + c], gs0 = a.g_sse[(b * 2 + 1) * 3 + c];
    const double gg = a.g_gcd[b * 3 + c] + 2.0 * gs1 * a.esum[(b * 2 + 0) * 3 + c] - 2.0 * gs0 * a.esum[(b * 2 + 1) * 3 + c];
    s_f[0][c] = (float)(2.0 * gs1);
    s_f[1][c] = (float)(-2.0 * gs0);
    s_f[2][c] = a.gcd_ok[b * 3 + c] ? (float)(-gg / (double)g.plane) : 0.0f;
    s_f[3][c] = a.gcd[b * 3 + c];
  }
  __syncthreads();
  const float* T = g.tst + (int64_t)b * 3 * g.plane;
  const int lx = threadIdx.x % kGradTX;
  #pragma unroll 1
  for(int rr = 0; rr < 2; rr++)
  {
    const int ly = threadIdx.x / kGradTX + 8 * rr;
    const int x = x0 + lx, y = y0 + ly;
    if(x >= g.W || y >= g.H) break;
    const int64_t q = (int64_t)y * g.W + x;
    const int cq = (ly + SR) * HW + lx + SR;
    // the stored index is the clamped displacement's window position: the target is inside the
    // picture and within the halo
    const int k1 = a.maps[(int64_t)b * g.plane + q] & 255;
    const int c1 = cq + (k1 / side - SR) * HW + (k1 % side - SR);
    float acc[3], tq[3];
    #pragma unroll
    for(int c = 0; c < 3; c++)
    {
      tq[c] = T[(int64_t)c * g.plane + q];
      const float e1 = __fsub_rn(__fadd_rn(tq[c], s_f[3][c]), s_r[c][c1]);
      acc[c] = a.g_tst[((int64_t)b * 3 + c) * g.plane + q] + s_f[0][c] * e1 + s_f[2][c];
    }
    // pixels p = q + (dx, dy) whose T2R argmin reads q: those whose stored (clamped) displacement
    // is (-dx, -dy); the halo's 0xffff never matches. The matches are gathered into a bit mask
    // first and then visited in the same (row-major) order, so that a warp runs the reads of a
    // neighbour only as many times as its busiest lane has matches, not once per neighbour.
    constexpr int NW = (side * side + 31) / 32;
    uint32_t hits[NW];
    #pragma unroll
    for(int w = 0; w < NW; w++) hits[w] = 0u;
    #pragma unroll
    for(int dy = -SR; dy <= SR; dy++)
      #pragma unroll
      for(int dx = -SR; dx <= SR; dx++)
        if((s_m0[cq + dy * HW + dx] & 255) == (SR - dy) * side + (SR - dx))
        {
          const int i = (dy + SR) * side + dx + SR;
          hits[i >> 5] |= 1u << (i & 31);
        }
    #pragma unroll
    for(int w = 0; w < NW; w++)
      while(hits[w])
      {
        const int i = 32 * w + __ffs(hits[w]) - 1;
        hits[w] &= hits[w] - 1;
        const int dy = i / side - SR, dx = i - (i / side) * side - SR;
        const int pi = cq + dy * HW + dx;
        const int m0 = s_m0[pi];
        #pragma unroll
        for(int c = 0; c < 3; c++)
        {
          const float e0 = __fsub_rn(__fsub_rn(s_r[c][pi], s_f[3][c]), tq[c]);
          float v = s_f[1][c] * e0;
          if(m0 & (256 << c)) v += s_d[c][pi];
          acc[c] += v;
        }
      }
    #pragma unroll
    for(int c = 0; c < 3; c++) a.g_tst[((int64_t)b * 3 + c) * g.plane + q] = acc[c];
  }
}

size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

// The SSIM jobs of the loss, job k = (b * 2 + d) * 3 + c: d 0 = R2T: SSIM(R, SCP0), d 1 = T2R:
// SSIM(T, SCP1). One definition serves the host (tile counts) and the device: the tables are
// written on the device from this by-value descriptor, so a call copies no host memory.
struct LossSsimDesc {
  const float* ref;
  const float* tst;
  const float* scp;
  float* partial;        // forward: per-tile row sums
  double* ssim;          // forward: values [n][2][3]
  const double* g_ssim;  // backward: upstream gradients [n][2][3]
  float* g_tst;          // backward: d/dT
  float* dy;             // backward: d/dSCP, T2R then R2T
  int n, W, H, tiles_x, tiles_y, btx, bty;
};

__host__ __device__ inline SsimJob loss_ssim_job(const LossSsimDesc& D, int k)
{
  const int b = k / 6, d = (k / 3) % 2, c = k % 3;
  const size_t plane = (size_t)D.W * D.H;
  SsimJob j{};
  j.a.ptr = (d == 0 ? D.ref : D.tst) + ((size_t)b * 3 + c) * plane; j.a.stride = D.W; j.a.sbytes = 4; j.a.shift = 0;
  j.b.ptr = D.scp + (((size_t)(d == 0 ? D.n : 0) + b) * 3 + c) * plane; j.b.stride = D.W; j.b.sbytes = 4; j.b.shift = 0;
  j.W = D.W; j.H = D.H; j.calc_l = 1;
  j.c1 = 0.01f * 0.01f; j.c2 = 0.03f * 0.03f;
  j.tiles_x = D.tiles_x; j.tiles_y = D.tiles_y; j.tile_base = k * D.tiles_x * D.tiles_y;
  j.partial = D.partial + (size_t)k * (D.H > 10 ? D.H - 10 : 0) * D.tiles_x;
  j.out = D.ssim + k;
  return j;
}

// T2R (d 1) writes d/dT into g_tst and d/dSCP1 into dy[0]; R2T (d 0) writes d/dSCP0 into dy[1]
__host__ __device__ inline SsimBwdJob loss_ssim_bwd_job(const LossSsimDesc& D, int k)
{
  const int b = k / 6, d = (k / 3) % 2, c = k % 3;
  const size_t plane = (size_t)D.W * D.H, pl = ((size_t)b * 3 + c) * plane;
  SsimBwdJob j{};
  j.a.ptr = (d == 0 ? D.ref : D.tst) + pl; j.a.stride = D.W; j.a.sbytes = 4;
  j.b.ptr = D.scp + (((size_t)(d == 0 ? D.n : 0) + b) * 3 + c) * plane; j.b.stride = D.W; j.b.sbytes = 4;
  j.W = D.W; j.H = D.H; j.c1 = 0.01f * 0.01f; j.c2 = 0.03f * 0.03f;
  j.tiles_x = D.btx; j.tiles_y = D.bty; j.tile_base = k * D.btx * D.bty;
  j.g = D.g_ssim + k;
  j.outx = d == 1 ? D.g_tst + pl : nullptr;
  j.outy = D.dy + (((size_t)(d == 1 ? 0 : D.n) + b) * 3 + c) * plane;
  return j;
}

__global__ void k_loss_ssim_jobs(LossSsimDesc D, SsimJob* __restrict__ out)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if(k < D.n * 6) out[k] = loss_ssim_job(D, k);
}

__global__ void k_loss_ssim_bwd_jobs(LossSsimDesc D, SsimBwdJob* __restrict__ out)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if(k < D.n * 6) out[k] = loss_ssim_bwd_job(D, k);
}

}  // namespace

LossLayout loss_layout(int n, int W, int H, int window)
{
  LossLayout L;
  std::memset(&L, 0, sizeof(L));
  L.n = n; L.W = W; L.H = H; L.window = window;
  L.tiles_x = ssim_tiles_x(W, window);
  L.tiles_y = ssim_tiles_y(H);
  L.cps_blocks = ((W + kCpsTX - 1) / kCpsTX) * ((H + kCpsTY - 1) / kCpsTY);
  L.gg_blocks = (int)(((int64_t)W * H + kLossGgPx - 1) / kLossGgPx);
  L.grad_blocks = ((W + kGradTX - 1) / kGradTX) * ((H + kGradTY - 1) / kGradTY);
  const size_t plane = (size_t)W * H;
  size_t o = 0;
  L.gcd_part = o; o += al256(sizeof(double) * n * 3 * kLossGcdChunks);
  L.gcd = o;      o += al256(sizeof(float) * n * 3) + al256(sizeof(int) * n * 3);
  L.maps = o;     o += al256(sizeof(uint16_t) * 2 * (size_t)n * plane);
  L.scp = o;      o += al256(sizeof(float) * 2 * (size_t)n * 3 * plane);
  L.sse_part = o; o += al256(sizeof(double) * 2 * (size_t)n * 6 * L.cps_blocks);
  L.esum = o;     o += al256(sizeof(double) * (size_t)n * 6);
  L.sjobs = o;    o += al256(std::max(sizeof(SsimJob), sizeof(SsimBwdJob)) * n * 6);
  L.partial = o;  o += al256(sizeof(float) * (size_t)n * 6 * std::max(0, H - 10) * L.tiles_x);
  L.dy = o;       o += al256(sizeof(float) * 2 * (size_t)n * 3 * plane);
  L.g_part = o;   o += al256(sizeof(double) * (size_t)n * 3 * L.gg_blocks) + al256(sizeof(double) * n * 3);
  L.bytes = o;
  return L;
}

cudaError_t loss_forward(const LossArgs& a, double* sse, double* ssim, cudaStream_t st)
{
  const LossLayout& L = a.L;
  Geo g = { a.tst, a.ref, a.n, a.W, a.H, (int64_t)a.W * a.H };
  double* gpart = (double*)(a.ws + L.gcd_part);
  float* gcd = (float*)(a.ws + L.gcd);
  int* ok = (int*)(a.ws + L.gcd + al256(sizeof(float) * a.n * 3));
  uint16_t* maps = (uint16_t*)(a.ws + L.maps);
  float* scp = (float*)(a.ws + L.scp);
  double* ssep = (double*)(a.ws + L.sse_part);
  k_loss_gcd_part<<<dim3(kLossGcdChunks, a.n * 3), 256, 0, st>>>(g, gpart);
  k_loss_gcd_final<<<(a.n * 3 + 63) / 64, 64, 0, st>>>(g, gpart, a.unc[0], a.unc[1], a.unc[2], gcd, ok);
  const dim3 grid(L.cps_blocks, a.n);
  switch(a.sr)
  {
    case 1: k_loss_cps<1><<<grid, kCpsTX * kCpsTY, 0, st>>>(g, a.w_search[0], a.w_search[1], a.w_search[2], gcd, maps, scp, ssep, L.cps_blocks); break;
    case 2: k_loss_cps<2><<<grid, kCpsTX * kCpsTY, 0, st>>>(g, a.w_search[0], a.w_search[1], a.w_search[2], gcd, maps, scp, ssep, L.cps_blocks); break;
    case 3: k_loss_cps<3><<<grid, kCpsTX * kCpsTY, 0, st>>>(g, a.w_search[0], a.w_search[1], a.w_search[2], gcd, maps, scp, ssep, L.cps_blocks); break;
    default: k_loss_cps<4><<<grid, kCpsTX * kCpsTY, 0, st>>>(g, a.w_search[0], a.w_search[1], a.w_search[2], gcd, maps, scp, ssep, L.cps_blocks); break;
  }
  k_loss_sum_parts<<<a.n * 6, kSumThreads, 0, st>>>(ssep, L.cps_blocks, a.n * 6, sse, 1.0);
  k_loss_sum_parts<<<a.n * 6, kSumThreads, 0, st>>>(ssep + (size_t)a.n * 6 * L.cps_blocks, L.cps_blocks, a.n * 6,
                                           (double*)(a.ws + L.esum), 1.0);
  // SSIM jobs: (b, d, c) -> ssim[b][d][c], their table written on the device
  LossSsimDesc D{};
  D.ref = a.ref; D.tst = a.tst; D.scp = scp; D.partial = (float*)(a.ws + L.partial); D.ssim = ssim;
  D.n = a.n; D.W = a.W; D.H = a.H; D.tiles_x = L.tiles_x; D.tiles_y = L.tiles_y;
  const int nj = a.n * 6;
  std::vector<SsimJob> jobs(nj);
  for(int k = 0; k < nj; k++) jobs[k] = loss_ssim_job(D, k);
  SsimJob* d_jobs = (SsimJob*)(a.ws + L.sjobs);
  k_loss_ssim_jobs<<<(nj + 127) / 128, 128, 0, st>>>(D, d_jobs);
  cudaError_t e = launch_ssim(d_jobs, jobs.data(), nj, a.window, st);
  if(e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t loss_backward(const LossArgs& a, const double* g_sse, const double* g_ssim, float* g_tst, cudaStream_t st)
{
  const LossLayout& L = a.L;
  Geo g = { a.tst, a.ref, a.n, a.W, a.H, (int64_t)a.W * a.H };
  float* scp = (float*)(a.ws + L.scp);
  float* dy = (float*)(a.ws + L.dy);
  // SSIM backward jobs, their table written on the device
  LossSsimDesc D{};
  D.ref = a.ref; D.tst = a.tst; D.scp = scp; D.g_ssim = g_ssim; D.g_tst = g_tst; D.dy = dy;
  D.n = a.n; D.W = a.W; D.H = a.H; D.btx = ssim_bwd_tiles(a.W); D.bty = ssim_bwd_segments(a.H);
  const int nj = a.n * 6;
  std::vector<SsimBwdJob> jobs(nj);
  for(int k = 0; k < nj; k++) jobs[k] = loss_ssim_bwd_job(D, k);
  SsimBwdJob* d_jobs = (SsimBwdJob*)(a.ws + L.sjobs);
  k_loss_ssim_bwd_jobs<<<(nj + 127) / 128, 128, 0, st>>>(D, d_jobs);
  cudaError_t e = launch_ssim_bwd(d_jobs, jobs.data(), nj, a.window, st);
  if(e != cudaSuccess) return e;
  BwdArgs ba;
  ba.g = g; ba.sr = a.sr;
  ba.gcd = (const float*)(a.ws + L.gcd);
  ba.gcd_ok = (const int*)(a.ws + L.gcd + al256(sizeof(float) * a.n * 3));
  ba.maps = (const uint16_t*)(a.ws + L.maps);
  ba.dy = dy;
  ba.g_sse = g_sse;
  ba.esum = (const double*)(a.ws + L.esum);
  ba.g_part = (double*)(a.ws + L.g_part);
  double* g_gcd = (double*)(a.ws + L.g_part + al256(sizeof(double) * (size_t)a.n * 3 * L.gg_blocks));
  ba.g_gcd = g_gcd;
  ba.g_tst = g_tst;
  ba.blocks_per_image = L.gg_blocks;
  k_loss_gcd_grad_part<<<dim3(L.gg_blocks, a.n), 256, 0, st>>>(ba);
  k_loss_sum_parts<<<a.n * 3, kSumThreads, 0, st>>>(ba.g_part, L.gg_blocks, a.n * 3, g_gcd, 1.0);
  const dim3 grid(L.grad_blocks, a.n);
  switch(a.sr)
  {
    case 1: k_loss_grad<1><<<grid, 256, 0, st>>>(ba); break;
    case 2: k_loss_grad<2><<<grid, 256, 0, st>>>(ba); break;
    case 3: k_loss_grad<3><<<grid, 256, 0, st>>>(ba); break;
    default: k_loss_grad<4><<<grid, 256, 0, st>>>(ba); break;
  }
  return cudaGetLastError();
}

}  // namespace qmiv
