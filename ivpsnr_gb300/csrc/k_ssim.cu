// SSIM family kernels: windowed structural similarity (libs/pmbb-ivqm/src/xStructSim.cpp:15-60),
// its picture mean (xSSIM.cpp:91-140), the MS-SSIM pyramid (xSSIM.cpp:67-87,142-148 with
// DownsampleHV, libs/pmbb-core/src/xPixelOpsSTD.cpp:50-67) and the IV-SSIM combination
// (xSSIM.cpp:166-210).
//
// The reference evaluates 10x10 (REF10) window moments in FP64 with FP32 coefficients per
// output pixel (800 multiply-adds). Here the window is separable: the coefficient table is
// the outer product of the normalised 11-tap Gaussian g rounded to 10 decimals, so the
// moments are computed as a horizontal then a vertical 10-tap (or 11-tap) pass in FP32
// (~100 multiply-adds per pixel), on samples centred by a per-tile integer offset c so that
// E[x^2] - E[x]^2 does not cancel. With W0 = (sum g)^2 the moments about zero follow from
// the centred sums S1 = sum w (x-c), S2 = sum w (x-c)^2:
//   mu  = S1 + c W0,   var = S2 - S1^2 + (1-W0)(2c S1 + c^2 W0),
//   cov = Sxy - S1x S1y + (1-W0)(c (S1x + S1y) + c^2 W0).
// Rows are summed per 32-pixel tile in FP32 and across tiles and rows in FP64 (compensated),
// the picture sum divided by W*H as the reference does.
#include <cfloat>

#include "qmiv_device.cuh"
#include "qmiv_ssim.h"

namespace qmiv {

__constant__ float c_g[11];      // 1-D window factor
__constant__ float c_w0[2];      // W0 = (sum g)^2 for the 10- and 11-tap windows
__constant__ float c_om[2];      // 1 - W0, rounded from FP64 (not formed in FP32)
__constant__ double c_w0d[2];
__constant__ double c_omd[2];

namespace {

constexpr int kTX = 32, kThreads = 256, kIH = 64;  // staged rows: output rows + window - 1
template <int WIN> struct SGeo {
  static constexpr int TY = kIH - WIN + 1;          // 55 output rows (REF10), 54 (GAUSS11)
  static constexpr int IW = kTX + WIN - 1;          // staged columns
  static constexpr int RS = ((IW + 2) / 4) * 4 + 1; // row stride = 1 (mod 4): conflict-free h-pass reads
  static constexpr int HS = kTX + 1;                // h-moment row stride (= 1 mod 4)
  static constexpr int RPT = (TY + 7) / 8;          // output rows per thread in the v-pass
  static constexpr int SMEM = (2 * kIH * RS + 5 * kIH * HS) * 4;
};

__device__ __forceinline__ int ld_plane(const SsimPlane& p, int x, int y)
{
  const int64_t o = (int64_t)(y >> p.shift) * p.stride + (x >> p.shift);
  return p.sbytes == 1 ? (int)__ldg((const uint8_t*)p.ptr + o) : (int)__ldg((const uint16_t*)p.ptr + o);
}

__device__ __forceinline__ int find_ssim_job(const SsimJob* __restrict__ jobs, int n, int b)
{
  int lo = 0, hi = n - 1;
  while(lo < hi) { const int mid = (lo + hi + 1) >> 1; if(jobs[mid].tile_base <= b) lo = mid; else hi = mid - 1; }
  return lo;
}

// Stage one plane's rows (warp per row, lanes along x) as centred floats; rows and columns past
// the picture clamp (they only feed outputs outside the valid region).
template <typename T, int SH, int IW, int RS>
__device__ __forceinline__ void stage_rows(const SsimPlane& P, float* dst, int x0, int y0, int W, int H, int c)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for(int r = warp; r < kIH; r += kThreads / 32)
  {
    const int gy = min(y0 - 5 + r, H - 1);
    const T* row = reinterpret_cast<const T*>(P.ptr) + (int64_t)(gy >> SH) * P.stride;
    for(int q = lane; q < IW; q += 32)
    {
      const int gx = min(x0 - 5 + q, W - 1);
      dst[r * RS + q] = (float)((int)__ldg(row + (gx >> SH)) - c);
    }
  }
}

template <int IW, int RS>
__device__ __forceinline__ void stage_plane(const SsimPlane& P, float* dst, int x0, int y0, int W, int H, int c)
{
  if(P.sbytes == 1) { if(P.shift) stage_rows<uint8_t, 1, IW, RS>(P, dst, x0, y0, W, H, c); else stage_rows<uint8_t, 0, IW, RS>(P, dst, x0, y0, W, H, c); }
  else              { if(P.shift) stage_rows<uint16_t, 1, IW, RS>(P, dst, x0, y0, W, H, c); else stage_rows<uint16_t, 0, IW, RS>(P, dst, x0, y0, W, H, c); }
}

template <int WIN>
__global__ void __launch_bounds__(kThreads) k_ssim(const SsimJob* __restrict__ jobs, int njobs)
{
  using G = SGeo<WIN>;
  extern __shared__ float smem[];
  float* s_in = smem;                       // [2][kIH][RS]
  float* s_h = smem + 2 * kIH * G::RS;      // [5][kIH][HS]
  __shared__ int s_c;

  const int jb = find_ssim_job(jobs, njobs, blockIdx.x);
  const SsimJob& J = jobs[jb];
  const int local = blockIdx.x - J.tile_base;
  const int ty = local / J.tiles_x, tx = local - ty * J.tiles_x;
  const int W = J.W, H = J.H;
  const int x0 = 5 + tx * kTX, y0 = 5 + ty * G::TY;
  const int x1 = min(x0 + kTX, W - 5), y1 = min(y0 + G::TY, H - 5);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  if(tid == 0) s_c = ld_plane(J.b, min((x0 + x1) >> 1, W - 1), min((y0 + y1) >> 1, H - 1));
  __syncthreads();
  const int c = s_c;
  stage_plane<G::IW, G::RS>(J.a, s_in, x0, y0, W, H, c);
  stage_plane<G::IW, G::RS>(J.b, s_in + kIH * G::RS, x0, y0, W, H, c);
  __syncthreads();

  // horizontal pass: item = (row, 4 consecutive output columns); 8 items per row
  #pragma unroll 1
  for(int item = tid; item < kIH * (kTX / 4); item += kThreads)
  {
    const int r = item >> 3, q0 = (item & 7) * 4;
    float a[4 + WIN - 1], b[4 + WIN - 1], aa[4 + WIN - 1], bb[4 + WIN - 1], ab[4 + WIN - 1];
    #pragma unroll
    for(int i = 0; i < 4 + WIN - 1; i++)
    {
      a[i] = s_in[r * G::RS + q0 + i];
      b[i] = s_in[kIH * G::RS + r * G::RS + q0 + i];
      aa[i] = a[i] * a[i]; bb[i] = b[i] * b[i]; ab[i] = a[i] * b[i];
    }
    #pragma unroll
    for(int o = 0; o < 4; o++)
    {
      float m0 = 0.f, m1 = 0.f, m2 = 0.f, m3 = 0.f, m4 = 0.f;
      #pragma unroll
      for(int k = 0; k < WIN; k++)
      {
        const float g = c_g[k];
        m0 = fmaf(g, a[o + k], m0); m1 = fmaf(g, b[o + k], m1);
        m2 = fmaf(g, aa[o + k], m2); m3 = fmaf(g, bb[o + k], m3); m4 = fmaf(g, ab[o + k], m4);
      }
      float* h = s_h + r * G::HS + q0 + o;
      h[0] = m0; h[kIH * G::HS] = m1; h[2 * kIH * G::HS] = m2; h[3 * kIH * G::HS] = m3; h[4 * kIH * G::HS] = m4;
    }
  }
  __syncthreads();

  // vertical pass: lane = column, warp = RPT consecutive output rows
  float acc[G::RPT][5];
  #pragma unroll
  for(int o = 0; o < G::RPT; o++)
    #pragma unroll
    for(int m = 0; m < 5; m++) acc[o][m] = 0.f;
  #pragma unroll
  for(int i = 0; i < G::RPT + WIN - 1; i++)
  {
    const int r = min(warp * G::RPT + i, kIH - 1);
    float hv[5];
    #pragma unroll
    for(int m = 0; m < 5; m++) hv[m] = s_h[m * kIH * G::HS + r * G::HS + lane];
    #pragma unroll
    for(int o = 0; o < G::RPT; o++)
    {
      const int k = i - o;
      if(k < 0 || k >= WIN) continue;
      const float g = c_g[k];
      #pragma unroll
      for(int m = 0; m < 5; m++) acc[o][m] = fmaf(g, hv[m], acc[o][m]);
    }
  }

  const int wi = WIN == 11 ? 1 : 0;
  const float w0 = c_w0[wi];
  const float om = c_om[wi];
  const float cf = (float)c;
  const float k_cc = (float)(c_omd[wi] * (double)c * (double)c * c_w0d[wi]);
  const float cw0 = cf * w0, om2c = om * 2.0f * cf, omc = om * cf;
  const float C1 = J.c1, C2 = J.c2;
  const bool calc_l = J.calc_l != 0;
  #pragma unroll
  for(int o = 0; o < G::RPT; o++)
  {
    const float S1a = acc[o][0], S1b = acc[o][1], S2a = acc[o][2], S2b = acc[o][3], Sab = acc[o][4];
    const float va = S2a - S1a * S1a + fmaf(om2c, S1a, k_cc);
    const float vb = S2b - S1b * S1b + fmaf(om2c, S1b, k_cc);
    const float cov = Sab - S1a * S1b + fmaf(omc, S1a + S1b, k_cc);
    float num = 2.0f * cov + C2, den = va + vb + C2;
    if(calc_l)
    { // L * CS = (nL nCS) / (dL dCS): one division (xStructSim.cpp:50-51)
      const float mua = S1a + cw0, mub = S1b + cw0;
      num *= 2.0f * mua * mub + C1;
      den *= mua * mua + mub * mub + C1;
    }
    const int y = y0 + warp * G::RPT + o, x = x0 + lane;
    float v = (y < y1 && x < x1) ? __fdividef(num, den) : 0.0f;
    #pragma unroll
    for(int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    if(lane == 0 && y < y1) J.partial[(int64_t)(y - 5) * J.tiles_x + tx] = v;
  }
}

// Picture sum of one SSIM job: rows summed over their tiles in FP64 (fixed order), rows combined
// with a compensated sum, divided by W*H (xSSIM.cpp:106-111).
__global__ void __launch_bounds__(256) k_ssim_finalize(const SsimJob* __restrict__ jobs, int njobs)
{
  __shared__ double scratch[16];
  const SsimJob& J = jobs[blockIdx.x];
  const int rows = max(0, J.H - 10);
  Kbns k = { 0.0, 0.0 };
  for(int r = threadIdx.x; r < rows; r += blockDim.x)
  {
    double s = 0.0;
    for(int t = 0; t < J.tiles_x; t++) s = __dadd_rn(s, (double)__ldcg(J.partial + (int64_t)r * J.tiles_x + t));
    k = kbns_add(k, s);
  }
  const double tot = block_kbns(k, scratch);
  if(threadIdx.x == 0) *J.out = __ddiv_rn(tot, (double)((int64_t)J.W * J.H));
}

// DownsampleHV to a 16-bit plane: d(x,y) = (s(2x,2y)+s(2x+1,2y)+s(2x,2y+1)+s(2x+1,2y+1)+2)>>2
__global__ void __launch_bounds__(256) k_downsample(const PyrStep* __restrict__ steps, int nsteps)
{
  const PyrStep& S = steps[blockIdx.y];
  const int x = blockIdx.x * 64 + (threadIdx.x & 63);
  for(int y = threadIdx.x >> 6; y < S.dh; y += 4)
  {
    if(x >= S.dw) break;
    const int sx = 2 * x, sy = 2 * y;
    const int v = ld_plane(S.src, sx, sy) + ld_plane(S.src, sx + 1, sy) + ld_plane(S.src, sx, sy + 1) + ld_plane(S.src, sx + 1, sy + 1);
    S.dst[(int64_t)y * S.dst_stride + x] = (uint16_t)((v + 2) >> 2);
  }
}

// Per frame: SSIM, MS-SSIM (product of per-scale scores to the scale weights,
// xStructSimConsts.h:27) and IV-SSIM (weighted, worse of both directions).
__global__ void k_ssim_combine(const SsimFrame* __restrict__ frames, int nframes, Params p)
{
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if(f >= nframes) return;
  const SsimFrame& F = frames[f];
  qmiv_frame_result* R = F.result;
  const double* v = F.vals;
  if(F.metrics & QMIV_M_SSIM)
  {
    double s[3] = { v[0], v[1], v[2] };
    for(int c = 0; c < 3; c++) R->ssim[c] = s[c];
    R->ssim[3] = 0.0;
    R->ssim_pic = weighted3(s, p.w_avg);
  }
  if(F.metrics & QMIV_M_MSSSIM)
  {
    const double wts[5] = { 0.0448, 0.2856, 0.3001, 0.2363, 0.1333 };
    double m[3];
    for(int c = 0; c < 3; c++)
    {
      double acc = 1.0;
      for(int i = 0; i < 5; i++) acc = __dmul_rn(acc, pow(v[3 + i * 3 + c], wts[i]));
      m[c] = acc;
      R->msssim[c] = acc;
    }
    R->msssim[3] = 0.0;
    R->msssim_pic = weighted3(m, p.w_avg);
  }
  if(F.metrics & QMIV_M_IVSSIM)
  {
    const double t2r[3] = { v[18], v[19], v[20] }, r2t[3] = { v[21], v[22], v[23] };
    const double a = weighted3(t2r, p.w_avg), b = weighted3(r2t, p.w_avg);
    R->ivssim_t2r = a;
    R->ivssim_r2t = b;
    R->ivssim = b < a ? b : a; // std::min(SSIM_T2R, SSIM_R2T) (xSSIM.cpp:205)
  }
}

}  // namespace

cudaError_t ssim_set_window_constants(const float g[11], const double w0[2])
{
  const float w0f[2] = { (float)w0[0], (float)w0[1] };
  const double omd[2] = { 1.0 - w0[0], 1.0 - w0[1] };
  const float omf[2] = { (float)omd[0], (float)omd[1] };
  cudaError_t e = cudaMemcpyToSymbol(c_g, g, sizeof(float) * 11);
  if(e == cudaSuccess) e = cudaMemcpyToSymbol(c_w0, w0f, sizeof(w0f));
  if(e == cudaSuccess) e = cudaMemcpyToSymbol(c_om, omf, sizeof(omf));
  if(e == cudaSuccess) e = cudaMemcpyToSymbol(c_w0d, w0, sizeof(double) * 2);
  if(e == cudaSuccess) e = cudaMemcpyToSymbol(c_omd, omd, sizeof(omd));
  return e;
}

int ssim_tiles_x(int W) { return W > 10 ? (W - 10 + kTX - 1) / kTX : 0; }
int ssim_tiles_y(int H, int window)
{
  const int ty = window == QMIV_SSIM_GAUSS11 ? SGeo<11>::TY : SGeo<10>::TY;
  return H > 10 ? (H - 10 + ty - 1) / ty : 0;
}

cudaError_t launch_ssim(const SsimJob* d_jobs, const SsimJob* h_jobs, int n, int window, cudaStream_t st)
{
  int blocks = 0;
  for(int i = 0; i < n; i++) blocks = h_jobs[i].tile_base + h_jobs[i].tiles_x * h_jobs[i].tiles_y;
  if(blocks > 0)
  {
    static bool attr = false;
    if(!attr)
    {
      cudaError_t e = cudaFuncSetAttribute(k_ssim<10>, cudaFuncAttributeMaxDynamicSharedMemorySize, SGeo<10>::SMEM);
      if(e == cudaSuccess) e = cudaFuncSetAttribute(k_ssim<11>, cudaFuncAttributeMaxDynamicSharedMemorySize, SGeo<11>::SMEM);
      if(e != cudaSuccess) return e;
      attr = true;
    }
    if(window == QMIV_SSIM_GAUSS11) k_ssim<11><<<blocks, kThreads, SGeo<11>::SMEM, st>>>(d_jobs, n);
    else                            k_ssim<10><<<blocks, kThreads, SGeo<10>::SMEM, st>>>(d_jobs, n);
    cudaError_t e = cudaGetLastError();
    if(e != cudaSuccess) return e;
  }
  k_ssim_finalize<<<n, 256, 0, st>>>(d_jobs, n);
  return cudaGetLastError();
}

cudaError_t launch_downsample(const PyrStep* d_steps, const PyrStep* h_steps, int n, cudaStream_t st)
{
  int maxw = 0;
  for(int i = 0; i < n; i++) maxw = h_steps[i].dw > maxw ? h_steps[i].dw : maxw;
  if(n == 0 || maxw == 0) return cudaSuccess;
  dim3 grid((maxw + 63) / 64, n);
  k_downsample<<<grid, 256, 0, st>>>(d_steps, n);
  return cudaGetLastError();
}

cudaError_t launch_ssim_combine(const SsimFrame* d_frames, int n, const Params& p, cudaStream_t st)
{
  if(n == 0) return cudaSuccess;
  k_ssim_combine<<<(n + 63) / 64, 64, 0, st>>>(d_frames, n, p);
  return cudaGetLastError();
}

}  // namespace qmiv
