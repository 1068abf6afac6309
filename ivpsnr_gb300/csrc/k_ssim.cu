// SSIM family kernels: windowed structural similarity (libs/pmbb-ivqm/src/xStructSim.cpp:15-60),
// its picture mean (xSSIM.cpp:91-140), the MS-SSIM pyramid (xSSIM.cpp:67-87,142-148 with
// DownsampleHV, libs/pmbb-core/src/xPixelOpsSTD.cpp:50-67) and the IV-SSIM combination
// (xSSIM.cpp:166-210).
//
// The reference evaluates 10x10 (REF10) window moments in FP64 with FP32 coefficients per
// output pixel (800 multiply-adds). Here the window is separable: the coefficient table is
// the outer product of the normalised 11-tap Gaussian g rounded to 10 decimals, so the
// moments are computed as a vertical then a horizontal 10-tap (or 11-tap) pass in FP32
// (~80 multiply-adds per pixel), on samples centred by a per-tile integer offset c so that
// E[x^2] - E[x]^2 does not cancel. With W0 = (sum g)^2 the moments about zero follow from
// the centred sums S1 = sum w (x-c), S2 = sum w (x-c)^2:
//   mu  = S1 + c W0,   var = S2 - S1^2 + (1-W0)(2c S1 + c^2 W0),
//   cov = Sxy - S1x S1y + (1-W0)(c (S1x + S1y) + c^2 W0).
// Only var_a + var_b enters the index, so four moment streams are filtered per pixel:
// S1a, S1b, S(a^2 + b^2) and S(ab). Two vertically adjacent rows travel together in one
// float2 through Blackwell's packed FP32 multiply-add (FFMA2), which halves the issue slots
// of the filter taps. Rows are summed per tile in FP32 and across tiles and rows in FP64
// (compensated), the picture sum divided by W*H as the reference does.
#include <cfloat>

#include "qmiv_device.cuh"
#include "qmiv_ssim.h"

namespace qmiv {

__constant__ float c_g[11];      // 1-D window factor
__constant__ float2 c_g2[11];    // (g, g) pairs for the packed filter
__constant__ float c_w0[2];      // W0 = (sum g)^2 for the 10- and 11-tap windows
__constant__ float c_om[2];      // 1 - W0, rounded from FP64 (not formed in FP32)
__constant__ double c_w0d[2];
__constant__ double c_omd[2];

namespace {

// Tile geometry. A block of 256 threads stages a 64-column strip of IH rows of both planes,
// filters it vertically into TY output rows (thread = staged column x 8 output rows, rows
// paired in float2), then horizontally (thread = output row pair x 4 output columns).
constexpr int kThreads = 256, kIW = 64, kTY = 32, kPairs = kTY / 2, kGroups = 14, kPS = 67;
template <int WIN> struct SGeo {
  static constexpr int TX = kIW - WIN + 1;          // 55 output columns (REF10), 54 (GAUSS11)
  static constexpr int IH = kTY + WIN - 1;          // staged rows
  static constexpr int RPW = (IH + 7) / 8;          // staged rows per warp
  // staged planes [2][IH][64] floats, vertical moments [4][16 pairs][kPS] float2 (odd pitch:
  // conflict-free reads down a column), row-pair reduction [7][16] float2
  static constexpr int SMEM = 2 * IH * kIW * 4 + 4 * kPairs * kPS * 8 + 7 * kPairs * 8;
  static_assert(4 * kGroups >= TX && 4 * (kGroups - 1) + 3 + WIN - 1 < kPS, "tile columns");
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

// Stage one plane: warp w loads rows w, w+8, ..., lanes the columns lane and lane+32; all loads
// are issued before the first store. Rows and columns past the picture clamp (they only feed
// outputs outside the valid region).
template <typename T, int SH, int IH>
__device__ __forceinline__ void stage_rows(const SsimPlane& P, float* dst, int x0, int y0, int W, int H, int c)
{
  constexpr int RPW = (IH + 7) / 8;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const T* base = reinterpret_cast<const T*>(P.ptr);
  const int gx0 = min(x0 - 5 + lane, W - 1) >> SH, gx1 = min(x0 + 27 + lane, W - 1) >> SH;
  int v[RPW][2];
  #pragma unroll
  for(int k = 0; k < RPW; k++)
  {
    const int i = min(warp + 8 * k, IH - 1);
    const T* row = base + (int64_t)(min(y0 - 5 + i, H - 1) >> SH) * P.stride;
    v[k][0] = __ldg(row + gx0);
    v[k][1] = __ldg(row + gx1);
  }
  #pragma unroll
  for(int k = 0; k < RPW; k++)
  {
    const int i = warp + 8 * k;
    if(i < IH)
    {
      dst[i * kIW + lane] = (float)(v[k][0] - c);
      dst[i * kIW + lane + 32] = (float)(v[k][1] - c);
    }
  }
}

template <int IH>
__device__ __forceinline__ void stage_plane(const SsimPlane& P, float* dst, int x0, int y0, int W, int H, int c)
{
  if(P.sbytes == 1) { if(P.shift) stage_rows<uint8_t, 1, IH>(P, dst, x0, y0, W, H, c); else stage_rows<uint8_t, 0, IH>(P, dst, x0, y0, W, H, c); }
  else              { if(P.shift) stage_rows<uint16_t, 1, IH>(P, dst, x0, y0, W, H, c); else stage_rows<uint16_t, 0, IH>(P, dst, x0, y0, W, H, c); }
}

__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }

template <int WIN>
__global__ void __launch_bounds__(kThreads, 3) k_ssim(const SsimJob* __restrict__ jobs, int njobs)
{
  using G = SGeo<WIN>;
  extern __shared__ __align__(16) float smem[];
  float* s_in = smem;                                              // [2][IH][64]
  float2* s_v = reinterpret_cast<float2*>(smem + 2 * G::IH * kIW); // [4][16][kPS]
  float2* s_red = s_v + 4 * kPairs * kPS;                          // [7][16]

  const int jb = find_ssim_job(jobs, njobs, blockIdx.x);
  const SsimJob& J = jobs[jb];
  const int local = blockIdx.x - J.tile_base;
  const int ty = local / J.tiles_x, tx = local - ty * J.tiles_x;
  const int W = J.W, H = J.H;
  const int x0 = 5 + tx * G::TX, y0 = 5 + ty * kTY;
  const int x1 = min(x0 + G::TX, W - 5), y1 = min(y0 + kTY, H - 5);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  // centring offset: the tile-centre sample of plane b (every thread loads the same address)
  const int c = ld_plane(J.b, min((x0 + x1) >> 1, W - 1), min((y0 + y1) >> 1, H - 1));
  stage_plane<G::IH>(J.a, s_in, x0, y0, W, H, c);
  stage_plane<G::IH>(J.b, s_in + G::IH * kIW, x0, y0, W, H, c);
  __syncthreads();

  // vertical pass: column q, output rows 8rg .. 8rg+7 as four row pairs; position i holds
  // the staged rows (8rg+i, 8rg+i+1), which output pair u takes with weight g[i - 2u]
  {
    const int q = tid & (kIW - 1), rg = tid >> 6;
    const float* sa = s_in + 8 * rg * kIW + q;
    const float* sb = sa + G::IH * kIW;
    float2 acc[4][4];
    #pragma unroll
    for(int u = 0; u < 4; u++)
      #pragma unroll
      for(int s = 0; s < 4; s++) acc[u][s] = make_float2(0.f, 0.f);
    #pragma unroll
    for(int i = 0; i < 6 + WIN; i++)
    {
      const float2 pa = make_float2(sa[i * kIW], sa[(i + 1) * kIW]);
      const float2 pb = make_float2(sb[i * kIW], sb[(i + 1) * kIW]);
      const float2 pq = __ffma2_rn(pa, pa, __fmul2_rn(pb, pb));
      const float2 px = __fmul2_rn(pa, pb);
      #pragma unroll
      for(int u = 0; u < 4; u++)
      {
        const int k = i - 2 * u;
        if(k < 0 || k >= WIN) continue;
        const float2 g = c_g2[k];
        acc[u][0] = __ffma2_rn(g, pa, acc[u][0]);
        acc[u][1] = __ffma2_rn(g, pb, acc[u][1]);
        acc[u][2] = __ffma2_rn(g, pq, acc[u][2]);
        acc[u][3] = __ffma2_rn(g, px, acc[u][3]);
      }
    }
    #pragma unroll
    for(int u = 0; u < 4; u++)
      #pragma unroll
      for(int s = 0; s < 4; s++) s_v[(s * kPairs + 4 * rg + u) * kPS + q] = acc[u][s];
  }
  __syncthreads();

  // horizontal pass and the index: row pair p (lanes 0-15 / 16-31), output columns 4gi .. 4gi+3
  if(warp < 7)
  {
    const int p = lane & 15, gi = 2 * warp + (lane >> 4), j0 = 4 * gi;
    float2 m[4][4];                                                 // [column][stream]
    #pragma unroll
    for(int s = 0; s < 4; s++)
    {
      const float2* v = s_v + (s * kPairs + p) * kPS + j0;
      #pragma unroll
      for(int jj = 0; jj < 4; jj++) m[jj][s] = make_float2(0.f, 0.f);
      #pragma unroll
      for(int t = 0; t < 3 + WIN; t++)
      {
        const float2 val = v[t];
        #pragma unroll
        for(int jj = 0; jj < 4; jj++)
        {
          const int k = t - jj;
          if(k < 0 || k >= WIN) continue;
          m[jj][s] = __ffma2_rn(c_g2[k], val, m[jj][s]);
        }
      }
    }

    const int wi = WIN == 11 ? 1 : 0;
    const float cf = (float)c;
    const float k_cc = (float)(c_omd[wi] * (double)c * (double)c * c_w0d[wi]);
    const float2 cw0 = f2(cf * c_w0[wi]), om2c = f2(c_om[wi] * 2.0f * cf), omc = f2(c_om[wi] * cf);
    const float2 vq0 = f2(2.0f * k_cc + J.c2), cv0 = f2(k_cc), two = f2(2.0f), c1 = f2(J.c1), c2 = f2(J.c2);
    const bool calc_l = J.calc_l != 0;
    const int ya = y0 + 2 * p;
    const bool row0 = ya < y1, row1 = ya + 1 < y1;
    float2 rs = make_float2(0.f, 0.f);
    #pragma unroll
    for(int jj = 0; jj < 4; jj++)
    {
      const float2 S1a = m[jj][0], S1b = m[jj][1], Sq = m[jj][2], Sx = m[jj][3];
      const float2 sab = __fadd2_rn(S1a, S1b);
      const float2 na = make_float2(-S1a.x, -S1a.y);
      // den: var_a + var_b + C2; num: 2 cov + C2
      float2 den = __ffma2_rn(om2c, sab, vq0);
      den = __fadd2_rn(den, __ffma2_rn(na, S1a, Sq));
      den = __ffma2_rn(make_float2(-S1b.x, -S1b.y), S1b, den);
      float2 cov = __ffma2_rn(omc, sab, cv0);
      cov = __fadd2_rn(cov, __ffma2_rn(na, S1b, Sx));
      float2 num = __ffma2_rn(two, cov, c2);
      if(calc_l)
      { // L * CS = (nL nCS) / (dL dCS): one division (xStructSim.cpp:50-51)
        const float2 mua = __fadd2_rn(S1a, cw0), mub = __fadd2_rn(S1b, cw0);
        num = __fmul2_rn(num, __ffma2_rn(__fmul2_rn(two, mua), mub, c1));
        den = __fmul2_rn(den, __ffma2_rn(mua, mua, __ffma2_rn(mub, mub, c1)));
      }
      const bool col = x0 + j0 + jj < x1;
      rs.x += (col && row0) ? __fdividef(num.x, den.x) : 0.0f;
      rs.y += (col && row1) ? __fdividef(num.y, den.y) : 0.0f;
    }
    rs.x += __shfl_xor_sync(0xffffffffu, rs.x, 16);
    rs.y += __shfl_xor_sync(0xffffffffu, rs.y, 16);
    if(lane < 16) s_red[warp * kPairs + p] = rs;
  }
  __syncthreads();
  if(tid < kTY)
  { // row tid of the tile: fixed-order sum over the 7 column warps
    const float* red = reinterpret_cast<const float*>(s_red) + ((tid >> 1) << 1) + (tid & 1);
    float s = 0.0f;
    #pragma unroll
    for(int w = 0; w < 7; w++) s += red[w * 2 * kPairs];
    const int y = y0 + tid;
    if(y < y1) J.partial[(int64_t)(y - 5) * J.tiles_x + tx] = s;
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
  float2 g2[11];
  for(int k = 0; k < 11; k++) g2[k] = make_float2(g[k], g[k]);
  cudaError_t e = cudaMemcpyToSymbol(c_g, g, sizeof(float) * 11);
  if(e == cudaSuccess) e = cudaMemcpyToSymbol(c_g2, g2, sizeof(g2));
  if(e == cudaSuccess) e = cudaMemcpyToSymbol(c_w0, w0f, sizeof(w0f));
  if(e == cudaSuccess) e = cudaMemcpyToSymbol(c_om, omf, sizeof(omf));
  if(e == cudaSuccess) e = cudaMemcpyToSymbol(c_w0d, w0, sizeof(double) * 2);
  if(e == cudaSuccess) e = cudaMemcpyToSymbol(c_omd, omd, sizeof(omd));
  return e;
}

int ssim_tiles_x(int W, int window)
{
  const int tx = window == QMIV_SSIM_GAUSS11 ? SGeo<11>::TX : SGeo<10>::TX;
  return W > 10 ? (W - 10 + tx - 1) / tx : 0;
}
int ssim_tiles_y(int H) { return H > 10 ? (H - 10 + kTY - 1) / kTY : 0; }

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
