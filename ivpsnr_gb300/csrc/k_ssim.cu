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
// S1a, S1b, S(a^2 + b^2) and S(ab), as two float2 pairs through Blackwell's packed FP32
// multiply-add (FFMA2), which halves the issue slots of the filter taps. Rows are summed per
// tile in FP32 and across tiles and rows in FP64 (compensated), the picture sum divided by
// W*H as the reference does.
#include <algorithm>
#include <cfloat>
#include <type_traits>

#include "qmiv_device.cuh"
#include "qmiv_ptx.cuh"
#include "qmiv_ssim.h"

namespace qmiv {

__constant__ float c_g[11];      // 1-D window factor
__constant__ float2 c_g2[11];    // (g, g) pairs for the packed filter
__constant__ float c_w0[2];      // W0 = (sum g)^2 for the 10- and 11-tap windows
__constant__ float c_om[2];      // 1 - W0, rounded from FP64 (not formed in FP32)
__constant__ double c_w0d[2];
__constant__ double c_omd[2];

namespace {

// Tile geometry. A persistent block of 256 threads walks the tiles of all jobs; per tile it
// stages a 64-column strip of IH rows of both planes as (a, b) pairs, filters it vertically
// into TY output rows (thread = staged column x 8 output rows), then horizontally (thread =
// output row x 7 output columns, all eight warps) and evaluates the index.
constexpr int kThreads = 256, kIW = 64, kTY = 32, kRP = 66, kHO = 7;
template <int WIN> struct SGeo {
  static constexpr int TX = kIW - WIN + 1;          // 55 output columns (REF10), 54 (GAUSS11)
  static constexpr int IH = kTY + WIN - 1;          // staged rows
  static constexpr int RPW = (IH + 7) / 8;          // staged rows per warp
  // staged (a, b) pairs [IH][64] float2; vertical moments [32][kRP] float4 (S1a, S1b,
  // S(a^2+b^2), S(ab))
  static constexpr int SMEM = IH * kIW * 8 + kTY * kRP * 16;
  static_assert(8 * kHO >= TX && 8 * kHO + WIN - 2 < kRP, "tile columns");
};

__device__ __forceinline__ float ld_plane(const SsimPlane& p, int x, int y)
{
  const int64_t o = (int64_t)(y >> p.shift) * p.stride + (x >> p.shift);
  if(p.sbytes == 4) return __ldg((const float*)p.ptr + o);
  return p.sbytes == 1 ? (float)__ldg((const uint8_t*)p.ptr + o) : (float)__ldg((const uint16_t*)p.ptr + o);
}

__device__ __forceinline__ int ld_int(const SsimPlane& p, int x, int y)
{
  const int64_t o = (int64_t)(y >> p.shift) * p.stride + (x >> p.shift);
  return p.sbytes == 1 ? (int)__ldg((const uint8_t*)p.ptr + o) : (int)__ldg((const uint16_t*)p.ptr + o);
}

// One plane's part of a staged tile, in registers: warp w takes staged rows w, w+8, ...,
// lanes the staged columns lane and lane+32. Rows and columns past the picture clamp (they
// only feed outputs outside the valid region). Integer samples convert exactly.
template <typename T, int SH, int IH>
__device__ __forceinline__ void load_rows(const SsimPlane& P, float (&v)[(IH + 7) / 8][2], int xs, int ys, int W, int H)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const T* base = reinterpret_cast<const T*>(P.ptr);
  const int gx0 = min(xs + lane, W - 1) >> SH, gx1 = min(xs + 32 + lane, W - 1) >> SH;
  #pragma unroll
  for(int k = 0; k < (IH + 7) / 8; k++)
  {
    const int i = min(warp + 8 * k, IH - 1);
    const T* row = base + (int64_t)(min(ys + i, H - 1) >> SH) * P.stride;
    v[k][0] = (float)__ldg(row + gx0);
    v[k][1] = (float)__ldg(row + gx1);
  }
}

template <int IH>
__device__ __forceinline__ void load_plane(const SsimPlane& P, float (&v)[(IH + 7) / 8][2], int xs, int ys, int W, int H)
{
  if(P.sbytes == 4)      load_rows<float, 0, IH>(P, v, xs, ys, W, H);
  else if(P.sbytes == 1) { if(P.shift) load_rows<uint8_t, 1, IH>(P, v, xs, ys, W, H); else load_rows<uint8_t, 0, IH>(P, v, xs, ys, W, H); }
  else                   { if(P.shift) load_rows<uint16_t, 1, IH>(P, v, xs, ys, W, H); else load_rows<uint16_t, 0, IH>(P, v, xs, ys, W, H); }
}

// Where tile `tile` is: its job (found by a forward scan from jb) and its origin.
struct TilePos { int jb, tx, x0, y0; };
template <int TX>
__device__ __forceinline__ TilePos locate(const SsimJob* __restrict__ jobs, int njobs, int jb, int tile)
{
  while(jb + 1 < njobs && jobs[jb + 1].tile_base <= tile) jb++;
  const int local = tile - jobs[jb].tile_base, tiles_x = jobs[jb].tiles_x;
  const int ty = local / tiles_x, tx = local - ty * tiles_x;
  TilePos t; t.jb = jb; t.tx = tx; t.x0 = 5 + tx * TX; t.y0 = 5 + ty * kTY;
  return t;
}

__device__ __forceinline__ float2 lo2(const float4& v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(const float4& v) { return make_float2(v.z, v.w); }

template <int WIN>
__global__ void __launch_bounds__(kThreads, 3) k_ssim(const SsimJob* __restrict__ jobs, int njobs, int ntiles)
{
  using G = SGeo<WIN>;
  extern __shared__ __align__(16) float smem[];
  __shared__ float s_kcc;  // (1 - W0) tc^2 W0 of the current tile, formed in FP64 by one thread
  float2* s_in = reinterpret_cast<float2*>(smem);                    // [IH][64]
  float4* s_v = reinterpret_cast<float4*>(smem + 2 * G::IH * kIW);   // [32][kRP]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  // window factor pairs (g, g), kept in registers for the whole kernel
  float2 gk[WIN];
  #pragma unroll
  for(int k = 0; k < WIN; k++)
  {
    gk[k] = c_g2[k];
    asm volatile("" : "+f"(gk[k].x), "+f"(gk[k].y));
  }
  const int wi = WIN == 11 ? 1 : 0;

  // a contiguous range of tiles per block: its first job by binary search, then at most one step
  // of the job walk per tile (a range strided by the grid crossed several small pyramid-level
  // jobs per tile, each a dependent load)
  const int t_begin = (int)((int64_t)ntiles * blockIdx.x / gridDim.x);
  const int t_end = (int)((int64_t)ntiles * (blockIdx.x + 1) / gridDim.x);
  int jb = 0;
  {
    int lo = 0, hi = njobs - 1;
    while(lo < hi)
    {
      const int mid = (lo + hi + 1) >> 1;
      if(jobs[mid].tile_base <= t_begin) lo = mid; else hi = mid - 1;
    }
    jb = lo;
  }
  for(int tile = t_begin; tile < t_end; tile++)
  {
    const TilePos cur = locate<G::TX>(jobs, njobs, jb, tile);
    jb = cur.jb;
    const SsimJob& J = jobs[jb];
    const int tx = cur.tx, x0 = cur.x0, y0 = cur.y0;
    const int x1 = min(x0 + G::TX, J.W - 5), y1 = min(y0 + kTY, J.H - 5);

    // staging: centring offset c = the tile-centre sample of plane b, loaded with the tile
    float va[G::RPW][2], vb[G::RPW][2];
    const float tc = ld_plane(J.b, min((x0 + x1) >> 1, J.W - 1), min((y0 + y1) >> 1, J.H - 1));
    load_plane<G::IH>(J.a, va, x0 - 5, y0 - 5, J.W, J.H);
    load_plane<G::IH>(J.b, vb, x0 - 5, y0 - 5, J.W, J.H);
    if(tid == 0) s_kcc = (float)(c_omd[wi] * (double)tc * (double)tc * c_w0d[wi]);  // one FP64 product per tile
    #pragma unroll
    for(int k = 0; k < G::RPW; k++)
    {
      const int i = warp + 8 * k;
      if(i < G::IH)
      {
        s_in[i * kIW + lane] = make_float2((float)(va[k][0] - tc), (float)(vb[k][0] - tc));
        s_in[i * kIW + lane + 32] = make_float2((float)(va[k][1] - tc), (float)(vb[k][1] - tc));
      }
    }
    __syncthreads();

    // vertical pass: column q, output rows 8rg .. 8rg+7; staged row 8rg+i feeds output row
    // 8rg+o with weight g[i-o]; (S1a, S1b) and (S(a^2+b^2), S(ab)) travel as float2 pairs
    {
      const int q = tid & (kIW - 1), rg = tid >> 6;
      const float2* src = s_in + 8 * rg * kIW + q;
      float2 s1[8], sq[8];
      #pragma unroll
      for(int o = 0; o < 8; o++) { s1[o] = make_float2(0.f, 0.f); sq[o] = make_float2(0.f, 0.f); }
      #pragma unroll
      for(int i = 0; i < 7 + WIN; i++)
      {
        const float2 v = src[i * kIW];
        const float2 p = __fmul2_rn(v, v);
        const float2 qq = make_float2(p.x + p.y, v.x * v.y);
        #pragma unroll
        for(int o = 0; o < 8; o++)
        {
          const int k = i - o;
          if(k < 0 || k >= WIN) continue;
          s1[o] = __ffma2_rn(gk[k], v, s1[o]);
          sq[o] = __ffma2_rn(gk[k], qq, sq[o]);
        }
      }
      #pragma unroll
      for(int o = 0; o < 8; o++) s_v[(8 * rg + o) * kRP + q] = make_float4(s1[o].x, s1[o].y, sq[o].x, sq[o].y);
    }
    __syncthreads();

    // horizontal pass and the index: thread = output row r x outputs 7g .. 7g+6 (g = 0..7); lanes
    // 4g + i of warp w hold row 4w + i, so a row's eight groups reduce by shuffles. The float4
    // pitch kRP = 2 mod 8 keeps the reads of a quarter-warp on distinct bank groups.
    {
      const int g = lane >> 2, o = 4 * warp + (lane & 3), j0 = kHO * g;
      const float4* src = s_v + o * kRP + j0;
      float2 m1[kHO], m2[kHO];
      #pragma unroll
      for(int jj = 0; jj < kHO; jj++) { m1[jj] = make_float2(0.f, 0.f); m2[jj] = make_float2(0.f, 0.f); }
      #pragma unroll
      for(int t = 0; t < kHO - 1 + WIN; t++)
      {
        const float4 val = src[t];
        #pragma unroll
        for(int jj = 0; jj < kHO; jj++)
        {
          const int k = t - jj;
          if(k < 0 || k >= WIN) continue;
          m1[jj] = __ffma2_rn(gk[k], lo2(val), m1[jj]);
          m2[jj] = __ffma2_rn(gk[k], hi2(val), m2[jj]);
        }
      }
      const float cf = tc;
      const float k_cc = s_kcc;
      const float cw0 = cf * c_w0[wi], om2c = c_om[wi] * 2.0f * cf, omc = c_om[wi] * cf;
      const float vq0 = 2.0f * k_cc + J.c2, cv0 = k_cc, C1 = J.c1, C2 = J.c2;
      const bool calc_l = J.calc_l != 0;
      const bool row_ok = y0 + o < y1;
      float rs = 0.0f;
      #pragma unroll
      for(int jj = 0; jj < kHO; jj++)
      {
        const float S1a = m1[jj].x, S1b = m1[jj].y, Sq = m2[jj].x, Sx = m2[jj].y;
        const float sab = S1a + S1b;
        // den: var_a + var_b + C2; num: 2 cov + C2
        const float den_cs = fmaf(-S1b, S1b, fmaf(-S1a, S1a, Sq)) + fmaf(om2c, sab, vq0);
        const float cov = fmaf(-S1a, S1b, Sx) + fmaf(omc, sab, cv0);
        float num = fmaf(2.0f, cov, C2), den = den_cs;
        if(calc_l)
        { // L * CS = (nL nCS) / (dL dCS): one division (xStructSim.cpp:50-51)
          const float mua = S1a + cw0, mub = S1b + cw0;
          num *= fmaf(2.0f * mua, mub, C1);
          den *= fmaf(mua, mua, fmaf(mub, mub, C1));
        }
        rs += (row_ok && x0 + j0 + jj < x1) ? __fdividef(num, den) : 0.0f;
      }
      // fixed-order sum over the row's eight groups
      rs += __shfl_xor_sync(0xffffffffu, rs, 4);
      rs += __shfl_xor_sync(0xffffffffu, rs, 8);
      rs += __shfl_xor_sync(0xffffffffu, rs, 16);
      if(g == 0 && row_ok) J.partial[(int64_t)(y0 + o - 5) * J.tiles_x + tx] = rs;
    }
    __syncthreads();
    // the next tile's staging overwrites s_in and s_kcc after the barrier above; s_v is
    // rewritten after one more
  }
}

// ---- the full-resolution family of a component in one pass -----------------------------------
// Picture 0, picture 1 and the two shift-compensated pictures share their window sums: ten
// moment streams (S1 of the four planes; S(a^2+b^2) and S(ab) of the three pairs (P0,P1),
// (P0,SCP1), (P1,SCP0)) give SSIM, CS, IV-SSIM T2R and R2T, against sixteen for four separate
// pair evaluations.
//
// One block of 16 warps per SM walks its tiles (32 output rows x TX columns) as a two-stage
// pipeline with specialised warps: warps 0-7 form the vertical window sums of tile k (thread =
// staged column x 8 output rows, so each staged sample is converted and its products formed for
// eight outputs at once) into one of two vertical-sum buffers while warps 8-15 run the horizontal
// pass, the four indices and the row sums of tile k-1 from the other buffer (thread = output row
// x 7 consecutive outputs; the eight threads of a row reduce their sums by shuffles). One block
// barrier per tile separates the two; both halves carry about the same FP32 work.
//
// Staging: each tile needs one box per plane (the tile's rows and columns plus the window halo,
// its left edge rounded down to 16 bytes; half-resolution boxes for 4:2:0 chroma, which the
// vertical pass reads at (x >> 1, y >> 1)). Boxes are raw samples in two shared-memory stages:
// thread 0 issues the four bulk-tensor loads of tile k+2 into the stage tile k has just left
// (mbarrier per stage, every wait bounded). Planes that a tensor map cannot describe (unaligned
// base or pitch) are staged by the vertical warps with plain loads into the same box layout,
// coordinates clamped at the picture edges; the bulk loads read zeros there instead. Either way
// those samples feed only outputs outside the valid region. The vertical pass converts samples to
// FP32 as it reads them: 2^23 + v is formed by its bit pattern and (2^23 + tc) subtracted,
// exactly, which centres the tile on tc, the tile-centre sample of picture 1.
constexpr int kQTY = 32, kQPairs = 5;
constexpr int kQVR = 8;                    // output rows per vertical thread
constexpr int kQHO = 7;                    // outputs per horizontal thread (8 per row x 7 >= TX)
constexpr int kQVT = 64 * (kQTY / kQVR);   // vertical threads: 64 staged columns x 4 row groups
constexpr int kQHT = 8 * kQTY;             // horizontal threads: 32 rows x 8 groups
constexpr int kQThreads = kQVT + kQHT;
// float2 pitch of a vertical-sum row: a horizontal warp reads 4 rows x 8 groups 7 columns apart,
// lane = 4 group + row, so each half-warp reads 4 rows x 4 groups; with a pitch of 4 (mod 16)
// float2, row * 4 + group * 7 (mod 16) is different for all 16 lanes: no bank conflicts
constexpr int kQRP = 68;
constexpr uint32_t kQuadPolls = 1u << 22;
template <int WIN> struct QGeo {
  static constexpr int TX = kIW - WIN + 1;
  static constexpr int IH = kQTY + WIN - 1;                      // staged rows
  static constexpr int BH1 = (IH + 1) / 2 + 1;                   // box rows of a half-resolution plane
  static constexpr int SLOT = ((64 + 8) * 2 * IH + 127) / 128 * 128;  // largest box: uint16, full resolution
  static constexpr int STAGE = 4 * SLOT;
  static constexpr int SVB = kQPairs * kQTY * kQRP * 8;          // one vertical-sum buffer
  static constexpr int META = 32;
  static constexpr int SMEM = 2 * STAGE + 2 * SVB + 2 * META + 32;    // + 3 mbarriers
  static_assert(8 * kQHO >= TX && 7 * kQHO + kQHO - 1 + WIN - 1 < kQRP, "horizontal groups");
  static_assert(kQTY % kQVR == 0 && kQVT % 32 == 0 && kQHT % 32 == 0 && (kQHT / 32) * 4 == kQTY, "thread roles");
  static_assert(kQRP % 16 == 4, "conflict-free horizontal reads");
  static_assert(SMEM <= 227 * 1024, "shared memory");
};
// what the horizontal warps need of the tile the vertical warps staged an iteration earlier
struct QMeta { int jb, tx, x0, y0; float tc, kcc; int pad[2]; };
}  // namespace
int quad_box_h(int window, int shift) { const int ih = kQTY + (window == QMIV_SSIM_GAUSS11 ? 11 : 10) - 1; return shift ? (ih + 1) / 2 + 1 : ih; }
namespace {

__device__ __forceinline__ void fence_proxy_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void bar_vertical() { asm volatile("bar.sync 1, %0;" :: "n"(kQVT) : "memory"); }

// Box origin of plane `pl` for the tile whose staged region starts at (xr, yr) = (x0-5, y0-5).
__device__ __forceinline__ void quad_box_origin(const SsimPlane& pl, int xr, int yr, int& xs, int& ys)
{
  const int xa = 16 / pl.sbytes;
  xs = (pl.shift ? xr >> 1 : xr) & ~(xa - 1);
  ys = pl.shift ? yr >> 1 : yr;
}

__device__ __forceinline__ float ssim_index(float S1a, float S1b, float Sq, float Sx, float om2c, float omc,
                                            float k_cc, float cw0, float C1, float C2)
{
  const float sab = S1a + S1b;
  const float den_cs = fmaf(-S1b, S1b, fmaf(-S1a, S1a, Sq)) + fmaf(om2c, sab, fmaf(2.0f, k_cc, C2));
  const float cov = fmaf(-S1a, S1b, Sx) + fmaf(omc, sab, k_cc);
  const float mua = S1a + cw0, mub = S1b + cw0;
  // L * CS = (nL nCS) / (dL dCS): one division (xStructSim.cpp:50-51)
  const float num = fmaf(2.0f, cov, C2) * fmaf(2.0f * mua, mub, C1);
  const float den = den_cs * fmaf(mua, mua, fmaf(mub, mub, C1));
  return __fdividef(num, den);
}

// One plane's column pointer for the vertical pass: even/odd staged-row bases (they differ for a
// half-resolution plane whose first staged row is odd) and the row pitch in samples. row0: the
// thread's first staged row (even).
template <typename T, int SH>
struct QCol {
  const T* e;
  const T* o;
  __device__ __forceinline__ QCol(const unsigned char* box, int bw, int xr, int yr, int xs, int q, int row0)
  {
    const T* b = reinterpret_cast<const T*>(box);
    if(SH)
    {
      const int par = yr & 1, c = ((xr + q) >> 1) - xs;
      e = b + (row0 >> 1) * bw + c;
      o = e + par * bw;
    }
    else
    {
      e = b + row0 * bw + (xr - xs) + q;
      o = e;
    }
  }
  // staged row row0 + i, compile-time i
  template <int BW>
  __device__ __forceinline__ unsigned at(int i) const
  {
    if(SH) return (i & 1) ? (unsigned)o[((i - 1) >> 1) * BW] : (unsigned)e[(i >> 1) * BW];
    return (unsigned)e[i * BW];
  }
};

// Vertical pass of a tile: thread = staged column q x output rows kQVR*rg .. kQVR*rg+kQVR-1; five
// float2 stream pairs per output row into the vertical-sum buffer sv ([5][kQTY][kQRP]).
template <int WIN, typename T0, int SH0>
__device__ __forceinline__ void quad_vpass(const unsigned char* stg, const SsimQuadJob& J, int xr, int yr, float tc,
                                           const float2 (&gk)[WIN], float2* sv, int q, int rg)
{
  using G = QGeo<WIN>;
  constexpr int BW0 = quad_box_w((int)sizeof(T0), SH0), BWS = quad_box_w(2, 0);
  const int row0 = kQVR * rg;
  int xs, ys;
  quad_box_origin(J.p0, xr, yr, xs, ys);
  const QCol<T0, SH0> c0(stg, BW0, xr, yr, xs, q, row0);
  const QCol<T0, SH0> c1(stg + G::SLOT, BW0, xr, yr, xs, q, row0);
  quad_box_origin(J.scp1, xr, yr, xs, ys);
  const QCol<uint16_t, 0> c2(stg + 2 * G::SLOT, BWS, xr, yr, xs, q, row0);
  const QCol<uint16_t, 0> c3(stg + 3 * G::SLOT, BWS, xr, yr, xs, q, row0);
  const float2 mk = make_float2(-(8388608.0f + tc), -(8388608.0f + tc));
  float2 acc[kQVR][kQPairs];
  #pragma unroll
  for(int o = 0; o < kQVR; o++)
    #pragma unroll
    for(int m = 0; m < kQPairs; m++) acc[o][m] = make_float2(0.f, 0.f);
  #pragma unroll
  for(int i = 0; i < kQVR + WIN - 1; i++)
  {
    const float2 v01 = __fadd2_rn(make_float2(__uint_as_float(0x4B000000u | c0.template at<BW0>(i)),
                                              __uint_as_float(0x4B000000u | c1.template at<BW0>(i))), mk);
    const float2 v23 = __fadd2_rn(make_float2(__uint_as_float(0x4B000000u | c2.template at<BWS>(i)),
                                              __uint_as_float(0x4B000000u | c3.template at<BWS>(i))), mk);
    const float2 sq01 = __fmul2_rn(v01, v01);
    const float2 sq23 = __fmul2_rn(v23, v23);
    float2 st[kQPairs];
    st[0] = v01;
    st[1] = v23;
    st[2] = make_float2(sq01.x + sq01.y, v01.x * v01.y);   // (P0, P1)
    st[3] = make_float2(sq01.x + sq23.x, v01.x * v23.x);   // (P0, SCP1)
    st[4] = make_float2(sq01.y + sq23.y, v01.y * v23.y);   // (P1, SCP0)
    #pragma unroll
    for(int o = 0; o < kQVR; o++)
    {
      const int k = i - o;
      if(k < 0 || k >= WIN) continue;
      #pragma unroll
      for(int m = 0; m < kQPairs; m++) acc[o][m] = __ffma2_rn(gk[k], st[m], acc[o][m]);
    }
  }
  #pragma unroll
  for(int o = 0; o < kQVR; o++)
    #pragma unroll
    for(int m = 0; m < kQPairs; m++) sv[(m * kQTY + row0 + o) * kQRP + q] = acc[o][m];
}

// The boxes of a tile whose planes have no tensor maps, by plain loads with clamped coordinates
// (vertical threads tv = 0 .. kQVT-1).
template <int WIN>
__device__ __forceinline__ void quad_fill(unsigned char* stg, const SsimQuadJob& J, int xr, int yr, int tv)
{
  using G = QGeo<WIN>;
  #pragma unroll
  for(int p = 0; p < 4; p++)
  {
    const SsimPlane& P = p == 0 ? J.p0 : (p == 1 ? J.p1 : (p == 2 ? J.scp1 : J.scp0));
    int xs, ys;
    quad_box_origin(P, xr, yr, xs, ys);
    const int bw = quad_box_w(P.sbytes, P.shift), bh = P.shift ? G::BH1 : G::IH;
    const int wp = P.shift ? J.W >> 1 : J.W, hp = P.shift ? J.H >> 1 : J.H;
    unsigned char* box = stg + p * G::SLOT;
    for(int idx = tv; idx < bw * bh; idx += kQVT)
    {
      const int r = idx / bw, c = idx - r * bw;
      const int64_t o = (int64_t)min(ys + r, hp - 1) * P.stride + min(xs + c, wp - 1);
      if(P.sbytes == 1) box[idx] = __ldg((const uint8_t*)P.ptr + o);
      else reinterpret_cast<uint16_t*>(box)[idx] = __ldg((const uint16_t*)P.ptr + o);
    }
  }
}

// Horizontal pass, indices and row sums of a tile whose vertical sums are in sv: thread = output
// row r x outputs 7g .. 7g+6 (g = 0..7); lanes 4g + i (g = 0..7) of a warp hold its row i.
template <int WIN>
__device__ __forceinline__ void quad_hpass(const SsimQuadJob& J, const QMeta& M, const float2* sv,
                                           const float2 (&gk)[WIN], int r, int g)
{
  using G = QGeo<WIN>;
  const int j0 = kQHO * g;
  const float2* src = sv + r * kQRP + j0;
  float2 m[kQHO][kQPairs];
  #pragma unroll
  for(int jj = 0; jj < kQHO; jj++)
    #pragma unroll
    for(int s2 = 0; s2 < kQPairs; s2++) m[jj][s2] = make_float2(0.f, 0.f);
  #pragma unroll
  for(int t = 0; t < kQHO + WIN - 1; t++)
  {
    float2 val[kQPairs];
    #pragma unroll
    for(int s2 = 0; s2 < kQPairs; s2++) val[s2] = src[s2 * kQTY * kQRP + t];
    #pragma unroll
    for(int jj = 0; jj < kQHO; jj++)
    {
      const int k = t - jj;
      if(k < 0 || k >= WIN) continue;
      #pragma unroll
      for(int s2 = 0; s2 < kQPairs; s2++) m[jj][s2] = __ffma2_rn(gk[k], val[s2], m[jj][s2]);
    }
  }
  const int wi = WIN == 11 ? 1 : 0;
  const float cf = M.tc, k_cc = M.kcc;
  const float cw0 = cf * c_w0[wi], om2c = c_om[wi] * 2.0f * cf, omc = c_om[wi] * cf;
  const float C1 = J.c1, C2 = J.c2, vq0 = fmaf(2.0f, k_cc, C2);
  const int y = M.y0 + r;
  const int x1 = min(M.x0 + G::TX, J.W - 5), y1 = min(M.y0 + kQTY, J.H - 5);
  const bool row_ok = y < y1;
  const uint32_t outs = J.outs;
  float rs[4] = { 0.f, 0.f, 0.f, 0.f };
  #pragma unroll
  for(int jj = 0; jj < kQHO; jj++)
  {
    if(!(row_ok && M.x0 + j0 + jj < x1)) continue;
    const float S0 = m[jj][0].x, S1 = m[jj][0].y, Ss1 = m[jj][1].x, Ss0 = m[jj][1].y;
    if(outs & 3u)
    { // SSIM(P0, P1) and CS(P0, P1) from one reciprocal
      const float sab = S0 + S1;
      const float den_cs = fmaf(-S1, S1, fmaf(-S0, S0, m[jj][2].x)) + fmaf(om2c, sab, vq0);
      const float cov = fmaf(-S0, S1, m[jj][2].y) + fmaf(omc, sab, k_cc);
      const float num_cs = fmaf(2.0f, cov, C2);
      const float mua = S0 + cw0, mub = S1 + cw0;
      const float nl = fmaf(2.0f * mua, mub, C1), dl = fmaf(mua, mua, fmaf(mub, mub, C1));
      const float rc = __fdividef(1.0f, den_cs * dl);
      rs[0] += num_cs * nl * rc;
      rs[1] += num_cs * dl * rc;
    }
    if(outs & 4u) rs[2] += ssim_index(S0, Ss1, m[jj][3].x, m[jj][3].y, om2c, omc, k_cc, cw0, C1, C2);
    if(outs & 8u) rs[3] += ssim_index(S1, Ss0, m[jj][4].x, m[jj][4].y, om2c, omc, k_cc, cw0, C1, C2);
  }
  // fixed-order sum over the row's eight groups, then one store per output kind
  #pragma unroll
  for(int k = 0; k < 4; k++)
  {
    float v = rs[k];
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 8);
    v += __shfl_xor_sync(0xffffffffu, v, 16);
    rs[k] = v;
  }
  if(g == 0 && row_ok)
  {
    #pragma unroll
    for(int k = 0; k < 4; k++)
      if(outs & (1u << k)) J.partial[k][(int64_t)(y - 5) * J.tiles_x + M.tx] = rs[k];
  }
}

template <int WIN>
__global__ void __launch_bounds__(kQThreads, 1) k_ssim_quad(const SsimQuadJob* __restrict__ jobs, int njobs, int ntiles,
                                                             uint32_t first_wait_test_polls)
{
  using G = QGeo<WIN>;
  extern __shared__ __align__(128) unsigned char qsm[];
  float2* s_v = reinterpret_cast<float2*>(qsm + 2 * G::STAGE);                       // [2][5][kQTY][kQRP]
  QMeta* meta = reinterpret_cast<QMeta*>(qsm + 2 * G::STAGE + 2 * G::SVB);           // [2]
  uint64_t* bar = reinterpret_cast<uint64_t*>(qsm + 2 * G::STAGE + 2 * G::SVB + 2 * G::META);
  const int tid = threadIdx.x;
  const bool vert = tid < kQVT;
  // window factor pairs: left to the compiler (pinning them in registers took 20 of the 128 and
  // left the vertical pass no room to load ahead: 1.58 ms against 1.49 ms unpinned)
  float2 gk[WIN];
  #pragma unroll
  for(int k = 0; k < WIN; k++) gk[k] = c_g2[k];
  const int wi = WIN == 11 ? 1 : 0;
  if(tid == 0)
  {
    ptx::mbar_init(&bar[0], 1);
    ptx::mbar_init(&bar[1], 1);
    ptx::mbar_init(&bar[2], 1);  // no copy ever arrives on it: the target of the timeout test hook
    ptx::fence_mbar_init();
  }
  __syncthreads();

  // bulk loads of tile `t` (job jn) into stage `sg`: issued by thread 0 only
  auto issue = [&](int t, int jn, int sg) {
    const SsimQuadJob& N = jobs[jn];
    const int local = t - N.tile_base;
    const int ty = local / N.tiles_x, tx = local - ty * N.tiles_x;
    const int xr = tx * G::TX, yr = ty * kQTY;
    // pictures: sample size and resolution of p0 (p1 alike); shift-compensated pictures: uint16
    const int sb = N.p0.sbytes, sh = N.p0.shift;
    const uint32_t bytes = 2u * (uint32_t)(quad_box_w(sb, sh) * (sh ? G::BH1 : G::IH) * sb) +
                           2u * (uint32_t)(quad_box_w(2, 0) * G::IH * 2);
    fence_proxy_async_shared();
    ptx::mbar_arrive_expect_tx(&bar[sg], bytes);
    const unsigned char* tm = reinterpret_cast<const unsigned char*>(N.tmaps);
    int xs, ys;
    quad_box_origin(N.p0, xr, yr, xs, ys);
    ptx::tma_load_2d(qsm + sg * G::STAGE, tm, xs, ys, &bar[sg]);
    ptx::tma_load_2d(qsm + sg * G::STAGE + G::SLOT, tm + 128, xs, ys, &bar[sg]);
    quad_box_origin(N.scp1, xr, yr, xs, ys);
    ptx::tma_load_2d(qsm + sg * G::STAGE + 2 * G::SLOT, tm + 256, xs, ys, &bar[sg]);
    ptx::tma_load_2d(qsm + sg * G::STAGE + 3 * G::SLOT, tm + 384, xs, ys, &bar[sg]);
  };
  auto job_of = [&](int t, int jb) {
    while(jb + 1 < njobs && jobs[jb + 1].tile_base <= t) jb++;
    return jb;
  };

  // Every thread keeps the same bookkeeping: pend bit s = stage s has bulk loads in flight,
  // phase bit s = parity of stage s's next completion.
  uint32_t pend = 0, phase = 0;
  int jv = 0, jp = 0;  // forward-scan positions: the vertical pass's tile, the prefetched tile
  #pragma unroll
  for(int s = 0; s < 2; s++)
  {
    const int t = blockIdx.x + s * gridDim.x;
    if(t < ntiles)
    {
      jp = job_of(t, jp);
      if(jobs[jp].tmaps) { if(tid == 0) issue(t, jp, s); pend |= 1u << s; }
    }
  }
  for(int it = 0;; it++)
  {
    const int tv_tile = blockIdx.x + it * gridDim.x;   // tile of the vertical pass
    const bool do_v = tv_tile < ntiles, do_h = it >= 1 && tv_tile - (int)gridDim.x < ntiles;
    if(!do_v && !do_h) break;
    const int stg = it & 1;
    bool ok = true;
    if(vert)
    {
      if(do_v)
      {
        jv = job_of(tv_tile, jv);
        const SsimQuadJob& J = jobs[jv];
        const int local = tv_tile - J.tile_base;
        const int ty = local / J.tiles_x, tx = local - ty * J.tiles_x;
        const int x0 = 5 + tx * G::TX, y0 = 5 + ty * kQTY;
        const int x1 = min(x0 + G::TX, J.W - 5), y1 = min(y0 + kQTY, J.H - 5);
        const int xr = x0 - 5, yr = y0 - 5;
        unsigned char* stage = qsm + stg * G::STAGE;
        if(pend & (1u << stg))
          ok = (it == 0 && first_wait_test_polls) ? ptx::mbar_wait_bounded(&bar[2], 0u, first_wait_test_polls)
                                                  : ptx::mbar_wait_bounded(&bar[stg], (phase >> stg) & 1u, kQuadPolls);
        else { quad_fill<WIN>(stage, J, xr, yr, tid); bar_vertical(); }
        if(ok)
        {
          // centring offset: the tile-centre sample of picture 1, from its box
          const int xc = min((x0 + x1) >> 1, J.W - 1), yc = min((y0 + y1) >> 1, J.H - 1);
          int xs, ys;
          quad_box_origin(J.p1, xr, yr, xs, ys);
          const int bw = quad_box_w(J.p1.sbytes, J.p1.shift);
          const int cx = (J.p1.shift ? xc >> 1 : xc) - xs, cy = (J.p1.shift ? yc >> 1 : yc) - ys;
          const unsigned char* box = stage + G::SLOT;
          const float tc = J.p1.sbytes == 1 ? (float)box[cy * bw + cx] : (float)reinterpret_cast<const uint16_t*>(box)[cy * bw + cx];
          if(tid == 0)
          {
            QMeta mt;
            mt.jb = jv; mt.tx = tx; mt.x0 = x0; mt.y0 = y0; mt.tc = tc;
            mt.kcc = (float)(c_omd[wi] * (double)tc * (double)tc * c_w0d[wi]);  // one FP64 product per tile
            mt.pad[0] = mt.pad[1] = 0;
            meta[stg] = mt;
          }
          const int q = tid & 63, rg = tid >> 6;
          float2* sv = s_v + stg * (G::SVB / 8);
          if(J.p0.sbytes == 1)
          {
            if(J.p0.shift) quad_vpass<WIN, uint8_t, 1>(stage, J, xr, yr, tc, gk, sv, q, rg);
            else           quad_vpass<WIN, uint8_t, 0>(stage, J, xr, yr, tc, gk, sv, q, rg);
          }
          else
          {
            if(J.p0.shift) quad_vpass<WIN, uint16_t, 1>(stage, J, xr, yr, tc, gk, sv, q, rg);
            else           quad_vpass<WIN, uint16_t, 0>(stage, J, xr, yr, tc, gk, sv, q, rg);
          }
        }
      }
    }
    else if(do_h)
    { // the tile the vertical warps finished in the previous iteration
      const QMeta M = meta[stg ^ 1];
      const int th = tid - kQVT, lane = th & 31;
      quad_hpass<WIN>(jobs[M.jb], M, s_v + (stg ^ 1) * (G::SVB / 8), gk, 4 * (th >> 5) + (lane & 3), lane >> 2);
    }
    if(__syncthreads_or(!ok))
    { // a bulk load did not arrive: record it, let every load in flight land, and stop
      if(tid == 0)
      {
        if(jobs[jv].status) atomicExch(jobs[jv].status, (int)QMIV_DEVICE_TIMEOUT);
        for(int s = 0; s < 2; s++)
          if(pend & (1u << s)) ptx::mbar_wait_bounded(&bar[s], (phase >> s) & 1u, kQuadPolls);
      }
      __syncthreads();
      return;
    }
    if(do_v && (pend & (1u << stg))) { pend &= ~(1u << stg); phase ^= 1u << stg; }
    // the stage this iteration's vertical pass read is free: tile tv_tile + 2 grid goes there
    const int nt = tv_tile + 2 * (int)gridDim.x;
    if(nt < ntiles)
    {
      jp = job_of(nt, jp);
      if(jobs[jp].tmaps) { if(tid == 0) issue(nt, jp, stg); pend |= 1u << stg; }
    }
  }
}

// Picture sum of one SSIM job (xSSIM.cpp:106-111), in two passes. Row pass: a warp per row adds
// the row's per-tile sums as an FP32 pair (TwoSum), lane t taking tiles t, t + 32, ... in order,
// and the lanes' pairs are combined by a fixed butterfly of TwoSums (every lane ends with the
// same pair: TwoSum's error term is exact whatever the order of its operands); the pair replaces
// the row's first two tile sums (a one-tile row keeps its value). Job pass: the row values go to
// FP64 once, are combined with a compensated sum in a fixed order, and the picture sum is
// divided by W*H. FP32 pairs rather than FP64 adds per tile: GB300's FP64 rate made the per-tile
// adds the cost of this step on large pictures. The row pass spreads a job over several blocks:
// a block per job with a thread per row took 0.27 ms for an 8K frame's 21 jobs on 21 SMs.
__device__ __forceinline__ void fin_two_sum(float a, float b, float& s, float& e)
{
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

constexpr int kFinThreads = 256, kFinWarps = kFinThreads / 32;
__global__ void __launch_bounds__(kFinThreads) k_ssim_fin_rows(const SsimJob* __restrict__ jobs)
{
  const SsimJob& J = jobs[blockIdx.y];
  const int rows = max(0, J.H - 10), tx = J.tiles_x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for(int r = blockIdx.x * kFinWarps + w; r < rows; r += gridDim.x * kFinWarps)
  {
    float* pr = J.partial + (int64_t)r * tx;
    float hi = 0.0f, lo = 0.0f;
    for(int t = lane; t < tx; t += 32)
    {
      float e;
      fin_two_sum(hi, __ldcg(pr + t), hi, e);
      lo = __fadd_rn(lo, e);
    }
    #pragma unroll
    for(int off = 16; off; off >>= 1)
    {
      const float h2 = __shfl_xor_sync(0xffffffffu, hi, off), l2 = __shfl_xor_sync(0xffffffffu, lo, off);
      float e;
      fin_two_sum(hi, h2, hi, e);
      lo = __fadd_rn(__fadd_rn(lo, l2), e);
    }
    if(lane == 0 && tx >= 2) { pr[0] = hi; pr[1] = lo; }
  }
}

__global__ void __launch_bounds__(kFinThreads) k_ssim_fin_jobs(const SsimJob* __restrict__ jobs)
{
  __shared__ double scratch[2 * kFinWarps];
  const SsimJob& J = jobs[blockIdx.x];
  const int rows = max(0, J.H - 10), tx = J.tiles_x;
  Kbns k = { 0.0, 0.0 };
  for(int r = threadIdx.x; r < rows; r += kFinThreads)
  {
    const float* pr = J.partial + (int64_t)r * tx;
    // a row of no tiles (a plane at most 10 wide) contributes 0
    k = kbns_add(k, tx >= 2 ? __dadd_rn((double)__ldcg(pr), (double)__ldcg(pr + 1)) : (tx == 1 ? (double)__ldcg(pr) : 0.0));
  }
  const double tot = block_kbns(k, scratch);
  if(threadIdx.x == 0) *J.out = __ddiv_rn(tot, (double)((int64_t)J.W * J.H));
}

// DownsampleHV to a 16-bit plane: d(x,y) = (s(2x,2y)+s(2x+1,2y)+s(2x,2y+1)+s(2x+1,2y+1)+2)>>2
// Grid: x = 64-column groups, y = groups of kDownRows output rows, z = steps; a thread makes
// kDownRows / 4 outputs of one column, all loads issued before the stores.
constexpr int kDownRows = 16;
__global__ void __launch_bounds__(256) k_downsample(const PyrStep* __restrict__ steps, int nsteps)
{
  const PyrStep& S = steps[blockIdx.z];
  const int x = blockIdx.x * 64 + (threadIdx.x & 63);
  const int y0 = blockIdx.y * kDownRows + (threadIdx.x >> 6);
  if(x >= S.dw || y0 >= S.dh) return;
  constexpr int K = kDownRows / 4;
  int v[K];
  #pragma unroll
  for(int k = 0; k < K; k++)
  {
    const int sx = 2 * x, sy = 2 * min(y0 + 4 * k, S.dh - 1);
    v[k] = ld_int(S.src, sx, sy) + ld_int(S.src, sx + 1, sy) + ld_int(S.src, sx, sy + 1) + ld_int(S.src, sx + 1, sy + 1);
  }
  #pragma unroll
  for(int k = 0; k < K; k++)
  {
    const int y = y0 + 4 * k;
    if(y < S.dh) S.dst[(int64_t)y * S.dst_stride + x] = (uint16_t)((v[k] + 2) >> 2);
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

// ---- backward ---------------------------------------------------------------------------
// d SSIM / d a(q) and d SSIM / d b(q) for every sample q of two FP32 planes. SSIM is the mean
// over the valid region of s(p) = L(p) CS(p), built from the raw window moments
// mu_a = sum w a, E_aa = sum w a^2, E_bb, E_ab (var = E - mu^2, cov = E_ab - mu_a mu_b). With
//   B = ds/dE_aa = ds/dE_bb = -L CS / D2,  C = ds/dE_ab = 2 L / D2,
//   A_a = ds/dmu_a = CS (2 mu_b - 2 mu_a L) / D1 - 2 mu_a B - mu_b C  (and A_b symmetric),
// the chain rule gives d SSIM / d a(q) = (1/WH) sum_p w(q-p) [A_a(p) + 2 a(q) B(p) + b(q) C(p)],
// i.e. the coefficient maps filtered with the window and combined with the samples at q.
// Statistics are recomputed from the pictures (nothing is stored by the forward pass).
//
// A block walks one 32-column strip of a picture down a segment of its rows in steps of 32
// output rows. A window at p reaches the samples [p-5, p+K1] (K1 = WIN-6), so the outputs of a
// step need the maps of 32 + WIN - 1 position rows, of which WIN - 1 were made by the step above:
// each step stages only its 32 new sample rows, computes window moments and maps only for its
// 32 new position rows, and keeps from the step above the WIN - 1 last sample rows and the WIN - 1
// last rows of the transposed horizontal pass. (A first, output-less step primes a segment.)
// Samples are centred by the step's centre sample c; maps are formed as A'' = A + c (2B + C) so
// that they combine with centred samples, and the kept rows of the transposed pass, which are
// linear in the maps, move to the next step's c as A'' += (c' - c)(2B + C).
constexpr int kBwdT = 32;          // strip width and step height
constexpr int kBwdSegSteps = 16;   // steps per block: strips are cut into segments of 512 rows
template <int WIN> struct BGeo {
  static constexpr int K1 = WIN - 6;                 // a window reaches K1 samples right of / below its position
  static constexpr int PW = kBwdT + WIN - 1;         // position columns whose maps reach the strip
  static constexpr int SW = PW + WIN - 1;            // sample columns
  static constexpr int KR = WIN - 1;                 // rows kept from one step to the next
  static constexpr int SR = kBwdT + KR;              // sample rows (and transposed-pass rows) held
  // row pitches (float4) read down a column by consecutive lanes are odd: conflict-free
  static constexpr int VP = SW | 1, MP = PW | 1, FP = kBwdT + 1;
  static constexpr int S_SMP = SR * SW * 8;          // raw samples (a, b), float2
  static constexpr int S_K = KR * FP * 16;           // transposed horizontal sums kept from the step above
  static constexpr int S_V = kBwdT * VP * 16;        // vertical moments of the step's new position rows; once
                                                     // they are consumed, the new transposed sums (pitch FP)
  static constexpr int S_M = kBwdT * MP * 16;        // coefficient maps of the new position rows
  static constexpr int SMEM = S_SMP + S_K + S_V + S_M;
  static_assert(4 * SW <= 256 && 32 * ((PW + 5) / 6) <= 256 && KR <= kBwdT && FP <= VP, "one round of the block per pass");
};

// acc += g * v on a float4 as two packed FP32 multiply-adds
__device__ __forceinline__ void fma4(float2 g, const float4& v, float4& acc)
{
  const float2 lo = __ffma2_rn(g, make_float2(v.x, v.y), make_float2(acc.x, acc.y));
  const float2 hi = __ffma2_rn(g, make_float2(v.z, v.w), make_float2(acc.z, acc.w));
  acc = make_float4(lo.x, lo.y, hi.x, hi.y);
}

// Each pass is register-blocked: a thread filters 4 to 8 consecutive outputs along the pass
// direction from that many + WIN - 1 shared-memory reads.
template <int WIN>
__global__ void __launch_bounds__(256, 3) k_ssim_bwd(const SsimBwdJob* __restrict__ jobs, int njobs)
{
  using G = BGeo<WIN>;
  constexpr int PW = G::PW, SW = G::SW, KR = G::KR, SR = G::SR, VP = G::VP, MP = G::MP, FP = G::FP, K1 = G::K1;
  constexpr int MG = 6, NG = (PW + MG - 1) / MG;  // map pass: MG position columns per thread
  extern __shared__ __align__(16) float smem[];
  float2* s_s = reinterpret_cast<float2*>(smem);                                      // [SR][SW]
  // transposed horizontal sums [SR][FP]: the KR kept rows directly before the vertical-moment
  // buffer [32][VP], whose space the 32 new rows take once the moments are consumed
  float4* s_f = reinterpret_cast<float4*>(smem + G::S_SMP / 4);
  float4* s_v = reinterpret_cast<float4*>(smem + (G::S_SMP + G::S_K) / 4);
  float4* s_m = reinterpret_cast<float4*>(smem + (G::S_SMP + G::S_K + G::S_V) / 4);   // [32][MP]
  __shared__ float s_kcc;  // (1 - W0) c^2 W0 of the step, formed in FP64 by one thread
  float2 gk[WIN];
  #pragma unroll
  for(int k = 0; k < WIN; k++) gk[k] = c_g2[k];
  int jb = 0;
  { int lo = 0, hi = njobs - 1;
    while(lo < hi) { const int mid = (lo + hi + 1) >> 1; if(jobs[mid].tile_base <= (int)blockIdx.x) lo = mid; else hi = mid - 1; }
    jb = lo; }
  const SsimBwdJob& J = jobs[jb];
  const int local = blockIdx.x - J.tile_base;
  const int seg = local / J.tiles_x, strip = local - seg * J.tiles_x;
  const int W = J.W, H = J.H, tid = threadIdx.x;
  const int qx0 = strip * kBwdT, px0 = qx0 - K1, sx0 = px0 - 5;
  const int y_begin = seg * kBwdT * kBwdSegSteps, y_end = min(H, y_begin + kBwdT * kBwdSegSteps);
  const int nsteps = (y_end - y_begin + kBwdT - 1) / kBwdT;
  const float* pa = (const float*)J.a.ptr;
  const float* pb = (const float*)J.b.ptr;
  const int wi = WIN == 11 ? 1 : 0;
  const float w0 = c_w0[wi], om = c_om[wi];
  const float C1 = J.c1, C2 = J.c2;
  const float scale = (float)(*J.g / ((double)W * (double)H));
  float c_prev = 0.0f;

  for(int st = -1; st < nsteps; st++)
  {
    const int y = y_begin + kBwdT * st;   // output rows [y, y+32); sample row r is picture row y + r
    const bool prime = st < 0;            // the step above the segment: makes the kept rows only
    { // stage the new sample rows (all rows when priming), coordinates clamped; all loads first
      const int r_lo = prime ? 0 : KR;
      constexpr int NI = (SR * SW + 255) / 256;
      float va[NI], vb[NI];
      #pragma unroll
      for(int k = 0; k < NI; k++)
      {
        const int i = min(r_lo * SW + tid + 256 * k, SR * SW - 1);
        const int r = i / SW, q = i - r * SW;
        const int gx = min(max(sx0 + q, 0), W - 1), gy = min(max(y + r, 0), H - 1);
        va[k] = __ldg(pa + (int64_t)gy * J.a.stride + gx);
        vb[k] = __ldg(pb + (int64_t)gy * J.b.stride + gx);
      }
      #pragma unroll
      for(int k = 0; k < NI; k++)
      {
        const int i = r_lo * SW + tid + 256 * k;
        if(i < SR * SW) s_s[i] = make_float2(va[k], vb[k]);
      }
    }
    __syncthreads();
    // centring: the step's centre sample of b
    const float c = s_s[(kBwdT / 2) * SW + kBwdT / 2 + WIN - 1].y;
    if(tid == 0) s_kcc = (float)(c_omd[wi] * (double)c * (double)c * c_w0d[wi]);
    if(!prime)
    { // the kept rows of the transposed pass move from the previous step's centring to this one's
      const float d = c - c_prev;
      for(int i = tid; i < KR * kBwdT; i += 256)
      {
        float4& f = s_f[(i >> 5) * FP + (i & 31)];
        const float t = d * fmaf(2.0f, f.z, f.w);
        f.x += t;
        f.y += t;
      }
    }
    c_prev = c;
    // vertical moments of the new position rows j (position row y + 5 + j): thread = sample
    // column x 8 position rows
    for(int it = tid; it < 4 * SW; it += 256)
    {
      const int q = it % SW, g8 = it / SW;
      if(prime && 8 * g8 + 7 < kBwdT - KR) continue;
      float4 acc[8];
      #pragma unroll
      for(int o = 0; o < 8; o++) acc[o] = make_float4(0.f, 0.f, 0.f, 0.f);
      #pragma unroll
      for(int i = 0; i < 7 + WIN; i++)
      {
        const float2 ab = s_s[(8 * g8 + i) * SW + q];
        const float a = ab.x - c, b = ab.y - c;
        const float4 v = make_float4(a, b, fmaf(a, a, b * b), a * b);
        #pragma unroll
        for(int o = 0; o < 8; o++)
          if(i - o >= 0 && i - o < WIN) fma4(gk[i - o], v, acc[o]);
      }
      #pragma unroll
      for(int o = 0; o < 8; o++) s_v[(8 * g8 + o) * VP + q] = acc[o];
    }
    __syncthreads();
    // horizontal moments -> coefficient maps (zero outside the valid region): thread = position
    // row x 6 consecutive position columns (32 x 7 items: 7 of the block's 8 warps; groups of 8
    // columns left two warps idle at the next barrier)
    {
      const float k_cc = s_kcc;
      for(int it = tid; it < kBwdT * NG; it += 256)
      {
        const int r = it % kBwdT, c0 = min(MG * (it / kBwdT), PW - MG);
        if(prime && r < kBwdT - KR) continue;
        float4 acc[MG];
        #pragma unroll
        for(int o = 0; o < MG; o++) acc[o] = make_float4(0.f, 0.f, 0.f, 0.f);
        #pragma unroll
        for(int i = 0; i < MG - 1 + WIN; i++)
        {
          const float4 v = s_v[r * VP + c0 + i];
          #pragma unroll
          for(int o = 0; o < MG; o++)
            if(i - o >= 0 && i - o < WIN) fma4(gk[i - o], v, acc[o]);
        }
        const int py = y + 5 + r;
        const bool row_ok = py >= 5 && py < H - 5;
        #pragma unroll
        for(int o = 0; o < MG; o++)
        {
          const int px = px0 + c0 + o;
          float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
          if(row_ok && px >= 5 && px < W - 5)
          {
            const float4 m = acc[o];
            const float S1a = m.x, S1b = m.y, sab = S1a + S1b;
            const float mua = S1a + c * w0, mub = S1b + c * w0;
            const float vsum = fmaf(-S1b, S1b, fmaf(-S1a, S1a, m.z)) + fmaf(om * 2.0f * c, sab, 2.0f * k_cc);
            const float cov = fmaf(-S1a, S1b, m.w) + fmaf(om * c, sab, k_cc);
            const float N1 = fmaf(2.0f * mua, mub, C1), D1 = fmaf(mua, mua, fmaf(mub, mub, C1));
            const float N2 = fmaf(2.0f, cov, C2), D2 = vsum + C2;
            const float r1 = __fdividef(1.0f, D1), r2 = __fdividef(1.0f, D2);  // D1 >= C1, D2 ~ >= C2: far from 0
            const float L = N1 * r1, CS = N2 * r2;
            const float B = -L * CS * r2, Cc = 2.0f * L * r2;
            const float Aa = CS * (2.0f * mub - 2.0f * mua * L) * r1 - 2.0f * mua * B - mub * Cc;
            const float Ab = CS * (2.0f * mua - 2.0f * mub * L) * r1 - 2.0f * mub * B - mua * Cc;
            const float cc = c * (2.0f * B + Cc);
            out = make_float4(Aa + cc, Ab + cc, B, Cc);
          }
          s_m[r * MP + c0 + o] = out;
        }
      }
    }
    __syncthreads();
    // transposed horizontal pass of the new rows: F[KR + r][qc] = sum_j g[j] M[r][qc + WIN-1-j];
    // thread = position row x 4 consecutive output columns (all 256 threads)
    {
      const int r = tid % kBwdT, q0 = 4 * (tid / kBwdT);
      if(!(prime && r < kBwdT - KR))
      {
        float4 acc[4];
        #pragma unroll
        for(int o = 0; o < 4; o++) acc[o] = make_float4(0.f, 0.f, 0.f, 0.f);
        #pragma unroll
        for(int i = 0; i < 3 + WIN; i++)
        {
          const float4 v = s_m[r * MP + q0 + i];
          #pragma unroll
          for(int o = 0; o < 4; o++)
            if(o + WIN - 1 - i >= 0 && o + WIN - 1 - i < WIN) fma4(gk[o + WIN - 1 - i], v, acc[o]);
        }
        #pragma unroll
        for(int o = 0; o < 4; o++) s_f[(KR + r) * FP + q0 + o] = acc[o];
      }
    }
    __syncthreads();
    if(!prime)
    { // transposed vertical pass and the combination: thread = output column x 4 consecutive
      // output rows (transposed-pass row f is position row y - K1 + f)
      const int cq = tid % kBwdT, q0 = 4 * (tid / kBwdT);
      const int x = qx0 + cq;
      float4 acc[4];
      #pragma unroll
      for(int o = 0; o < 4; o++) acc[o] = make_float4(0.f, 0.f, 0.f, 0.f);
      #pragma unroll
      for(int i = 0; i < 3 + WIN; i++)
      {
        const float4 v = s_f[(q0 + i) * FP + cq];
        #pragma unroll
        for(int o = 0; o < 4; o++)
          if(o + WIN - 1 - i >= 0 && o + WIN - 1 - i < WIN) fma4(gk[o + WIN - 1 - i], v, acc[o]);
      }
      if(x < W)
      {
        #pragma unroll
        for(int o = 0; o < 4; o++)
        {
          const int yy = y + q0 + o;
          if(yy >= y_end) break;
          const float4 f = acc[o];
          const float2 s = s_s[(q0 + o) * SW + cq + WIN - 1];  // the samples at q
          const float a = s.x - c, b = s.y - c;
          if(J.outx) J.outx[(int64_t)yy * W + x] = scale * (f.x + 2.0f * a * f.z + b * f.w);
          if(J.outy) J.outy[(int64_t)yy * W + x] = scale * (f.y + 2.0f * b * f.z + a * f.w);
        }
      }
    }
    __syncthreads();
    // keep the last WIN - 1 sample rows and transposed-pass rows for the next step
    for(int i = tid; i < KR * SW; i += 256) s_s[i] = s_s[kBwdT * SW + i];
    for(int i = tid; i < KR * kBwdT; i += 256) s_f[(i >> 5) * FP + (i & 31)] = s_f[(kBwdT + (i >> 5)) * FP + (i & 31)];
    __syncthreads();
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

cudaError_t launch_ssim_finalize(const SsimJob* d_jobs, const SsimJob* h_jobs, int n, cudaStream_t st)
{
  if(n <= 0) return cudaSuccess;
  int rows = 0;
  for(int i = 0; i < n; i++) rows = std::max(rows, h_jobs[i].H - 10);
  // row-pass blocks per job: about 16 rows per warp for the tallest job, at most 8
  const int per_job = std::min(8, std::max(1, (rows + 16 * kFinWarps - 1) / (16 * kFinWarps)));
  k_ssim_fin_rows<<<dim3(per_job, n), kFinThreads, 0, st>>>(d_jobs);
  k_ssim_fin_jobs<<<n, kFinThreads, 0, st>>>(d_jobs);
  return cudaGetLastError();
}

cudaError_t launch_ssim(const SsimJob* d_jobs, const SsimJob* h_jobs, int n, int window, cudaStream_t st)
{
  int tiles = 0;
  for(int i = 0; i < n; i++) tiles = h_jobs[i].tile_base + h_jobs[i].tiles_x * h_jobs[i].tiles_y;
  if(tiles > 0)
  {
    static std::atomic<int> resident[kStaticMaxDevices][2];  // blocks per SM x SMs, per device and window
    const int wi = window == QMIV_SSIM_GAUSS11 ? 1 : 0, dv = device_slot();
    int slots = resident[dv][wi].load(std::memory_order_acquire);
    if(!slots)
    {
      int sms = 0, r = 0;
      cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dv);
      if(e == cudaSuccess) e = cudaFuncSetAttribute(k_ssim<10>, cudaFuncAttributeMaxDynamicSharedMemorySize, SGeo<10>::SMEM);
      if(e == cudaSuccess) e = cudaFuncSetAttribute(k_ssim<11>, cudaFuncAttributeMaxDynamicSharedMemorySize, SGeo<11>::SMEM);
      if(e == cudaSuccess)
        e = wi ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_ssim<11>, kThreads, SGeo<11>::SMEM)
               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_ssim<10>, kThreads, SGeo<10>::SMEM);
      if(e != cudaSuccess) return e;
      slots = std::max(1, r) * std::max(1, sms);
      resident[dv][wi].store(slots, std::memory_order_release);
    }
    const int grid = std::min(tiles, slots);
    if(wi) k_ssim<11><<<grid, kThreads, SGeo<11>::SMEM, st>>>(d_jobs, n, tiles);
    else   k_ssim<10><<<grid, kThreads, SGeo<10>::SMEM, st>>>(d_jobs, n, tiles);
    cudaError_t e = cudaGetLastError();
    if(e != cudaSuccess) return e;
  }
  return launch_ssim_finalize(d_jobs, h_jobs, n, st);
}

int ssim_bwd_tiles(int dim) { return (dim + kBwdT - 1) / kBwdT; }
int ssim_bwd_segments(int H) { return (H + kBwdT * kBwdSegSteps - 1) / (kBwdT * kBwdSegSteps); }

cudaError_t launch_ssim_bwd(const SsimBwdJob* d_jobs, const SsimBwdJob* h_jobs, int n, int window, cudaStream_t st)
{
  int blocks = 0;
  for(int i = 0; i < n; i++) blocks = h_jobs[i].tile_base + h_jobs[i].tiles_x * h_jobs[i].tiles_y;
  if(blocks == 0) return cudaSuccess;
  static std::atomic<bool> attr[kStaticMaxDevices];
  const int dv = device_slot();
  if(!attr[dv].load(std::memory_order_acquire))
  {
    cudaError_t e = cudaFuncSetAttribute(k_ssim_bwd<10>, cudaFuncAttributeMaxDynamicSharedMemorySize, BGeo<10>::SMEM);
    if(e == cudaSuccess) e = cudaFuncSetAttribute(k_ssim_bwd<11>, cudaFuncAttributeMaxDynamicSharedMemorySize, BGeo<11>::SMEM);
    // three resident blocks of 67-70 KB need the unified L1 mostly as shared memory
    if(e == cudaSuccess) e = cudaFuncSetAttribute(k_ssim_bwd<10>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if(e == cudaSuccess) e = cudaFuncSetAttribute(k_ssim_bwd<11>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if(e != cudaSuccess) return e;
    attr[dv].store(true, std::memory_order_release);
  }
  if(window == QMIV_SSIM_GAUSS11) k_ssim_bwd<11><<<blocks, 256, BGeo<11>::SMEM, st>>>(d_jobs, n);
  else                            k_ssim_bwd<10><<<blocks, 256, BGeo<10>::SMEM, st>>>(d_jobs, n);
  return cudaGetLastError();
}

int ssim_quad_tiles_y(int H) { return H > 10 ? (H - 10 + kQTY - 1) / kQTY : 0; }

cudaError_t launch_ssim_quad(const SsimQuadJob* d_jobs, const SsimQuadJob* h_jobs, int n, int window,
                             uint32_t first_wait_test_polls, cudaStream_t st)
{
  int tiles = 0;
  for(int i = 0; i < n; i++) tiles = h_jobs[i].tile_base + h_jobs[i].tiles_x * h_jobs[i].tiles_y;
  if(tiles == 0) return cudaSuccess;
  static std::atomic<int> resident[kStaticMaxDevices][2];  // blocks per SM x SMs, per device and window
  const int wi = window == QMIV_SSIM_GAUSS11 ? 1 : 0, dv = device_slot();
  int slots = resident[dv][wi].load(std::memory_order_acquire);
  if(!slots)
  {
    int sms = 0, r = 0;
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dv);
    if(e == cudaSuccess) e = cudaFuncSetAttribute(k_ssim_quad<10>, cudaFuncAttributeMaxDynamicSharedMemorySize, QGeo<10>::SMEM);
    if(e == cudaSuccess) e = cudaFuncSetAttribute(k_ssim_quad<11>, cudaFuncAttributeMaxDynamicSharedMemorySize, QGeo<11>::SMEM);
    // one resident block of ~218 KB: nearly all of the unified L1 as shared memory
    if(e == cudaSuccess) e = cudaFuncSetAttribute(k_ssim_quad<10>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if(e == cudaSuccess) e = cudaFuncSetAttribute(k_ssim_quad<11>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if(e == cudaSuccess)
      e = wi ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_ssim_quad<11>, kQThreads, QGeo<11>::SMEM)
             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_ssim_quad<10>, kQThreads, QGeo<10>::SMEM);
    if(e != cudaSuccess) return e;
    slots = std::max(1, r) * std::max(1, sms);
    resident[dv][wi].store(slots, std::memory_order_release);
  }
  const int grid = std::min(tiles, slots);
  if(wi) k_ssim_quad<11><<<grid, kQThreads, QGeo<11>::SMEM, st>>>(d_jobs, n, tiles, first_wait_test_polls);
  else   k_ssim_quad<10><<<grid, kQThreads, QGeo<10>::SMEM, st>>>(d_jobs, n, tiles, first_wait_test_polls);
  return cudaGetLastError();
}

cudaError_t launch_downsample(const PyrStep* d_steps, const PyrStep* h_steps, int n, cudaStream_t st)
{
  int maxw = 0, maxh = 0;
  for(int i = 0; i < n; i++) { maxw = std::max(maxw, h_steps[i].dw); maxh = std::max(maxh, h_steps[i].dh); }
  if(n == 0 || maxw == 0 || maxh == 0) return cudaSuccess;
  dim3 grid((maxw + 63) / 64, (maxh + kDownRows - 1) / kDownRows, n);
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
