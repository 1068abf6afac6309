// Corresponding-pixel-shift (CPS) kernels: for every pixel of each picture, the first
// strict minimum over the (2B+1)^2 window of the other picture of
//     E = w0*(tY-rY)^2 + w1*(tCb-rCb)^2 + w2*(tCr-rCr)^2,  t = own pixel + GCD,
// scanned row-major (libs/pmbb-ivqm/src/xCorrespPixelShift.cpp:48-85,
// xCorrespPixelShiftSSE.cpp:40-70), then per-row per-component squared errors at the
// argmin (xCorrespPixelShift.cpp:20-46) and, on request, the shift-compensated pictures
// (xShftCompPic.cpp:69-96). One kernel does both directions (R2T: pixels of picture 0
// searched in picture 1 with +GCD, which also yields SCP1; T2R: picture 1 in picture 0
// with -GCD, which yields SCP0), so one pass serves IV-PSNR and IV-SSIM. The last block
// of each job turns the exact per-row sums into IV-PSNR (xIVPSNR.cpp:18-56,100-133).
//
// Fast path (4:2:0 inputs): integer-pipe bound. Tie-breaking is made order-free by
// minimising the packed key  M*E + k  (k = row-major window index, M > k) with a single
// unsigned min. The luma term is formed as (s*tY - s*rY)^2 with s^2 = M*w0, so one
// multiply-add per candidate covers it; the chroma term of a 4:2:0 picture depends only on
// the chroma sample a candidate falls on, and the four luma pixels of a 2x2 quad share
// their chroma and their (chroma-resolution) window, so each chroma cost is computed once
// per quad and reused by every candidate that falls on that chroma sample.
// Borders clamp coordinates, which equals the reference's edge-replicated margin of
// roundup4(B) >= B pixels (apps/QMIV/src/xAppQMIV.cpp:330, xPixelOpsSTD.cpp:210).
#include <climits>

#include "qmiv_cps_common.cuh"

namespace qmiv {

namespace {


constexpr int kChunk = 64; // columns per chunk: 32 lanes x 2 columns

template <int SR, int RPT, int NWG>
struct Geo {
  static constexpr int N    = (2 * SR + 1) * (2 * SR + 1);
  static constexpr int R    = RPT * NWG;                       // strip rows
  static constexpr int TW   = kChunk + 2 * SR;                 // luma tile width
  static constexpr int TH   = R + 2 * SR;                      // luma tile height
  static constexpr int CS   = ceil2(SR);                       // chroma halo before the tile
  static constexpr int CTW  = fdiv2(kChunk - 1 + SR) + CS + 1; // chroma tile width
  static constexpr int CTH  = fdiv2(R - 1 + SR) + CS + 1;      // chroma tile height
  static constexpr int NC   = fdiv2(1 + SR) + CS + 1;          // chroma columns a quad's window spans
  static constexpr int NQ   = RPT / 2;                         // quads per thread column
  static constexpr int NT   = 2 * NWG * 32;                    // threads
};


// ------------------------------------------------------------------------------------
// Fast 4:2:0 kernel
// ------------------------------------------------------------------------------------
template <int SR, int RPT, int NWG, typename KeyT>
__global__ void __launch_bounds__(Geo<SR, RPT, NWG>::NT)
k_cps420(const DevJob* __restrict__ jobs, int njobs, Params p)
{
  using G = Geo<SR, RPT, NWG>;
  constexpr int W2 = 2 * SR + 1;
  __shared__ __align__(16) int s_lum[2][G::TH][G::TW];
  __shared__ __align__(16) int s_chr[2][2][G::CTH][G::CTW];
  __shared__ double scratch[2 * (G::NT / 32)];

  const int j = find_job<1>(jobs, njobs, blockIdx.x);
  const DevJob& J = jobs[j];
  const int local = blockIdx.x - J.cps_base;
  const int strip = local / J.cps_segs, seg = local % J.cps_segs;
  const int W = J.W, H = J.H, Wc = W >> 1, Hc = H >> 1;
  const int y0 = strip * G::R;
  const int nchunks = (W + kChunk - 1) / kChunk;
  const int ch0 = seg * J.cps_seg_chunks, ch1 = min(nchunks, ch0 + J.cps_seg_chunks);

  const int tid = threadIdx.x;
  const int dir = tid / (NWG * 32);          // 0: R2T (test = picture 0), 1: T2R (test = picture 1)
  const int g   = (tid >> 5) % NWG;          // row group
  const int l   = tid & 31;                  // column pair
  const int tp = dir, rp = dir ^ 1;
  const int gsgn = dir == 0 ? 1 : -1;
  const int gd0 = gsgn * J.sc->gcd[0], gd1 = gsgn * J.sc->gcd[1], gd2 = gsgn * J.sc->gcd[2];
  const int s = p.luma_scale;
  const KeyT Mw1 = (KeyT)p.key_m * (KeyT)p.w_search[1];
  const KeyT Mw2 = (KeyT)p.key_m * (KeyT)p.w_search[2];
  const int mx = (1 << J.bd) - 1;
  const int sb = J.sbytes;
  const int cyBase = (y0 >> 1) - G::CS;
  uint16_t* const* scp = dir == 0 ? J.scp1 : J.scp0;
  const bool want_scp = scp[0] != nullptr;
  int16_t* const cmap = J.cps_map[dir];

  unsigned int sse[RPT][3];
  #pragma unroll
  for(int i = 0; i < RPT; i++) { sse[i][0] = 0; sse[i][1] = 0; sse[i][2] = 0; }

  for(int ch = ch0; ch < ch1; ch++)
  {
    const int cx0 = ch * kChunk;
    const int cxBase = (cx0 >> 1) - G::CS;
    // ---- stage both pictures' tiles (clamped coordinates) ----
    __syncthreads();
    for(int idx = tid; idx < 2 * G::TH * G::TW; idx += G::NT)
    {
      const int pic = idx / (G::TH * G::TW), rem = idx - pic * (G::TH * G::TW);
      const int ty = rem / G::TW, tx = rem - ty * G::TW;
      const int gy = clampi(y0 - SR + ty, 0, H - 1), gx = clampi(cx0 - SR + tx, 0, W - 1);
      const void* pl = pic == 0 ? J.p0[0] : J.p1[0];
      const int st = pic == 0 ? J.stride0[0] : J.stride1[0];
      s_lum[pic][ty][tx] = s * ld_sample(pl, sb, (int64_t)gy * st + gx);
    }
    for(int idx = tid; idx < 4 * G::CTH * G::CTW; idx += G::NT)
    {
      const int pc = idx / (G::CTH * G::CTW), rem = idx - pc * (G::CTH * G::CTW);
      const int pic = pc >> 1, c = (pc & 1) + 1;
      const int ty = rem / G::CTW, tx = rem - ty * G::CTW;
      const int gy = clampi(cyBase + ty, 0, Hc - 1), gx = clampi(cxBase + tx, 0, Wc - 1);
      const void* pl = pic == 0 ? J.p0[c] : J.p1[c];
      const int st = pic == 0 ? J.stride0[c] : J.stride1[c];
      s_chr[pic][c - 1][ty][tx] = ld_sample(pl, sb, (int64_t)gy * st + gx);
    }
    __syncthreads();

    // ---- test values of this thread's 2 x RPT pixels ----
    int tY[RPT][2], tCb[G::NQ], tCr[G::NQ];
    #pragma unroll
    for(int i = 0; i < RPT; i++)
    {
      tY[i][0] = s_lum[tp][g * RPT + i + SR][2 * l + SR] + s * gd0;
      tY[i][1] = s_lum[tp][g * RPT + i + SR][2 * l + SR + 1] + s * gd0;
    }
    #pragma unroll
    for(int q = 0; q < G::NQ; q++)
    {
      tCb[q] = s_chr[tp][0][g * G::NQ + q + G::CS][l + G::CS] + gd1;
      tCr[q] = s_chr[tp][1][g * G::NQ + q + G::CS][l + G::CS] + gd2;
    }

    KeyT best[RPT][2];
    #pragma unroll
    for(int i = 0; i < RPT; i++) { best[i][0] = (KeyT)~(KeyT)0; best[i][1] = (KeyT)~(KeyT)0; }
    KeyT B[G::NQ][G::NC];
    #pragma unroll
    for(int q = 0; q < G::NQ; q++)
      #pragma unroll
      for(int c = 0; c < G::NC; c++) B[q][c] = 0;

    // ---- window search: stream the reference rows this thread's pixels see ----
    #pragma unroll
    for(int rr = 0; rr < RPT + 2 * SR; rr++)
    {
      int r[2 * SR + 2];
      const int* lrow = &s_lum[rp][g * RPT + rr][2 * l];
      #pragma unroll
      for(int jj = 0; jj < SR + 1; jj++) { const int2 v = *reinterpret_cast<const int2*>(lrow + 2 * jj); r[2 * jj] = v.x; r[2 * jj + 1] = v.y; }

      const int crow = fdiv2(rr - SR) + G::CS; // chroma tile row of this reference row (relative)
      const bool new_crow = (rr == 0) || (fdiv2(rr - SR) != fdiv2(rr - 1 - SR));
      if(new_crow)
      {
        int rcb[G::NC], rcr[G::NC];
        #pragma unroll
        for(int c = 0; c < G::NC; c++)
        {
          rcb[c] = s_chr[rp][0][g * G::NQ + crow][l + c];
          rcr[c] = s_chr[rp][1][g * G::NQ + crow][l + c];
        }
        // quads whose rows see this chroma row (reference rows rr and rr+1)
        const int ilo = rr - 2 * SR < 0 ? 0 : rr - 2 * SR;
        const int ihi = rr + 1 > RPT - 1 ? RPT - 1 : rr + 1;
        #pragma unroll
        for(int q = 0; q < G::NQ; q++)
        {
          if(2 * q + 1 < ilo || 2 * q > ihi) continue;
          #pragma unroll
          for(int c = 0; c < G::NC; c++)
          {
            const int db = tCb[q] - rcb[c], dr = tCr[q] - rcr[c];
            B[q][c] = (KeyT)(unsigned)(db * db) * Mw1 + (KeyT)(unsigned)(dr * dr) * Mw2;
          }
        }
      }

      #pragma unroll
      for(int i = 0; i < RPT; i++)
      {
        const int dy = rr - SR - i;
        if(dy < -SR || dy > SR) continue;
        const int q = i >> 1;
        #pragma unroll
        for(int px = 0; px < 2; px++)
        {
          #pragma unroll
          for(int dx = -SR; dx <= SR; dx++)
          {
            const int k = (dy + SR) * W2 + (dx + SR);
            const int cc = fdiv2(px + dx) + G::CS;
            const int dd = tY[i][px] - r[px + dx + SR];
            KeyT key;
            if(sizeof(KeyT) == 4) key = (KeyT)(unsigned)(dd * dd) + (B[q][cc] + (KeyT)k);
            else                  key = (KeyT)((long long)dd * dd) + (B[q][cc] + (KeyT)k);
            best[i][px] = min(best[i][px], key);
          }
        }
      }
    }

    // ---- at the argmin: exact per-component squared error and the SCP samples ----
    #pragma unroll
    for(int i = 0; i < RPT; i++)
    {
      const int y = y0 + g * RPT + i;
      #pragma unroll
      for(int px = 0; px < 2; px++)
      {
        const int x = cx0 + 2 * l + px;
        if(y >= H || x >= W) continue;
        const unsigned k = p.key_m_log2 >= 0 ? (unsigned)(best[i][px] & (KeyT)(p.key_m - 1))
                                             : (unsigned)(best[i][px] % (KeyT)p.key_m);
        const int dy = (int)(k / W2) - SR, dx = (int)(k % W2) - SR;
        const int rl = s_lum[rp][g * RPT + i + SR + dy][2 * l + px + SR + dx];
        const int crow = fdiv2(g * RPT + i + dy) + G::CS;
        const int ccol = l + fdiv2(px + dx) + G::CS;
        const int rcb = s_chr[rp][0][crow][ccol], rcr = s_chr[rp][1][crow][ccol];
        int rY, tYr;
        if(p.luma_scale_log2 >= 0) { rY = rl >> p.luma_scale_log2; tYr = tY[i][px] >> p.luma_scale_log2; }
        else                       { rY = rl / s; tYr = tY[i][px] / s; }
        const int d0 = tYr - rY, d1 = tCb[i >> 1] - rcb, d2 = tCr[i >> 1] - rcr;
        sse[i][0] += (unsigned)(d0 * d0); sse[i][1] += (unsigned)(d1 * d1); sse[i][2] += (unsigned)(d2 * d2);
        if(cmap) cmap[(int64_t)y * J.map_stride + x] = (int16_t)k;  // window index (dy + B)(2B + 1) + (dx + B)
        if(want_scp)
        { // clipU(ref - GCD) (xShftCompPic.cpp:88-92); for T2R the shift is -GCD
          const int v0 = clampi(rY - gd0, 0, mx), v1 = clampi(rcb - gd1, 0, mx), v2 = clampi(rcr - gd2, 0, mx);
          const int64_t o = (int64_t)y * J.scp_stride + x;
          scp[0][o] = (uint16_t)v0; scp[1][o] = (uint16_t)v1; scp[2][o] = (uint16_t)v2;
        }
      }
    }
  }

  // ---- per-row sums: warp reduction, one 64-bit atomic per row and component ----
  #pragma unroll
  for(int i = 0; i < RPT; i++)
  {
    const int y = y0 + g * RPT + i;
    #pragma unroll
    for(int c = 0; c < 3; c++)
    {
      const unsigned long long v = warp_sum((unsigned long long)sse[i][c]);
      if(l == 0 && y < H && v) atomicAdd(J.cps_rows + ((int64_t)dir * H + y) * 3 + c, v);
    }
  }

  if(cps_last_block(J)) { __threadfence(); finalize_cps(J, p, scratch); }
}

// ------------------------------------------------------------------------------------
// Generic kernel: any chroma format, any search range up to kMaxSR, 64-bit errors.
// One thread per pixel and direction, straight from global memory (L1/L2 cached).
// ------------------------------------------------------------------------------------
constexpr int kGenTX = 32, kGenTY = 4;

__device__ __forceinline__ int ld_pel(const DevJob& J, int pic, int c, int x, int y)
{
  const int sh = c ? J.cshift : 0;
  const void* pl = pic == 0 ? J.p0[c] : J.p1[c];
  const int st = pic == 0 ? J.stride0[c] : J.stride1[c];
  return ld_sample(pl, J.sbytes, (int64_t)(y >> sh) * st + (x >> sh));
}

__global__ void __launch_bounds__(kGenTX * kGenTY * 2) k_cps_generic(const DevJob* __restrict__ jobs, int njobs, Params p)
{
  __shared__ double scratch[2 * (kGenTX * kGenTY * 2 / 32)];
  const int jb = find_job<1>(jobs, njobs, blockIdx.x);
  const DevJob& J = jobs[jb];
  const int local = blockIdx.x - J.cps_base;
  const int ty = local / J.cps_segs, tx = local % J.cps_segs;
  const int dir = threadIdx.x / (kGenTX * kGenTY);
  const int t = threadIdx.x % (kGenTX * kGenTY);
  const int x = tx * kGenTX + (t % kGenTX), y = ty * kGenTY + (t / kGenTX);
  const int W = J.W, H = J.H, SR = p.sr, mx = (1 << J.bd) - 1;
  const int tp = dir, rp = dir ^ 1;
  const int gsgn = dir == 0 ? 1 : -1;
  const int gd[3] = { gsgn * J.sc->gcd[0], gsgn * J.sc->gcd[1], gsgn * J.sc->gcd[2] };
  unsigned long long e[3] = { 0, 0, 0 };
  if(x < W && y < H)
  {
    long long tv[3];
    for(int c = 0; c < 3; c++) tv[c] = ld_pel(J, tp, c, x, y) + gd[c];
    long long bestE = LLONG_MAX; int bx = x, by = y, bk = 0;
    for(int dy = -SR; dy <= SR; dy++)
    {
      const int yy = clampi(y + dy, 0, H - 1);
      for(int dx = -SR; dx <= SR; dx++)
      {
        const int xx = clampi(x + dx, 0, W - 1);
        long long E = 0;
        for(int c = 0; c < 3; c++) { const long long d = tv[c] - ld_pel(J, rp, c, xx, yy); E += d * d * p.w_search[c]; }
        if(E < bestE) { bestE = E; bx = xx; by = yy; bk = (dy + SR) * (2 * SR + 1) + dx + SR; }
      }
    }
    if(J.cps_map[dir]) J.cps_map[dir][(int64_t)y * J.map_stride + x] = (int16_t)bk;
    uint16_t* const* scp = dir == 0 ? J.scp1 : J.scp0;
    for(int c = 0; c < 3; c++)
    {
      const int rv = ld_pel(J, rp, c, bx, by);
      const long long d = tv[c] - rv;
      e[c] = (unsigned long long)(d * d);
      if(scp[0]) scp[c][(int64_t)y * J.scp_stride + x] = (uint16_t)clampi(rv - gd[c], 0, mx);
    }
  }
  // one row per warp (kGenTX == 32)
  for(int c = 0; c < 3; c++)
  {
    const unsigned long long v = warp_sum(e[c]);
    if((t % 32) == 0 && y < H && v) atomicAdd(J.cps_rows + ((int64_t)dir * H + y) * 3 + c, v);
  }
  if(cps_last_block(J)) { __threadfence(); finalize_cps(J, p, scratch); }
}

// ------------------------------------------------------------------------------------
// Variant table
// ------------------------------------------------------------------------------------
template <int SR, int RPT, int NWG, typename KT>
cudaError_t launch420(const DevJob* d, int n, int blocks, const Params& p, cudaStream_t st)
{
  k_cps420<SR, RPT, NWG, KT><<<blocks, Geo<SR, RPT, NWG>::NT, 0, st>>>(d, n, p);
  return cudaGetLastError();
}
cudaError_t launch_generic(const DevJob* d, int n, int blocks, const Params& p, cudaStream_t st)
{
  k_cps_generic<<<blocks, kGenTX * kGenTY * 2, 0, st>>>(d, n, p);
  return cudaGetLastError();
}

#define V420(SR, RPT, NWG, KT, K64, SUF) { "cps420_sr" #SR "_rpt" #RPT "_nwg" #NWG SUF, launch420<SR, RPT, NWG, KT>, launch420<SR, RPT, NWG, KT>, \
                                           SR, RPT * NWG, 64, K64, 1, 0 }
const CpsVariant kVariants[] = {
  { "cps_generic", launch_generic, launch_generic, 0, kGenTY, kGenTX, true, 0, 0 },
  V420(1, 8, 2, unsigned int, false, "_k32"),
  V420(2, 8, 2, unsigned int, false, "_k32"),
  V420(2, 4, 2, unsigned int, false, "_k32"),
  V420(2, 4, 4, unsigned int, false, "_k32"),
  V420(3, 8, 2, unsigned int, false, "_k32"),
  V420(4, 8, 2, unsigned int, false, "_k32"),
  V420(1, 8, 2, unsigned long long, true, "_k64"),
  V420(2, 8, 2, unsigned long long, true, "_k64"),
  V420(3, 8, 2, unsigned long long, true, "_k64"),
  V420(4, 8, 2, unsigned long long, true, "_k64"),
};
#undef V420

}  // namespace

const CpsVariant* cps_variants_staged(int* n)
{
  *n = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
  return kVariants;
}

}  // namespace qmiv
