// CPS kernel template with bulk-tensor (TMA) staging: the same search, sums and shift-compensated
// pictures as k_cps420 in k_cps.cu (libs/pmbb-ivqm/src/xCorrespPixelShift.cpp:20-85,
// xShftCompPic.cpp:69-96), restructured for the GB300:
//   * one thread issues 2-D tensor loads of both pictures' luma and chroma boxes for the
//     next column chunk into a second shared-memory stage while the block searches the
//     current one (double buffering on two mbarriers; every wait is bounded);
//   * the boxes start on 16-byte boundaries and read zeros outside the picture; a
//     conversion pass turns the raw luma box into the pre-scaled int32 tile the search
//     reads, clamping coordinates at picture borders (the reference's replicated margin),
//     and chroma is read straight from the raw box through clamped indices;
//   * each warp walks 2x2 quads of one direction down its rows in a compact loop: per
//     quad, 9 chroma costs (the quad's window covers 3x3 chroma samples), then 2B+2
//     reference rows, each turned once into z = R^2 + B + kk for the quad, and per pixel and
//     candidate one multiply-add and a share of a three-way minimum (the expanded 32-bit key
//     below; the 64-bit-key shapes evaluate the key directly); the argmin's reference samples
//     are read back from the raw box inside the picture;
//   * per-row squared errors are reduced with a single warp reduction per row and
//     component per chunk, kept in one lane's register for the whole block, and added to the
//     job's row sums once at the end.
//
// The kernel is instantiated twice per variant: without argmin-map writes (k_cps_tma.cu, every
// metric call) and with them (k_cps_tma_map.cu, qmiv_cps_maps), in separate translation units
// so that the two halves compile in parallel.
#pragma once
#include <climits>
#include <cstdio>
#include <type_traits>

#include "qmiv_cps_common.cuh"
#include "qmiv_ptx.cuh"

namespace qmiv {

namespace {

constexpr uint32_t kWaitPolls = 1u << 22;

template <int SR, int QPW, int NWD, typename T, typename KeyT>
struct TGeo {
  static constexpr int SB   = (int)sizeof(T);
  // ints per converted luma sample: (s*v, (s*v)^2) for the 32-bit expanded-key search
  static constexpr int CE   = sizeof(KeyT) == 4 ? 2 : 1;
  static constexpr int R    = 2 * QPW * NWD;                   // strip rows
  static constexpr int NT   = 64 * NWD;                        // threads (2 directions x NWD warps)
  static constexpr int XA   = 16 / SB;                         // box x alignment in samples
  static constexpr int TH   = R + 2 * SR;                      // luma rows staged
  static constexpr int TW   = 64 + 2 * SR;                     // converted luma tile width
  static constexpr int RW   = 64 + 2 * XA;                     // raw luma box width
  static constexpr int CS   = ceil2(SR);
  static constexpr int CTH  = fdiv2(R - 1 + SR) + CS + 1;      // chroma rows staged
  static constexpr int CRW  = 32 + 2 * XA;                     // raw chroma box width
  static constexpr int NC   = fdiv2(1 + SR) + CS + 1;          // chroma samples a quad's window spans per axis
  static constexpr int KS_LOG2 = (2 * SR + 1) <= 4 ? 2 : ((2 * SR + 1) <= 8 ? 3 : 4);
  static constexpr int KS   = 1 << KS_LOG2;                    // window-index row pitch (power of two)
  static constexpr int LBOX = (TH * RW * SB + 127) / 128 * 128;
  static constexpr int CBOX = (CTH * CRW * SB + 127) / 128 * 128;
  static constexpr int STAGE = 2 * LBOX + 4 * CBOX;
  static constexpr uint32_t TX = 2u * TH * RW * SB + 4u * CTH * CRW * SB;
  static constexpr int CVT  = 2 * TH * TW * 4 * CE;
  static constexpr int ACC  = 2 * R * 3 * 8;
  static constexpr int SMEM = 2 * STAGE + CVT + ACC + 32;    // + 3 mbarriers
  // resident blocks the register budget is sized for: 20 warps per SM at search range <= 2 (the
  // shared memory of the 128-thread shapes holds five blocks, so a tighter budget buys nothing)
  static constexpr int MINB = SR <= 2 ? 640 / NT : 512 / NT;
  static_assert(SR <= XA, "halo wider than the box alignment pad");
  static_assert(RW <= 256 && TH <= 256 && CRW <= 256 && CTH <= 256, "tensor box too large");
};

// MAP: the launch writes argmin maps (a separate instantiation, since even a never-taken map
// write keeps the window index live in the inner loop and cost 7% of the kernel's time)
template <int SR, int QPW, int NWD, typename KeyT, typename T, bool MAP>
__global__ void __launch_bounds__(TGeo<SR, QPW, NWD, T, KeyT>::NT, TGeo<SR, QPW, NWD, T, KeyT>::MINB)
k_cps420_tma(const DevJob* __restrict__ jobs, int njobs, Params p)
{
  using G = TGeo<SR, QPW, NWD, T, KeyT>;
  constexpr int W2 = 2 * SR + 1;
  constexpr int CE = G::CE;
  extern __shared__ __align__(128) unsigned char smem[];
  int* cvt = reinterpret_cast<int*>(smem + 2 * G::STAGE);
  unsigned long long* acc = reinterpret_cast<unsigned long long*>(smem + 2 * G::STAGE + G::CVT);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 2 * G::STAGE + G::CVT + G::ACC);
  __shared__ double scratch[2 * (G::NT / 32)];

  const int jb = find_job<1>(jobs, njobs, blockIdx.x);
  const DevJob& J = jobs[jb];
  const int local = blockIdx.x - J.cps_base;
  const int strip = local / J.cps_segs, seg = local % J.cps_segs;
  const int W = J.W, H = J.H, Wc = W >> 1, Hc = H >> 1;
  const int y0 = strip * G::R;
  const int nchunks = (W + 63) >> 6;
  const int ch0 = seg * J.cps_seg_chunks, ch1 = min(nchunks, ch0 + J.cps_seg_chunks);
  const unsigned char* tm = reinterpret_cast<const unsigned char*>(J.tmaps);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int dir = warp / NWD, wg = warp % NWD;
  const int tp = dir, rp = dir ^ 1;
  const int gs = dir == 0 ? 1 : -1;
  const int gd0 = gs * J.sc->gcd[0], gd1 = gs * J.sc->gcd[1], gd2 = gs * J.sc->gcd[2];
  const int s = p.luma_scale;
  const KeyT Mw1 = (KeyT)p.key_m * (KeyT)p.w_search[1];
  const KeyT Mw2 = (KeyT)p.key_m * (KeyT)p.w_search[2];
  const int mx = (1 << J.bd) - 1;
  uint16_t* const* scp = dir == 0 ? J.scp1 : J.scp0;
  const bool want_scp = scp[0] != nullptr;
  int16_t* const cmap = J.cps_map[dir];
  const int cry0 = (y0 >> 1) - G::CS;

  for(int i = tid; i < 2 * G::R * 3; i += G::NT) acc[i] = 0ull;
  if(tid == 0)
  {
    ptx::mbar_init(&bar[0], 1);
    ptx::mbar_init(&bar[1], 1);
    ptx::mbar_init(&bar[2], 1);  // no copy ever arrives on it: the target of the timeout test hook
    ptx::fence_mbar_init();
    for(int i = 0; i < 6; i++) ptx::prefetch_tmap(tm + 128 * i);
  }
  __syncthreads();

  auto issue = [&](int ch, int stg) {
    const int cx0 = ch << 6;
    unsigned char* sb = smem + stg * G::STAGE;
    ptx::mbar_arrive_expect_tx(&bar[stg], G::TX);
    ptx::tma_load_2d(sb, tm + 0 * 128, cx0 - G::XA, y0 - SR, &bar[stg]);
    ptx::tma_load_2d(sb + G::LBOX, tm + 3 * 128, cx0 - G::XA, y0 - SR, &bar[stg]);
    #pragma unroll
    for(int pc = 0; pc < 4; pc++)
    {
      const int pic = pc >> 1, c = (pc & 1) + 1;
      ptx::tma_load_2d(sb + 2 * G::LBOX + pc * G::CBOX, tm + (pic * 3 + c) * 128, (cx0 >> 1) - G::XA, cry0, &bar[stg]);
    }
  };
  if(tid == 0 && ch0 < ch1) issue(ch0, 0);

  bool failed = false;
  int it = 0;
  // Per-row squared errors: a warp owns the same 2 QPW rows of its direction in every chunk, so
  // each (quad, row, component) sum of the block lives in one lane's register (lane
  // 6 qi + 3 a + c), which takes the warp's reduction of that sum per chunk; the lanes write
  // them to shared memory once, after the last chunk. Shapes with more than 32 such sums per
  // warp add each reduction to shared memory instead.
  constexpr bool kLaneSums = 6 * QPW <= 32;
  unsigned long long lacc = 0;
  for(int ch = ch0; ch < ch1; ch++, it++)
  {
    const int stg = it & 1;
    if(tid == 0 && ch + 1 < ch1) issue(ch + 1, stg ^ 1);
    const bool ok = (it == 0 && p.first_wait_test_polls)
                        ? ptx::mbar_wait_bounded(&bar[2], 0u, p.first_wait_test_polls)
                        : ptx::mbar_wait_bounded(&bar[stg], (uint32_t)((it >> 1) & 1), kWaitPolls);
    if(__syncthreads_or(!ok)) { failed = true; break; }

    const int cx0 = ch << 6;
    const unsigned char* sb = smem + stg * G::STAGE;

    // ---- luma: raw box -> pre-scaled int32 tile with clamped coordinates ----
    {
      const bool border = (y0 - SR < 0) || (y0 + G::R + SR > H) || (cx0 - SR < 0) || (cx0 + 64 + SR > W);
      constexpr int PAIRS = G::TW / 2;
      bool done = false;
      if constexpr(CE == 2 && G::TW % 4 == 0)
      {
        if(!border)
        { // interior chunk, (sample, square) tile: four samples per item from two 2-sample
          // words, the scale as a shift when it is a power of two
          constexpr int QUADS = G::TW / 4;
          using W2 = typename std::conditional<sizeof(T) == 2, uint32_t, uint16_t>::type;
          constexpr int WB = 8 * (int)sizeof(T);
          const int ls = p.luma_scale_log2;
          constexpr int ITEMS = 2 * G::TH * QUADS, PER = (ITEMS + G::NT - 1) / G::NT;
          constexpr unsigned M = (1u << WB) - 1u;
          W2 w[PER][2];
          #pragma unroll
          for(int k = 0; k < PER; k++)
          { // every load first
            const int idx = min(tid + k * G::NT, ITEMS - 1);
            const int row = idx / QUADS, qd = idx - row * QUADS;  // row = picture * TH + staged row
            const int pic = row >= G::TH ? 1 : 0, ty = row - pic * G::TH;
            const T* rl = reinterpret_cast<const T*>(sb + pic * G::LBOX) + ty * G::RW + 4 * qd + G::XA - SR;
            w[k][0] = *reinterpret_cast<const W2*>(rl);
            w[k][1] = *reinterpret_cast<const W2*>(rl + 2);
          }
          #pragma unroll
          for(int k = 0; k < PER; k++)
          {
            const int idx = tid + k * G::NT;
            if(idx >= ITEMS) break;
            const int row = idx / QUADS, qd = idx - row * QUADS;
            int v[4] = { (int)(w[k][0] & M), (int)(w[k][0] >> WB), (int)(w[k][1] & M), (int)(w[k][1] >> WB) };
            #pragma unroll
            for(int j = 0; j < 4; j++) v[j] = ls >= 0 ? v[j] << ls : s * v[j];
            int* dst = &cvt[2 * (row * G::TW + 4 * qd)];
            *reinterpret_cast<int4*>(dst) = make_int4(v[0], v[0] * v[0], v[1], v[1] * v[1]);
            *reinterpret_cast<int4*>(dst + 4) = make_int4(v[2], v[2] * v[2], v[3], v[3] * v[3]);
          }
          done = true;
        }
      }
      for(int idx = tid; !done && idx < 2 * G::TH * PAIRS; idx += G::NT)
      {
        const int pic = idx / (G::TH * PAIRS);
        const int rem = idx - pic * (G::TH * PAIRS);
        const int ty = rem / PAIRS, tx = 2 * (rem - ty * PAIRS);
        const T* rl = reinterpret_cast<const T*>(sb + pic * G::LBOX);
        int v0, v1;
        if(!border)
        {
          const int o = ty * G::RW + tx + G::XA - SR;
          v0 = rl[o]; v1 = rl[o + 1];
        }
        else
        {
          const int ry = clampi(y0 - SR + ty, 0, H - 1) - (y0 - SR);
          const int x0 = clampi(cx0 - SR + tx, 0, W - 1) - (cx0 - G::XA);
          const int x1 = clampi(cx0 - SR + tx + 1, 0, W - 1) - (cx0 - G::XA);
          v0 = rl[ry * G::RW + x0]; v1 = rl[ry * G::RW + x1];
        }
        const int e = (pic * G::TH + ty) * G::TW + tx;
        if constexpr(CE == 2) *reinterpret_cast<int4*>(&cvt[2 * e]) = make_int4(s * v0, s * v0 * s * v0, s * v1, s * v1 * s * v1);
        else                  *reinterpret_cast<int2*>(&cvt[e]) = make_int2(s * v0, s * v1);
      }
    }
    __syncthreads();

    // ---- search ----
    {
      const int* cvtT = cvt + tp * G::TH * G::TW * CE;
      const int* cvtR = cvt + rp * G::TH * G::TW * CE;
      const T* chrT0 = reinterpret_cast<const T*>(sb + 2 * G::LBOX + (tp * 2 + 0) * G::CBOX);
      const T* chrT1 = reinterpret_cast<const T*>(sb + 2 * G::LBOX + (tp * 2 + 1) * G::CBOX);
      const T* chrR0 = reinterpret_cast<const T*>(sb + 2 * G::LBOX + (rp * 2 + 0) * G::CBOX);
      const T* chrR1 = reinterpret_cast<const T*>(sb + 2 * G::LBOX + (rp * 2 + 1) * G::CBOX);
      const int cxh = cx0 >> 1, crx0 = cxh - G::XA;
      int ccol[G::NC];
      #pragma unroll
      for(int j = 0; j < G::NC; j++) ccol[j] = clampi(cxh + lane - G::CS + j, 0, Wc - 1) - crx0;
      const int tcol = clampi(cxh + lane, 0, Wc - 1) - crx0;

      // Chunks whose search windows, chroma cells and pixels all lie inside the picture skip
      // every clamp and validity mask (IN = true); the edge chunks keep them.
      const bool interior = y0 >= 2 * SR + 2 && y0 + G::R + 2 * SR + 2 <= H && cx0 >= 2 * SR + 2 && cx0 + 64 + 2 * SR + 2 <= W;
      auto run_quads = [&](auto in_tag) {
      constexpr bool IN = decltype(in_tag)::value;
      #pragma unroll 1
      for(int qi = 0; qi < QPW; qi++)
      {
        const int qr = wg * QPW + qi;
        const int yq = y0 + 2 * qr;
        if(yq >= H) break;
        int tY[2][2];
        #pragma unroll
        for(int a = 0; a < 2; a++)
        {
          const int e = (2 * qr + a + SR) * G::TW + 2 * lane + SR;
          if constexpr(CE == 2)
          {
            if(SR & 1) { tY[a][0] = cvtT[2 * e]; tY[a][1] = cvtT[2 * e + 2]; }
            else       { const int4 v = *reinterpret_cast<const int4*>(&cvtT[2 * e]); tY[a][0] = v.x; tY[a][1] = v.z; }
          }
          else
          {
            const int2 v = *reinterpret_cast<const int2*>(&cvtT[e - (SR & 1)]);
            if(SR & 1) { tY[a][0] = v.y; tY[a][1] = cvtT[e + 1]; }
            else       { tY[a][0] = v.x; tY[a][1] = v.y; }
          }
          tY[a][0] += s * gd0; tY[a][1] += s * gd0;
        }
        const int qc = (y0 >> 1) + qr;
        const int trow = (IN ? qc : clampi(qc, 0, Hc - 1)) - cry0;
        const int tCb = (int)chrT0[trow * G::CRW + tcol] + gd1;
        const int tCr = (int)chrT1[trow * G::CRW + tcol] + gd2;
        KeyT B[G::NC][G::NC];
        #pragma unroll
        for(int jr = 0; jr < G::NC; jr++)
        {
          const int crow = (IN ? qc - G::CS + jr : clampi(qc - G::CS + jr, 0, Hc - 1)) - cry0;
          #pragma unroll
          for(int jc = 0; jc < G::NC; jc++)
          {
            const int db = tCb - (int)chrR0[crow * G::CRW + ccol[jc]];
            const int dr = tCr - (int)chrR1[crow * G::CRW + ccol[jc]];
            B[jr][jc] = (KeyT)(unsigned)(db * db) * Mw1 + (KeyT)(unsigned)(dr * dr) * Mw2;
          }
        }
        KeyT best[2][2];
        if constexpr(sizeof(KeyT) == 4)
        {
          // Expanded key. With TY the scaled tested luma, R a reference luma sample and B its
          // chroma cost, key(k) = (TY - R)^2 + B + k = TY^2 - 2 TY R + (R^2 + B + k). TY^2 is
          // constant per pixel, and so is the offset between the window index k and the
          // tile position kk = rr*KS + j of R (k = kk - (a*KS + px)), while B depends on R's
          // position only (its chroma cell). So per reference position z = R^2 + B + kk is
          // formed once for all four pixels of the quad, and each candidate is one
          // multiply-add (-2 TY) * R + z and a share of a three-way minimum. The candidates
          // of a pixel lie in [-TY^2 + c, kmax - TY^2 + c], inside int32 whenever the packed
          // key is below 2^31 (the host picks these variants only then), so wrapping
          // 32-bit arithmetic gives their exact values; the packed key is recovered by
          // adding TY^2 - c back.
          int nt[2][2], bs[2][2];
          #pragma unroll
          for(int a = 0; a < 2; a++)
            #pragma unroll
            for(int px = 0; px < 2; px++) { nt[a][px] = -2 * tY[a][px]; bs[a][px] = INT_MAX; }
          #pragma unroll
          for(int rr = 0; rr < 2 * SR + 2; rr++)
          {
            int r[2 * SR + 2];
            unsigned z[2 * SR + 2];
            const int* lrow = cvtR + ((2 * qr + rr) * G::TW + 2 * lane) * 2;
            const int jr = fdiv2(rr - SR) + G::CS;
            #pragma unroll
            for(int jj = 0; jj < SR + 1; jj++)
            {
              const int4 v = *reinterpret_cast<const int4*>(lrow + 4 * jj);
              r[2 * jj] = v.x; z[2 * jj] = (unsigned)v.y;
              r[2 * jj + 1] = v.z; z[2 * jj + 1] = (unsigned)v.w;
            }
            #pragma unroll
            for(int j = 0; j < 2 * SR + 2; j++) z[j] += (unsigned)B[jr][fdiv2(j - SR) + G::CS] + (unsigned)(rr * G::KS + j);
            #pragma unroll
            for(int a = 0; a < 2; a++)
            {
              const int dy = rr - SR - a;
              if(dy < -SR || dy > SR) continue;
              #pragma unroll
              for(int px = 0; px < 2; px++)
                #pragma unroll
                for(int dx = -SR; dx <= SR; dx++)
                {
                  const int j = px + dx + SR;
                  bs[a][px] = min(bs[a][px], (int)((unsigned)nt[a][px] * (unsigned)r[j] + z[j]));
                }
            }
          }
          #pragma unroll
          for(int a = 0; a < 2; a++)
            #pragma unroll
            for(int px = 0; px < 2; px++)
              best[a][px] = (KeyT)((unsigned)bs[a][px] + (unsigned)tY[a][px] * (unsigned)tY[a][px] - (unsigned)(a * G::KS + px));
        }
        else
        {
          best[0][0] = best[0][1] = best[1][0] = best[1][1] = (KeyT)~(KeyT)0;
          #pragma unroll
          for(int rr = 0; rr < 2 * SR + 2; rr++)
          {
            int r[2 * SR + 2];
            const int* lrow = cvtR + (2 * qr + rr) * G::TW + 2 * lane;
            #pragma unroll
            for(int jj = 0; jj < SR + 1; jj++) { const int2 v = *reinterpret_cast<const int2*>(lrow + 2 * jj); r[2 * jj] = v.x; r[2 * jj + 1] = v.y; }
            const int jr = fdiv2(rr - SR) + G::CS;
            #pragma unroll
            for(int a = 0; a < 2; a++)
            {
              const int dy = rr - SR - a;
              if(dy < -SR || dy > SR) continue;
              #pragma unroll
              for(int px = 0; px < 2; px++)
                #pragma unroll
                for(int dx = -SR; dx <= SR; dx++)
                {
                  // window index with a power-of-two row pitch: same order as the row-major scan
                  const int k = (dy + SR) * G::KS + (dx + SR);
                  const int jc = fdiv2(px + dx) + G::CS;
                  const int dd = tY[a][px] - r[px + dx + SR];
                  best[a][px] = min(best[a][px], (KeyT)((long long)dd * dd) + B[jr][jc] + (KeyT)k);
                }
            }
          }
        }

        // argmin: exact per-component squared error, SCP samples
        unsigned sq[2][3] = { { 0, 0, 0 }, { 0, 0, 0 } };
        int sv[2][2][3];
        #pragma unroll
        for(int a = 0; a < 2; a++)
          #pragma unroll
          for(int px = 0; px < 2; px++)
          {
            const unsigned k = p.key_m_log2 >= 0 ? (unsigned)(best[a][px] & (KeyT)(p.key_m - 1))
                                                 : (unsigned)(best[a][px] % (KeyT)p.key_m);
            const int dy = (int)(k >> G::KS_LOG2) - SR, dx = (int)(k & (G::KS - 1)) - SR;
            // the argmin's reference luma: from the raw 16-bit box inside the picture (one
            // shared-memory wavefront per warp), from the clamped, scaled tile at the edges
            int rl;
            if constexpr(IN)
              rl = reinterpret_cast<const T*>(sb + rp * G::LBOX)[(2 * qr + a + SR + dy) * G::RW + 2 * lane + px + dx + G::XA];
            else
              rl = cvtR[((2 * qr + a + SR + dy) * G::TW + 2 * lane + px + SR + dx) * CE];
            const int crow = (IN ? qc + ((a + dy) >> 1) : clampi(qc + ((a + dy) >> 1), 0, Hc - 1)) - cry0;
            const int ccl = (IN ? cxh + lane + ((px + dx) >> 1) : clampi(cxh + lane + ((px + dx) >> 1), 0, Wc - 1)) - crx0;
            const int rcb = chrR0[crow * G::CRW + ccl], rcr = chrR1[crow * G::CRW + ccl];
            int rY, tYr;
            if(p.luma_scale_log2 >= 0) { rY = IN ? rl : rl >> p.luma_scale_log2; tYr = tY[a][px] >> p.luma_scale_log2; }
            else                       { rY = IN ? rl : rl / s; tYr = tY[a][px] / s; }
            const int d0 = tYr - rY, d1 = tCb - rcb, d2 = tCr - rcr;
            if(IN)
            {
              sq[a][0] += (unsigned)(d0 * d0); sq[a][1] += (unsigned)(d1 * d1); sq[a][2] += (unsigned)(d2 * d2);
            }
            else
            {
              const unsigned vm = (yq + a < H && cx0 + 2 * lane + px < W) ? 0xFFFFFFFFu : 0u;
              sq[a][0] += (unsigned)(d0 * d0) & vm; sq[a][1] += (unsigned)(d1 * d1) & vm; sq[a][2] += (unsigned)(d2 * d2) & vm;
            }
            sv[a][px][0] = rY; sv[a][px][1] = rcb; sv[a][px][2] = rcr;
            if(MAP && cmap && (IN || (yq + a < H && cx0 + 2 * lane + px < W)))
            { // the reference's window index (dy + B)(2B + 1) + (dx + B)
              cmap[(int64_t)(yq + a) * J.map_stride + cx0 + 2 * lane + px] =
                  (int16_t)((int)(k >> G::KS_LOG2) * W2 + (int)(k & (G::KS - 1)));
            }
          }
        if(want_scp)
        { // clipU(ref - GCD) (xShftCompPic.cpp:88-92); for T2R the shift is -GCD
          #pragma unroll
          for(int a = 0; a < 2; a++)
            #pragma unroll
            for(int px = 0; px < 2; px++)
            {
              const int y = yq + a, x = cx0 + 2 * lane + px;
              if(!IN && !(y < H && x < W)) continue;
              const int64_t o = (int64_t)y * J.scp_stride + x;
              scp[0][o] = (uint16_t)clampi(sv[a][px][0] - gd0, 0, mx);
              scp[1][o] = (uint16_t)clampi(sv[a][px][1] - gd1, 0, mx);
              scp[2][o] = (uint16_t)clampi(sv[a][px][2] - gd2, 0, mx);
            }
        }
        {
          const int t = lane - 6 * qi;  // which of the quad's six sums this lane keeps, if any
          unsigned long long pick = 0;
          #pragma unroll
          for(int a = 0; a < 2; a++)
            #pragma unroll
            for(int c = 0; c < 3; c++)
            {
              unsigned long long v;
              if(sizeof(KeyT) == 4) v = __reduce_add_sync(0xffffffffu, sq[a][c]);
              else v = ((unsigned long long)__reduce_add_sync(0xffffffffu, sq[a][c] >> 16) << 16) +
                       __reduce_add_sync(0xffffffffu, sq[a][c] & 0xFFFFu);
              if constexpr(kLaneSums) pick = t == a * 3 + c ? v : pick;
              else if(lane == 0) acc[(dir * G::R + 2 * qr + a) * 3 + c] += v;
            }
          if constexpr(kLaneSums) lacc += pick;
        }
      }
      };
      if(interior) run_quads(std::true_type{});
      else         run_quads(std::false_type{});
    }
    __syncthreads();
  }

  if(kLaneSums && lane < 6 * QPW)
  {
    const int qi = lane / 6, rem = lane - 6 * qi, a = rem / 3, c = rem - 3 * a;
    acc[(dir * G::R + 2 * (wg * QPW + qi) + a) * 3 + c] = lacc;
  }
  if(failed && tid == 0)
  { // let the copies in flight land before the block's shared memory is released
    const int stg = it & 1;
    ptx::mbar_wait_bounded(&bar[stg], (uint32_t)((it >> 1) & 1), kWaitPolls);
    if(ch0 + it + 1 < ch1) ptx::mbar_wait_bounded(&bar[stg ^ 1], (uint32_t)(((it + 1) >> 1) & 1), kWaitPolls);
    atomicExch(&J.sc->status, (int)QMIV_DEVICE_TIMEOUT);
  }
  __syncthreads();
  for(int i = tid; i < 2 * G::R * 3; i += G::NT)
  {
    const int d = i / (G::R * 3), rem = i - d * (G::R * 3), row = rem / 3, c = rem - row * 3;
    const int y = y0 + row;
    const unsigned long long v = acc[i];
    if(y < H && v) atomicAdd(J.cps_rows + ((int64_t)d * H + y) * 3 + c, v);
  }
  if(cps_last_block(J)) { __threadfence(); finalize_cps(J, p, scratch); }
}

template <int SR, int QPW, int NWD, typename KeyT, typename T, bool MAP>
cudaError_t launch_tma_as(const DevJob* d, int n, int blocks, const Params& p, cudaStream_t st)
{
  using G = TGeo<SR, QPW, NWD, T, KeyT>;
  static std::atomic<bool> attr[kStaticMaxDevices];
  const int dv = device_slot();
  if(!attr[dv].load(std::memory_order_acquire))
  {
    cudaError_t e = cudaFuncSetAttribute(k_cps420_tma<SR, QPW, NWD, KeyT, T, MAP>, cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM);
    if(e != cudaSuccess) return e;
    // all of the unified L1 as shared memory: the kernel stages through TMA and reads no
    // global data through L1, and the default split held it to two resident blocks
    e = cudaFuncSetAttribute(k_cps420_tma<SR, QPW, NWD, KeyT, T, MAP>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if(e != cudaSuccess) return e;
    attr[dv].store(true, std::memory_order_release);
  }
  k_cps420_tma<SR, QPW, NWD, KeyT, T, MAP><<<blocks, G::NT, G::SMEM, st>>>(d, n, p);
  return cudaGetLastError();
}

}  // namespace
}  // namespace qmiv

// The TMA variants: search range, quads per warp, warps per direction, key type, sample type,
// 64-bit keys, sample bytes, name suffix.
#define QMIV_TMA_VARIANTS(X) \
  X(2, 4, 4, unsigned int, uint16_t, false, 2, _k32_u16) \
  X(2, 4, 2, unsigned int, uint16_t, false, 2, _k32_u16) \
  X(2, 2, 4, unsigned int, uint16_t, false, 2, _k32_u16) \
  X(2, 8, 2, unsigned int, uint16_t, false, 2, _k32_u16) \
  X(2, 8, 4, unsigned int, uint16_t, false, 2, _k32_u16) \
  X(1, 4, 4, unsigned int, uint16_t, false, 2, _k32_u16) \
  X(3, 4, 4, unsigned int, uint16_t, false, 2, _k32_u16) \
  X(4, 4, 4, unsigned int, uint16_t, false, 2, _k32_u16) \
  X(1, 4, 2, unsigned int, uint16_t, false, 2, _k32_u16) \
  X(3, 4, 2, unsigned int, uint16_t, false, 2, _k32_u16) \
  X(4, 4, 2, unsigned int, uint16_t, false, 2, _k32_u16) \
  X(1, 4, 4, unsigned long long, uint16_t, true, 2, _k64_u16) \
  X(2, 4, 4, unsigned long long, uint16_t, true, 2, _k64_u16) \
  X(3, 4, 4, unsigned long long, uint16_t, true, 2, _k64_u16) \
  X(4, 4, 4, unsigned long long, uint16_t, true, 2, _k64_u16) \
  X(1, 4, 4, unsigned int, uint8_t, false, 1, _k32_u8) \
  X(2, 4, 4, unsigned int, uint8_t, false, 1, _k32_u8) \
  X(3, 4, 4, unsigned int, uint8_t, false, 1, _k32_u8) \
  X(4, 4, 4, unsigned int, uint8_t, false, 1, _k32_u8)

#define QMIV_TMA_MAP_LAUNCHER(SR, QPW, NWD, KT, T, K64, SB, SUF) \
  launch_tma_map_sr##SR##_q##QPW##_w##NWD##SUF
#define QMIV_TMA_MAP_DECL(SR, QPW, NWD, KT, T, K64, SB, SUF) \
  cudaError_t QMIV_TMA_MAP_LAUNCHER(SR, QPW, NWD, KT, T, K64, SB, SUF)(const DevJob* d, int n, int blocks, \
                                                                      const Params& p, cudaStream_t st)
