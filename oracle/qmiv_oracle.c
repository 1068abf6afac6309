/*
 * CPU restatement of the QMIV metric hot path — TEST INFRASTRUCTURE ONLY (the oracle).
 * See qmiv_oracle.h for scope and how its parity with the reference is pinned.
 * Build: gcc -O2 -std=c11 -ffp-contract=off -fPIC -shared -pthread (oracle/Makefile).
 */
#include "qmiv_oracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------------------ */
/* small helpers                                                                         */
/* ------------------------------------------------------------------------------------ */

static inline int32_t clampi(int32_t v, int32_t lo, int32_t hi) { return v < lo ? lo : (v > hi ? hi : v); }
static inline int32_t maxval(int32_t bd) { return (1 << bd) - 1; }  /* xCommonDefCORE.h:113 */

/* Round half to even, as _mm_cvtsd_si32 / _mm_cvtss_si32 do under the default MXCSR
 * (xCommonDefCORE.h:130-131, the x86 SIMD builds the reference ships). */
static inline int32_t rne_f64(double v) { return (int32_t)nearbyint(v); }
static inline int32_t rne_f32(float v) { return (int32_t)nearbyintf(v); }

typedef void (*row_fn)(void* ctx, int32_t y0, int32_t y1);
typedef struct { row_fn fn; void* ctx; int32_t y0, y1; } row_task;
static void* row_task_main(void* p) { row_task* t = (row_task*)p; t->fn(t->ctx, t->y0, t->y1); return NULL; }

/* Static row partition over nthreads pthreads (the reference runs one task per row on its
 * pool, xThreadPool.h:20; results do not depend on the partition). */
static void par_rows(int32_t n, int32_t nthreads, row_fn fn, void* ctx)
{
  if(nthreads <= 1 || n < 2 * nthreads) { fn(ctx, 0, n); return; }
  if(nthreads > 256) nthreads = 256;
  pthread_t th[256];
  row_task tk[256];
  for(int32_t i = 0; i < nthreads; i++)
  {
    tk[i].fn = fn; tk[i].ctx = ctx;
    tk[i].y0 = (int32_t)((int64_t)n * i / nthreads);
    tk[i].y1 = (int32_t)((int64_t)n * (i + 1) / nthreads);
    pthread_create(&th[i], NULL, row_task_main, &tk[i]);
  }
  for(int32_t i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
}

void oq_default_opts(oq_opts* o)
{
  o->search_range = 2;
  o->w_search[0] = 4; o->w_search[1] = 1; o->w_search[2] = 1;
  o->w_avg[0] = 4; o->w_avg[1] = 1; o->w_avg[2] = 1;
  o->unnoticeable[0] = o->unnoticeable[1] = o->unnoticeable[2] = 0.01f;
  o->use_ws = 0; o->lat_range_deg = 180; o->ssim_window = 0; o->nthreads = 1;
}

/* ------------------------------------------------------------------------------------ */
/* a1: unpack (xSeq.cpp:179-213, UpsampleHV xPixelOpsSTD.cpp:30-49, Cvt :12)             */
/* ------------------------------------------------------------------------------------ */
int oq_unpack_frame(const uint8_t* packed, int32_t w, int32_t h, int32_t bps, int32_t cf, uint16_t* out)
{
  const size_t area = (size_t)w * h;
  #define SAMPLE(base, i) (bps == 1 ? (uint16_t)(base)[(i)] : (uint16_t)((base)[2*(i)] | ((base)[2*(i)+1] << 8)))
  for(size_t i = 0; i < area; i++) out[i] = SAMPLE(packed, i);
  const uint8_t* chroma = packed + area * bps;
  if(cf == 444)
  {
    for(int c = 0; c < 2; c++)
      for(size_t i = 0; i < area; i++) out[(c + 1) * area + i] = SAMPLE(chroma + c * area * bps, i);
    return 0;
  }
  if(cf == 420)
  {
    if((w & 1) || (h & 1)) return -1;
    const int32_t cw = w >> 1;
    const size_t carea = area >> 2;
    for(int c = 0; c < 2; c++)
    {
      const uint8_t* src = chroma + c * carea * bps;
      uint16_t* dst = out + (c + 1) * area;
      for(int32_t y = 0; y < h; y++)
        for(int32_t x = 0; x < w; x++) dst[(size_t)y * w + x] = SAMPLE(src, (size_t)(y >> 1) * cw + (x >> 1));
    }
    return 0;
  }
  if(cf == 422)
  { /* UpsampleH (xSeq.cpp:219-233): chroma planes (w/2) x h, doubled horizontally */
    if(w & 1) return -1;
    const int32_t cw = w >> 1;
    const size_t carea = area >> 1;
    for(int c = 0; c < 2; c++)
    {
      const uint8_t* src = chroma + c * carea * bps;
      uint16_t* dst = out + (c + 1) * area;
      for(int32_t y = 0; y < h; y++)
        for(int32_t x = 0; x < w; x++) dst[(size_t)y * w + x] = SAMPLE(src, (size_t)y * cw + (x >> 1));
    }
    return 0;
  }
  #undef SAMPLE
  return -1;
}

/* ------------------------------------------------------------------------------------ */
/* a15: xKBNS (xMathUtils.h:16-44, xMathUtils.cpp:12-26)                                 */
/* ------------------------------------------------------------------------------------ */
typedef struct { double s, c; } kbns;
static inline void kbns_acc(kbns* k, double v)
{
  double t = k->s + v;
  if(fabs(k->s) >= fabs(v)) k->c += ((k->s - t) + v);
  else                      k->c += ((v - t) + k->s);
  k->s = t;
}
static inline double kbns_result(const kbns* k) { return k->s + k->c; }

double oq_kbns(const double* x, size_t n)
{
  if(n == 0) return 0.0;
  kbns k = { x[0], 0.0 };
  for(size_t i = 1; i < n; i++) kbns_acc(&k, x[i]);
  return kbns_result(&k);
}

/* ------------------------------------------------------------------------------------ */
/* a3: GCD (xGlobClrDiff.cpp:15-48) with the application's argument swap                 */
/* (xGlobClrDiff.h:41): GCD_R2T = clip(rne(sum(P1-P0)/Area), +-rne_f32(unc*Max))         */
/* ------------------------------------------------------------------------------------ */
void oq_gcd(const oq_pic* p0, const oq_pic* p1, const float unc[3], int32_t gcd[3])
{
  const size_t area = (size_t)p0->width * p0->height;
  const int32_t mx = maxval(p0->bitdepth);
  for(int c = 0; c < 3; c++)
  {
    int64_t sd = 0;
    for(size_t i = 0; i < area; i++) sd += (int32_t)p1->plane[c][i] - (int32_t)p0->plane[c][i];
    const int32_t md = rne_f32(unc[c] * (float)mx);
    int32_t g = rne_f64((double)sd / (double)area);
    gcd[c] = g < -md ? -md : (g > md ? md : g);
  }
}

/* ------------------------------------------------------------------------------------ */
/* a4/a5/a10: CPS search (xCorrespPixelShift.cpp:20-85; SCP xShftCompPic.cpp:69-96)       */
/* ------------------------------------------------------------------------------------ */
typedef struct {
  const oq_pic *tst, *ref; const int32_t *gcd, *w; int32_t sr;
  uint64_t* row_sse; int8_t* argmin; int32_t* minerr; uint16_t* scp;
} cps_ctx;

static void cps_rows(void* vctx, int32_t y0, int32_t y1)
{
  const cps_ctx* k = (const cps_ctx*)vctx;
  const int32_t W = k->tst->width, H = k->tst->height, sr = k->sr, mx = maxval(k->ref->bitdepth);
  const uint16_t* const* T = k->tst->plane;
  const uint16_t* const* R = k->ref->plane;
  for(int32_t y = y0; y < y1; y++)
  {
    uint64_t rs[3] = { 0, 0, 0 };
    for(int32_t x = 0; x < W; x++)
    {
      const size_t o = (size_t)y * W + x;
      int32_t t[3];
      for(int c = 0; c < 3; c++) t[c] = (int32_t)T[c][o] + k->gcd[c];
      int32_t best = INT32_MAX, bi = -1; size_t bo = 0;
      /* row-major scan, first strict minimum wins (xCorrespPixelShift.cpp:63-80) */
      for(int32_t dy = -sr, idx = 0; dy <= sr; dy++)
      {
        const int32_t yy = clampi(y + dy, 0, H - 1);
        for(int32_t dx = -sr; dx <= sr; dx++, idx++)
        {
          const int32_t xx = clampi(x + dx, 0, W - 1);
          const size_t ro = (size_t)yy * W + xx;
          const int32_t d0 = t[0] - (int32_t)R[0][ro], d1 = t[1] - (int32_t)R[1][ro], d2 = t[2] - (int32_t)R[2][ro];
          const int32_t e = d0 * d0 * k->w[0] + d1 * d1 * k->w[1] + d2 * d2 * k->w[2];
          if(e < best) { best = e; bi = idx; bo = ro; }
        }
      }
      for(int c = 0; c < 3; c++)
      {
        const int32_t d = t[c] - (int32_t)R[c][bo];
        rs[c] += (uint64_t)(d * d);
        if(k->scp)
        {
          int32_t v = (int32_t)R[c][bo] - k->gcd[c];
          k->scp[(size_t)c * W * H + o] = (uint16_t)(v < 0 ? 0 : (v > mx ? mx : v));
        }
      }
      if(k->argmin) k->argmin[o] = (int8_t)bi;
      if(k->minerr) k->minerr[o] = best;
    }
    if(k->row_sse) for(int c = 0; c < 3; c++) k->row_sse[(size_t)y * 3 + c] = rs[c];
  }
}

void oq_cps_dir(const oq_pic* tst, const oq_pic* ref, const int32_t gcd[3], int32_t sr, const int32_t w[3],
                uint64_t* row_sse, int8_t* argmin, int32_t* minerr, uint16_t* scp, int32_t nthreads)
{
  cps_ctx k = { tst, ref, gcd, w, sr, row_sse, argmin, minerr, scp };
  par_rows(tst->height, nthreads, cps_rows, &k);
}

/* ------------------------------------------------------------------------------------ */
/* a8: CalcPSNRfromSSD (xPSNR.cpp:139-146)                                               */
/* ------------------------------------------------------------------------------------ */
double oq_psnr_from_ssd(double ssd, int32_t area, int32_t bd)
{
  const uint64_t mx = (uint64_t)maxval(bd);
  const uint64_t MAX = (uint64_t)area * (mx * mx);
  return ssd > 0 ? 10.0 * log10((double)MAX / ssd) : DBL_MAX;
}

static double psnr_from_masked_ssd(double ssd, int32_t nnm, int32_t bd, int32_t bdm) /* xPSNR.cpp:148-155 */
{
  const int64_t mp = maxval(bd), mm = maxval(bdm);
  const int64_t MAX = (int64_t)nnm * (mp * mp) * mm;
  return ssd > 0 ? 10.0 * log10((double)MAX / ssd) : DBL_MAX;
}

/* a6: xIVPSNR::xCalcQualAsymmetricPic (xIVPSNR.cpp:100-133) */
double oq_quality_from_rows(const uint64_t* row_sse, int32_t h, int32_t area, int32_t bd,
                            const double* ws, const int32_t wavg[3])
{
  double err[3];
  if(ws)
  { /* xKBNS4 over rows of (flt64)row * w[y], no H/sum(w) correction (:117-118) */
    for(int c = 0; c < 3; c++)
    {
      kbns k = { 0.0, 0.0 };
      for(int32_t y = 0; y < h; y++) kbns_acc(&k, (double)row_sse[(size_t)y * 3 + c] * ws[y]);
      err[c] = kbns_result(&k);
    }
  }
  else
  {
    for(int c = 0; c < 3; c++)
    {
      uint64_t s = 0;
      for(int32_t y = 0; y < h; y++) s += row_sse[(size_t)y * 3 + c];
      err[c] = (double)s;
    }
  }
  double q[3];
  for(int c = 0; c < 3; c++) q[c] = oq_psnr_from_ssd(err[c] > 0 ? err[c] : 1.0, area, bd);
  const int32_t sw = wavg[0] + wavg[1] + wavg[2];
  const double inv = 1.0 / (double)sw;
  const double a0 = q[0] * (double)wavg[0], a1 = q[1] * (double)wavg[1], a2 = q[2] * (double)wavg[2];
  return (((a0 + a1) + a2) + 0.0) * inv;
}

/* a9: xWeightedSpherically::initWS (xWeightedSpherically.cpp:13-29) */
void oq_ws_weights(int32_t h, int32_t lat_deg, double* w, double* correction)
{
  const double pi = 3.14159265358979323846;
  const double he = 180.0 * (double)h / (double)lat_deg;
  const double off = (he - h) / 2.0;
  for(int32_t y = 0; y < h; y++) w[y] = cos((y + off - (he / 2 - 0.5)) * pi / he);
  *correction = h / oq_kbns(w, (size_t)h);
}

/* a8: xPSNR::calcPicPSNR + xCalcCmpSSD (xPSNR.cpp:17-36,93-111) with the application's
 * exact-component replacement (xAppQMIV.cpp:837-844) */
void oq_psnr(const oq_pic* p0, const oq_pic* p1, double out[3], uint64_t ssd_out[3])
{
  const int32_t area = p0->width * p0->height;
  for(int c = 0; c < 3; c++)
  {
    uint64_t ssd = 0;
    for(int32_t i = 0; i < area; i++) { int32_t d = (int32_t)p1->plane[c][i] - (int32_t)p0->plane[c][i]; ssd += (uint64_t)(d * d); }
    out[c] = oq_psnr_from_ssd(ssd == 0 ? 1.0 : (double)ssd, area, p0->bitdepth);
    if(ssd_out) ssd_out[c] = ssd;
  }
}

/* a9: xWSPSNR::xCalcCmpWSPSNR (xWSPSNR.cpp:101-125) */
void oq_wspsnr(const oq_pic* p0, const oq_pic* p1, int32_t lat_deg, double out[3])
{
  const int32_t W = p0->width, H = p0->height, area = W * H;
  double* w = (double*)malloc(sizeof(double) * H);
  double corr;
  oq_ws_weights(H, lat_deg, w, &corr);
  for(int c = 0; c < 3; c++)
  {
    kbns k = { 0.0, 0.0 };
    for(int32_t y = 0; y < H; y++)
    {
      uint64_t s = 0;
      for(int32_t x = 0; x < W; x++) { int32_t d = (int32_t)p1->plane[c][(size_t)y * W + x] - (int32_t)p0->plane[c][(size_t)y * W + x]; s += (uint64_t)(d * d); }
      kbns_acc(&k, (double)s * w[y]);
    }
    const double err = kbns_result(&k) * corr;
    out[c] = oq_psnr_from_ssd(err == 0 ? 1.0 : err, area, p0->bitdepth);
  }
  free(w);
}

/* ------------------------------------------------------------------------------------ */
/* a11-a14: SSIM family                                                                  */
/* ------------------------------------------------------------------------------------ */

/* The window table: the normalised 11-tap Gaussian (sigma 1.5) outer product rounded to 10
 * decimals, which equals the reference's constant table entry for entry
 * (xStructSimConsts.h:31-44; pinned by tests/test_oracle_pins.py). The reference window
 * (xStructSim.cpp:19-21) uses rows/columns 0..9 of it; the GAUSS11 variant all 11. */
void oq_ssim_table(int32_t window, float table[11][11])
{
  double g[11], s = 0.0;
  for(int i = 0; i < 11; i++) { const double k = i - 5; g[i] = exp(-(k * k) / (2.0 * 1.5 * 1.5)); s += g[i]; }
  for(int i = 0; i < 11; i++) g[i] /= s;
  for(int i = 0; i < 11; i++)
    for(int j = 0; j < 11; j++) table[i][j] = (float)(nearbyint(g[i] * g[j] * 1e10) / 1e10);
  (void)window;
}

typedef struct {
  const uint16_t *t, *r; int32_t w, h, calc_l, window; double c1, c2; double* rowsum; float tab[11][11];
} ssim_ctx;

/* xStructSim<flt64,CalcL>::CalcPel (xStructSim.cpp:15-60) */
static double ssim_pel(const ssim_ctx* k, int32_t x, int32_t y)
{
  const int32_t hi = k->window == 1 ? 5 : 4;
  double sr = 0, st = 0, sr2 = 0, st2 = 0, srt = 0;
  for(int32_t dy = -5; dy <= hi; dy++)
  {
    for(int32_t dx = -5; dx <= hi; dx++)
    {
      const size_t o = (size_t)(y + dy) * k->w + (x + dx);
      const double R = (double)k->r[o], T = (double)k->t[o], C = (double)k->tab[dy + 5][dx + 5];
      sr += R * C; st += T * C; sr2 += (R * R) * C; st2 += (T * T) * C; srt += (R * T) * C;
    }
  }
  const double ar = sr, at = st;
  const double vr = sr2 - ar * ar, vt = st2 - at * at, cov = srt - ar * at;
  const double cs = (2 * cov + k->c2) / (vr + vt + k->c2);
  if(!k->calc_l) return cs;
  const double l = (2 * ar * at + k->c1) / (ar * ar + at * at + k->c1);
  return l * cs;
}

static void ssim_rows(void* vctx, int32_t y0, int32_t y1)
{
  ssim_ctx* k = (ssim_ctx*)vctx;
  for(int32_t y = y0; y < y1; y++)
  {
    const int32_t yy = y + 5; /* rows [5, H-5) (xSSIM.cpp:98) */
    double s = 0.0;
    for(int32_t x = 5; x < k->w - 5; x++) s += ssim_pel(k, x, yy);
    k->rowsum[yy] = s;
  }
}

/* xSSIM::xCalcCmpSSIM / xCalcRowSSIM (xSSIM.cpp:91-140): row sums over [5,H-5) x [5,W-5),
 * KBNS over all H rows (zeros outside), divided by W*H. */
double oq_ssim_plane(const uint16_t* t, const uint16_t* r, int32_t w, int32_t h, int32_t bd,
                     int32_t calc_l, int32_t window, int32_t nthreads)
{
  ssim_ctx k;
  k.t = t; k.r = r; k.w = w; k.h = h; k.calc_l = calc_l; k.window = window;
  const double mx = (double)maxval(bd);
  k.c1 = (0.01 * mx) * (0.01 * mx); k.c2 = (0.03 * mx) * (0.03 * mx); /* xSSIM.cpp:21-23 */
  oq_ssim_table(window, k.tab);
  k.rowsum = (double*)calloc((size_t)(h > 0 ? h : 1), sizeof(double));
  if(h > 10) par_rows(h - 10, nthreads, ssim_rows, &k);
  const double sum = oq_kbns(k.rowsum, (size_t)h);
  free(k.rowsum);
  return sum / (double)((int64_t)w * (int64_t)h);
}

void oq_ssim(const oq_pic* t, const oq_pic* r, int32_t calc_l, int32_t window, int32_t nthreads, double out[3])
{
  for(int c = 0; c < 3; c++) out[c] = oq_ssim_plane(t->plane[c], r->plane[c], t->width, t->height, t->bitdepth, calc_l, window, nthreads);
}

/* DownsampleHV (xPixelOpsSTD.cpp:50-67) to (sw>>1) x (sh>>1) */
void oq_downsample(const uint16_t* src, int32_t sw, int32_t sh, uint16_t* dst)
{
  const int32_t dw = sw >> 1, dh = sh >> 1;
  for(int32_t y = 0; y < dh; y++)
    for(int32_t x = 0; x < dw; x++)
    {
      const uint16_t* s0 = src + (size_t)(2 * y) * sw + 2 * x;
      const uint16_t* s1 = s0 + sw;
      dst[(size_t)y * dw + x] = (uint16_t)(((int32_t)s0[0] + s0[1] + s1[0] + s1[1] + 2) >> 2);
    }
}

/* xSSIM::calcPicMSSSIM (xSSIM.cpp:67-87): scale 0 CS, scales 1-3 L*CS, scale 4 CS,
 * product of score^weight (xStructSimConsts.h:27) */
void oq_msssim(const oq_pic* p0, const oq_pic* p1, int32_t window, int32_t nthreads, double out[3])
{
  static const double wts[5] = { 0.0448, 0.2856, 0.3001, 0.2363, 0.1333 };
  double sc[5][3];
  oq_ssim(p0, p1, 0, window, nthreads, sc[0]);
  int32_t w = p0->width, h = p0->height;
  uint16_t* prev[2][3] = { { 0 } };
  for(int i = 1; i < 5; i++)
  {
    const int32_t nw = w >> 1, nh = h >> 1;
    uint16_t* cur[2][3];
    for(int p = 0; p < 2; p++)
      for(int c = 0; c < 3; c++)
      {
        cur[p][c] = (uint16_t*)malloc(sizeof(uint16_t) * (size_t)(nw > 0 ? nw : 1) * (nh > 0 ? nh : 1));
        const uint16_t* src = i == 1 ? (p == 0 ? p0 : p1)->plane[c] : prev[p][c];
        oq_downsample(src, w, h, cur[p][c]);
      }
    oq_pic a = { nw, nh, p0->bitdepth, { cur[0][0], cur[0][1], cur[0][2] } };
    oq_pic b = { nw, nh, p0->bitdepth, { cur[1][0], cur[1][1], cur[1][2] } };
    oq_ssim(&a, &b, i != 4, window, nthreads, sc[i]);
    for(int p = 0; p < 2; p++) for(int c = 0; c < 3; c++) { free(prev[p][c]); prev[p][c] = cur[p][c]; }
    w = nw; h = nh;
  }
  for(int p = 0; p < 2; p++) for(int c = 0; c < 3; c++) free(prev[p][c]);
  for(int c = 0; c < 3; c++)
  {
    double v = 1.0;
    for(int i = 0; i < 5; i++) v = v * pow(sc[i][c], wts[i]);
    out[c] = v;
  }
}

/* ------------------------------------------------------------------------------------ */
/* the application's per-frame flow (xAppQMIV.cpp:661-751, 831-935)                      */
/* ------------------------------------------------------------------------------------ */
void oq_frame(const oq_pic* p0, const oq_pic* p1, const oq_opts* o, int32_t do_ssim, oq_frame_result* r)
{
  const int32_t W = p0->width, H = p0->height, area = W * H, bd = p0->bitdepth;
  memset(r, 0, sizeof(*r));
  uint64_t ssd[3];
  oq_psnr(p0, p1, r->psnr, ssd);
  for(int c = 0; c < 3; c++) r->exact[c] = ssd[c] == 0;
  double* ws = NULL; double corr = 1.0;
  if(o->use_ws) { ws = (double*)malloc(sizeof(double) * H); oq_ws_weights(H, o->lat_range_deg, ws, &corr); oq_wspsnr(p0, p1, o->lat_range_deg, r->wspsnr); }
  else { for(int c = 0; c < 3; c++) r->wspsnr[c] = r->psnr[c]; }

  oq_gcd(p0, p1, o->unnoticeable, r->gcd);
  const int32_t ng[3] = { -r->gcd[0], -r->gcd[1], -r->gcd[2] };

  uint64_t* rows0 = (uint64_t*)malloc(sizeof(uint64_t) * 3 * H);
  uint64_t* rows1 = (uint64_t*)malloc(sizeof(uint64_t) * 3 * H);
  uint16_t *scp0 = NULL, *scp1 = NULL;
  if(do_ssim) { scp0 = (uint16_t*)malloc(sizeof(uint16_t) * 3 * (size_t)area); scp1 = (uint16_t*)malloc(sizeof(uint16_t) * 3 * (size_t)area); }
  /* R2T: pixels of P0 (+GCD) searched in P1; its argmin also builds SCP1 (xShftCompPic.cpp:12-20) */
  oq_cps_dir(p0, p1, r->gcd, o->search_range, o->w_search, rows0, NULL, NULL, scp1, o->nthreads);
  oq_cps_dir(p1, p0, ng, o->search_range, o->w_search, rows1, NULL, NULL, scp0, o->nthreads);
  for(int c = 0; c < 3; c++)
  {
    r->sse_r2t[c] = 0; r->sse_t2r[c] = 0;
    for(int32_t y = 0; y < H; y++) { r->sse_r2t[c] += rows0[(size_t)y * 3 + c]; r->sse_t2r[c] += rows1[(size_t)y * 3 + c]; }
  }
  r->ivpsnr_r2t = oq_quality_from_rows(rows0, H, area, bd, ws, o->w_avg);
  r->ivpsnr_t2r = oq_quality_from_rows(rows1, H, area, bd, ws, o->w_avg);
  r->ivpsnr = r->ivpsnr_t2r < r->ivpsnr_r2t ? r->ivpsnr_t2r : r->ivpsnr_r2t; /* std::min(R2T,T2R) */

  if(do_ssim)
  {
    oq_ssim(p0, p1, 1, o->ssim_window, o->nthreads, r->ssim);
    oq_msssim(p0, p1, o->ssim_window, o->nthreads, r->msssim);
    oq_pic s0 = { W, H, bd, { scp0, scp0 + area, scp0 + 2 * (size_t)area } };
    oq_pic s1 = { W, H, bd, { scp1, scp1 + area, scp1 + 2 * (size_t)area } };
    double t2r[3], r2t[3];
    oq_ssim(p0, &s1, 1, o->ssim_window, o->nthreads, t2r); /* xSSIM.cpp:197 */
    oq_ssim(p1, &s0, 1, o->ssim_window, o->nthreads, r2t); /* xSSIM.cpp:198 */
    const double inv = 1.0 / (double)(o->w_avg[0] + o->w_avg[1] + o->w_avg[2]);
    const double vt = (((t2r[0] * o->w_avg[0] + t2r[1] * o->w_avg[1]) + t2r[2] * o->w_avg[2]) + 0.0) * inv;
    const double vr = (((r2t[0] * o->w_avg[0] + r2t[1] * o->w_avg[1]) + r2t[2] * o->w_avg[2]) + 0.0) * inv;
    r->ivssim_t2r = vt; r->ivssim_r2t = vr;
    r->ivssim = vr < vt ? vr : vt; /* std::min(T2R,R2T) */
  }
  free(rows0); free(rows1); free(scp0); free(scp1); free(ws);
}

/* ------------------------------------------------------------------------------------ */
/* masked variants                                                                       */
/* ------------------------------------------------------------------------------------ */
int32_t oq_count_nonzero(const uint16_t* m, int32_t w, int32_t h) /* xPixelOpsSTD.cpp:273 */
{
  int32_t n = 0;
  for(size_t i = 0; i < (size_t)w * h; i++) n += m[i] != 0;
  return n;
}

/* xGlobClrDiff::CalcGlobalColorDiffM (xGlobClrDiff.cpp:52-83), application argument order */
void oq_gcd_masked(const oq_pic* p0, const oq_pic* p1, const uint16_t* mask, int32_t nnm, int32_t mask_bd,
                   const float unc[3], int32_t gcd[3])
{
  const size_t area = (size_t)p0->width * p0->height;
  const int32_t mx = maxval(p0->bitdepth);
  for(int c = 0; c < 3; c++)
  {
    int64_t sd = 0;
    for(size_t i = 0; i < area; i++) sd += ((int32_t)p1->plane[c][i] - (int32_t)p0->plane[c][i]) * (int32_t)mask[i];
    const int32_t md = rne_f32(unc[c] * (float)mx);
    int32_t g = rne_f64((double)sd / (double)((int64_t)nnm * (int64_t)maxval(mask_bd)));
    gcd[c] = g < -md ? -md : (g > md ? md : g);
  }
}

/* xPSNR::calcPicPSNRM / xWSPSNR::calcPicWSPSNRM (xPSNR.cpp:92-121,163-185; xWSPSNR.cpp:150-159) */
void oq_psnr_masked(const oq_pic* p0, const oq_pic* p1, const uint16_t* mask, int32_t nnm, int32_t mask_bd,
                    const double* ws, double corr, double out[3])
{
  const int32_t W = p0->width, H = p0->height;
  for(int c = 0; c < 3; c++)
  {
    kbns k = { 0.0, 0.0 };
    uint64_t tot = 0;
    for(int32_t y = 0; y < H; y++)
    {
      uint64_t s = 0;
      for(int32_t x = 0; x < W; x++)
      {
        const size_t o = (size_t)y * W + x;
        int32_t d = (int32_t)p1->plane[c][o] - (int32_t)p0->plane[c][o];
        s += (uint64_t)(d * d) * (uint64_t)mask[o];
      }
      tot += s;
      if(ws) kbns_acc(&k, (double)s * ws[y]);
    }
    double err = ws ? kbns_result(&k) * corr : (double)tot;
    out[c] = psnr_from_masked_ssd(err, nnm, p0->bitdepth, mask_bd);
  }
}

/* xIVPSNRM::calcPicIVPSNRM (xIVPSNR.cpp:153-200; xCorrespPixelShiftSTD.cpp:80-138) */
static double quality_masked(const oq_pic* tst, const oq_pic* ref, const uint16_t* mask, int32_t nnm, int32_t mask_bd,
                             const int32_t g[3], const oq_opts* o, const double* ws)
{
  const int32_t W = tst->width, H = tst->height, sr = o->search_range;
  uint64_t* rows = (uint64_t*)calloc((size_t)H * 3, sizeof(uint64_t));
  for(int32_t y = 0; y < H; y++)
  {
    for(int32_t x = 0; x < W; x++)
    {
      const size_t po = (size_t)y * W + x;
      const int32_t m = mask[po];
      if(m == 0) continue;
      int32_t t[3];
      for(int c = 0; c < 3; c++) t[c] = (int32_t)tst->plane[c][po] + g[c];
      int32_t best = INT32_MAX; size_t bo = po;
      for(int32_t dy = -sr; dy <= sr; dy++)
      {
        const int32_t yy = clampi(y + dy, 0, H - 1);
        for(int32_t dx = -sr; dx <= sr; dx++)
        {
          const int32_t xx = clampi(x + dx, 0, W - 1);
          const size_t ro = (size_t)yy * W + xx;
          if(mask[ro] == 0) continue;
          const int32_t d0 = t[0] - (int32_t)ref->plane[0][ro], d1 = t[1] - (int32_t)ref->plane[1][ro], d2 = t[2] - (int32_t)ref->plane[2][ro];
          const int32_t e = d0 * d0 * o->w_search[0] + d1 * d1 * o->w_search[1] + d2 * d2 * o->w_search[2];
          if(e < best) { best = e; bo = ro; }
        }
      }
      for(int c = 0; c < 3; c++) { const int32_t d = t[c] - (int32_t)ref->plane[c][bo]; rows[(size_t)y * 3 + c] += (uint64_t)(d * d) * (uint64_t)m; }
    }
  }
  double err[3];
  for(int c = 0; c < 3; c++)
  {
    if(ws) { kbns k = { 0.0, 0.0 }; for(int32_t y = 0; y < H; y++) kbns_acc(&k, (double)rows[(size_t)y * 3 + c] * ws[y]); err[c] = kbns_result(&k); }
    else   { uint64_t s = 0; for(int32_t y = 0; y < H; y++) s += rows[(size_t)y * 3 + c]; err[c] = (double)s; }
  }
  free(rows);
  double q[3];
  for(int c = 0; c < 3; c++) q[c] = psnr_from_masked_ssd(err[c] > 0 ? err[c] : 1.0, nnm, tst->bitdepth, mask_bd);
  const double inv = 1.0 / (double)(o->w_avg[0] + o->w_avg[1] + o->w_avg[2]);
  return (((q[0] * o->w_avg[0] + q[1] * o->w_avg[1]) + q[2] * o->w_avg[2]) + 0.0) * inv;
}

double oq_ivpsnr_masked(const oq_pic* p0, const oq_pic* p1, const uint16_t* mask, int32_t nnm, int32_t mask_bd,
                        const int32_t g[3], const oq_opts* o, const double* ws, double* r2t_out, double* t2r_out)
{
  const int32_t ng[3] = { -g[0], -g[1], -g[2] };
  /* the application passes (I0, I1) as (Tst, Ref): R2T = Q(I1, I0, -GCD), T2R = Q(I0, I1, +GCD) */
  const double r2t = quality_masked(p1, p0, mask, nnm, mask_bd, ng, o, ws);
  const double t2r = quality_masked(p0, p1, mask, nnm, mask_bd, g, o, ws);
  if(r2t_out) *r2t_out = r2t;
  if(t2r_out) *t2r_out = t2r;
  return t2r < r2t ? t2r : r2t;
}

/* ------------------------------------------------------------------------------------ */
/* input-side operations                                                                 */
/* ------------------------------------------------------------------------------------ */
/* xColorSpaceCoeff::xRnd (xColorSpaceCoeff.h:172-176): round half away from zero */
static int32_t color_rnd(double v) { return v >= 0.0 ? (int32_t)(v + 0.5) : -(int32_t)(-v + 0.5); }

/* fixed-point matrices (xColorSpaceCoeff.h:36-100,178-203), 16 fraction bits */
void oq_color_matrix(int32_t space, int32_t to_ycbcr, int32_t m[3][3])
{
  static const double base[4][3] = { { 0.299, 0.587, 0.114 }, { 0.2126, 0.7152, 0.0722 },
                                     { 0.2120, 0.7010, 0.0870 }, { 0.2627, 0.6780, 0.0593 } };
  const double kr = base[space][0], kg = base[space][1], kb = base[space][2];
  double d[3][3];
  if(to_ycbcr)
  {
    const double sb = 0.5 / (kb - 1.0), sr = 0.5 / (kr - 1.0);
    const double t[3][3] = { { kr, kg, kb }, { sb * kr, sb * kg, 0.5 }, { 0.5, sr * kg, sr * kb } };
    memcpy(d, t, sizeof(d));
  }
  else
  {
    const double t[3][3] = { { 1.0, 0.0, 2 - 2 * kr },
                             { 1.0, 2.0 * (kb * kb - kb) / kg, 2.0 * (kr * kr - kr) / kg },
                             { 1.0, 2 - 2 * kb, 0.0 } };
    memcpy(d, t, sizeof(d));
  }
  for(int i = 0; i < 3; i++)
    for(int j = 0; j < 3; j++) m[i][j] = color_rnd(65536.0 * d[i][j]);
}

/* xColorSpaceSTD::ConvertRGB2YCbCr_I32 / ConvertYCbCr2RGB_I32 (xColorSpaceSTD.cpp:195-272) */
void oq_color_convert(const uint16_t* in, uint16_t* out, int32_t w, int32_t h, int32_t bd, int32_t space, int32_t to_ycbcr)
{
  int32_t m[3][3];
  oq_color_matrix(space, to_ycbcr, m);
  const size_t a = (size_t)w * h;
  const int32_t mid = 1 << (bd - 1), mx = maxval(bd), add = 1 << 15;
  for(size_t i = 0; i < a; i++)
  {
    const int32_t p = in[i], q = in[a + i], r = in[2 * a + i];
    int32_t o0, o1, o2;
    if(to_ycbcr)
    {
      o0 = clampi((m[0][0] * p + m[0][1] * q + m[0][2] * r + add) >> 16, 0, mx);
      o1 = clampi(((m[1][0] * p + m[1][1] * q + (r << 15) + add) >> 16) + mid, 0, mx);
      o2 = clampi((((p << 15) + m[2][1] * q + m[2][2] * r + add) >> 16) + mid, 0, mx);
    }
    else
    {
      const int32_t iu = q - mid, iv = r - mid, sy = (p << 16) + add;
      o0 = clampi((sy + m[0][2] * iv) >> 16, 0, mx);
      o1 = clampi((sy + m[1][1] * iu + m[1][2] * iv) >> 16, 0, mx);
      o2 = clampi((sy + m[2][1] * iu) >> 16, 0, mx);
    }
    out[i] = (uint16_t)o0; out[a + i] = (uint16_t)o1; out[2 * a + i] = (uint16_t)o2;
  }
}

/* xPixelOpsSTD::CheckIfInRange + ClipToRange (xPixelOpsSTD.cpp:163-209): returns the number of
   samples above 2^bd - 1 and clips them in place */
int64_t oq_range_clip(uint16_t* p, int32_t w, int32_t h, int32_t bd)
{
  const int32_t mx = maxval(bd);
  int64_t n = 0;
  for(size_t i = 0; i < (size_t)w * h; i++) if(p[i] > mx) { n++; p[i] = (uint16_t)mx; }
  return n;
}
