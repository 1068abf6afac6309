/*
 * Deterministic synthetic picture-pair generator for the QMIV metric path.
 *
 * Stands in for the reference's test sequences (which are not redistributable and not
 * needed): a smooth reference field and a tested picture displaced block-wise, offset
 * and noisy, with the shapes, bit depths and value ranges of the workloads the library
 * is measured on. Every arithmetic step is an IEEE basic operation (+ - * / sqrt) on
 * doubles with contraction disabled, and the trigonometric and exponential factors come
 * from the polynomials below rather than libm, so the same parameters give the same
 * bytes on x86-64 and aarch64.
 *
 * Reference field (per plane, chroma at half resolution):
 *   f(x,y) = sum_{k<8} a_k sin(2*pi*(x cos t_k + y sin t_k)/T_k + p_k) + gx*x + gy*y + c
 *   T_k log-uniform in [16, 512] px, t_k, p_k uniform in [0, 2*pi), quantised to
 *   [16,235] (luma) / [16,240] (chroma) in 8-bit units, scaled by 2^(bd-8).
 * Tested picture: each 32x32 luma block read from the reference at an integer shift in
 *   [-2,2]^2 (edge clamp), the co-located 16x16 chroma block at the shift halved
 *   (truncated toward zero); a global per-component offset; additive noise of standard
 *   deviation sigma (Irwin-Hall sum of 12 uniforms); rounding and clipping to [0, Max].
 *   Optional: 2-6 elliptical holes (1-4% of the area) filled with a constant, and block
 *   shifts that drift by one step every 4 frames.
 * RNG: xorshift32 (Marsaglia 2003).
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "qmiv_synth.h"

#define QS_PI 3.14159265358979323846

static inline uint32_t xs32(uint32_t* s) { uint32_t x = *s; x ^= x << 13; x ^= x >> 17; x ^= x << 5; *s = x; return x; }
static inline double uni(uint32_t* s) { return (double)(xs32(s) >> 8) * (1.0 / 16777216.0); } /* [0,1) */
static inline uint32_t mix(uint32_t a, uint32_t b)
{ /* integer hash used to derive independent per-row / per-purpose seeds */
  uint32_t h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u + (a << 6) + (a >> 2));
  h ^= h >> 16; h *= 0x85EBCA6Bu; h ^= h >> 13; h *= 0xC2B2AE35u; h ^= h >> 16;
  return h ? h : 0x1234567u;
}

/* sin on any finite argument: reduction by 2*pi (two-part constant), then an odd Taylor
 * polynomial on [-pi, pi] (truncation error < 1e-9, ample for a test field). */
static double det_sin(double x)
{
  const double inv2pi = 0.15915494309189535, c1 = 6.28318530717958623, c2 = 2.4492935982947064e-16;
  double n = x * inv2pi;
  n = (double)(int64_t)(n >= 0 ? n + 0.5 : n - 0.5);
  double r = (x - n * c1) - n * c2;
  if(r > QS_PI) r -= 2 * QS_PI;
  if(r < -QS_PI) r += 2 * QS_PI;
  const double r2 = r * r;
  double t = r, s = r;
  for(int k = 1; k <= 12; k++) { t = t * (-r2) / (double)((2 * k) * (2 * k + 1)); s += t; }
  return s;
}
static double det_cos(double x) { return det_sin(x + QS_PI / 2); }
/* 2^u for u in [0, 8]: integer part by doubling, fraction by Taylor of e^(f ln2) */
static double det_exp2(double u)
{
  int i = (int)u; double f = u - i, r = 1.0, t = 1.0;
  const double ln2 = 0.69314718055994531;
  for(int k = 1; k <= 20; k++) { t = t * f * ln2 / k; r += t; }
  while(i-- > 0) r *= 2.0;
  return r;
}

typedef struct { double a[8], ct[8], st[8], per[8], ph[8], gx, gy, c; } field_params;

static void draw_field(uint32_t* s, double lo, double hi, field_params* f)
{
  const double mid = 0.5 * (lo + hi), span = hi - lo;
  for(int k = 0; k < 8; k++)
  {
    f->per[k] = 16.0 * det_exp2(5.0 * uni(s)); /* log-uniform in [16, 512] */
    const double th = 2 * QS_PI * uni(s);
    f->ct[k] = det_cos(th); f->st[k] = det_sin(th);
    f->ph[k] = 2 * QS_PI * uni(s);
    f->a[k] = span * (0.01 + 0.05 * uni(s));
  }
  f->gx = span * (uni(s) - 0.5) * 0.2; /* total gradient over the picture, normalised below */
  f->gy = span * (uni(s) - 0.5) * 0.2;
  f->c = mid + span * (uni(s) - 0.5) * 0.2;
}

/* Evaluate a field on a w x h grid, quantise to [lo, hi] * scale; separable in x and y. */
typedef struct {
  const field_params* f; int32_t w, h; double lo, hi, scale; uint16_t* out;
  double *sx, *cx, *sy, *cy; /* per-k tables: sin/cos of the x- and y- phase parts */
} field_job;

static void field_rows(field_job* j, int32_t y0, int32_t y1)
{
  const field_params* f = j->f;
  for(int32_t y = y0; y < y1; y++)
  {
    for(int32_t x = 0; x < j->w; x++)
    {
      double v = f->c + f->gx * ((double)x / j->w) + f->gy * ((double)y / j->h);
      for(int k = 0; k < 8; k++)
      {
        const double sa = j->sx[k * j->w + x], ca = j->cx[k * j->w + x];
        const double sb = j->sy[k * j->h + y], cb = j->cy[k * j->h + y];
        v += f->a[k] * (sa * cb + ca * sb);
      }
      if(v < j->lo) v = j->lo;
      if(v > j->hi) v = j->hi;
      j->out[(size_t)y * j->w + x] = (uint16_t)(int32_t)(v * j->scale + 0.5);
    }
  }
}

typedef struct { void (*fn)(void*, int32_t, int32_t); void* ctx; int32_t y0, y1; } qs_task;
static void* qs_task_main(void* p) { qs_task* t = (qs_task*)p; t->fn(t->ctx, t->y0, t->y1); return NULL; }
static void qs_par(int32_t n, int32_t nth, void (*fn)(void*, int32_t, int32_t), void* ctx)
{
  if(nth <= 1 || n < 64) { fn(ctx, 0, n); return; }
  if(nth > 64) nth = 64;
  pthread_t th[64]; qs_task tk[64];
  for(int32_t i = 0; i < nth; i++)
  {
    tk[i].fn = fn; tk[i].ctx = ctx;
    tk[i].y0 = (int32_t)((int64_t)n * i / nth); tk[i].y1 = (int32_t)((int64_t)n * (i + 1) / nth);
    pthread_create(&th[i], NULL, qs_task_main, &tk[i]);
  }
  for(int32_t i = 0; i < nth; i++) pthread_join(th[i], NULL);
}

static void field_rows_v(void* j, int32_t y0, int32_t y1) { field_rows((field_job*)j, y0, y1); }

static void make_field(const field_params* f, int32_t w, int32_t h, double lo, double hi, double scale, uint16_t* out, int32_t nth)
{
  field_job j = { f, w, h, lo, hi, scale, out, NULL, NULL, NULL, NULL };
  j.sx = (double*)malloc(sizeof(double) * 8 * (size_t)w); j.cx = (double*)malloc(sizeof(double) * 8 * (size_t)w);
  j.sy = (double*)malloc(sizeof(double) * 8 * (size_t)h); j.cy = (double*)malloc(sizeof(double) * 8 * (size_t)h);
  for(int k = 0; k < 8; k++)
  {
    const double kx = 2 * QS_PI * f->ct[k] / f->per[k], ky = 2 * QS_PI * f->st[k] / f->per[k];
    for(int32_t x = 0; x < w; x++) { const double a = kx * x; j.sx[k * w + x] = det_sin(a); j.cx[k * w + x] = det_cos(a); }
    for(int32_t y = 0; y < h; y++) { const double b = ky * y + f->ph[k]; j.sy[k * h + y] = det_sin(b); j.cy[k * h + y] = det_cos(b); }
  }
  qs_par(h, nth, field_rows_v, &j);
  free(j.sx); free(j.cx); free(j.sy); free(j.cy);
}

typedef struct {
  const qs_params* p; const uint16_t* ref; uint16_t* tst; int32_t w, h, cmp, sub; /* sub: 1 for chroma */
  const int8_t* shifts; int32_t bw_blocks; double sigma, offset; int32_t mx;
} tst_job;

static void tst_rows(void* vj, int32_t y0, int32_t y1)
{
  tst_job* j = (tst_job*)vj;
  const int32_t bs = j->sub ? 16 : 32;
  for(int32_t y = y0; y < y1; y++)
  {
    uint32_t rs = mix(j->p->seed ^ (0xA5A5u * (uint32_t)(j->cmp + 1)), (uint32_t)y);
    for(int32_t x = 0; x < j->w; x++)
    {
      const int32_t bi = (y / bs) * j->bw_blocks + (x / bs);
      int32_t dx = j->shifts[2 * bi], dy = j->shifts[2 * bi + 1];
      if(j->sub) { dx /= 2; dy /= 2; } /* C division truncates toward zero */
      int32_t sx = x + dx, sy = y + dy;
      sx = sx < 0 ? 0 : (sx >= j->w ? j->w - 1 : sx);
      sy = sy < 0 ? 0 : (sy >= j->h ? j->h - 1 : sy);
      double n = 0.0;
      for(int i = 0; i < 12; i++) n += uni(&rs);
      double v = (double)j->ref[(size_t)sy * j->w + sx] + j->offset + j->sigma * (n - 6.0);
      int32_t q = (int32_t)(v >= 0 ? v + 0.5 : v - 0.5);
      j->tst[(size_t)y * j->w + x] = (uint16_t)(q < 0 ? 0 : (q > j->mx ? j->mx : q));
    }
  }
}

int qs_generate_pair(const qs_params* p, uint16_t* ref, uint16_t* tst)
{
  const int32_t W = p->width, H = p->height, bd = p->bitdepth;
  if(W < 2 || H < 2 || (W & 1) || (H & 1) || bd < 8 || bd > 14) return -1;
  const int32_t nth = p->nthreads > 0 ? p->nthreads : 1;
  const double scale = (double)(1 << (bd - 8));
  const int32_t mx = (1 << bd) - 1;
  const int32_t cw = W / 2, ch = H / 2;
  uint16_t* rp[3] = { ref, ref + (size_t)W * H, ref + (size_t)W * H + (size_t)cw * ch };
  uint16_t* tp[3] = { tst, tst + (size_t)W * H, tst + (size_t)W * H + (size_t)cw * ch };

  uint32_t s = mix(p->seed, 1u);
  for(int c = 0; c < 3; c++)
  {
    field_params f;
    const double lo = 16.0, hi = c == 0 ? 235.0 : 240.0;
    draw_field(&s, lo, hi, &f);
    make_field(&f, c ? cw : W, c ? ch : H, lo, hi, scale, rp[c], nth);
  }

  /* block shifts: 32x32 luma blocks; drift variant keeps per-view base shifts and steps
   * them every 4 frames, wrapping within [-2, 2] */
  const int32_t bw = (W + 31) / 32, bh = (H + 31) / 32;
  int8_t* sh = (int8_t*)malloc((size_t)2 * bw * bh);
  uint32_t ss = mix(p->drift ? p->shift_seed : p->seed, 2u);
  for(int32_t i = 0; i < bw * bh; i++)
  {
    int32_t dx = (int32_t)(xs32(&ss) % 5u) - 2, dy = (int32_t)(xs32(&ss) % 5u) - 2;
    if(p->drift)
    {
      const int32_t step = p->frame >> 2;
      dx = ((dx + 2 + step) % 5) - 2;
      dy = ((dy + 2 + 2 * step) % 5) - 2;
    }
    sh[2 * i] = (int8_t)dx; sh[2 * i + 1] = (int8_t)dy;
  }
  for(int c = 0; c < 3; c++)
  {
    tst_job j = { p, rp[c], tp[c], c ? cw : W, c ? ch : H, c, c ? 1 : 0, sh, bw, p->noise_sigma * scale, p->offset[c] * scale, mx };
    qs_par(j.h, nth, tst_rows, &j);
  }
  free(sh);

  if(p->holes)
  { /* 2-6 ellipses covering 1-4% of the picture in total, constant fill in all planes */
    uint32_t hs = mix(p->seed, 3u);
    const int32_t n = 2 + (int32_t)(xs32(&hs) % 5u);
    const double frac = 0.01 + 0.03 * uni(&hs);
    const double area_each = frac * (double)W * H / n;
    const uint16_t fill = (uint16_t)(128 * (1 << (bd - 8)));
    for(int32_t e = 0; e < n; e++)
    {
      const double ratio = 0.5 + 1.5 * uni(&hs);
      /* a * b * pi = area_each, a = ratio * b */
      double b2 = area_each / (QS_PI * ratio);
      double b = b2, prev = 0.0;
      for(int it = 0; it < 60 && b != prev; it++) { prev = b; b = 0.5 * (b + b2 / b); } /* sqrt by Newton */
      const double a = ratio * b;
      const double cx0 = W * uni(&hs), cy0 = H * uni(&hs);
      const int32_t x0 = (int32_t)(cx0 - a) - 1, x1 = (int32_t)(cx0 + a) + 1;
      const int32_t y0 = (int32_t)(cy0 - b) - 1, y1 = (int32_t)(cy0 + b) + 1;
      for(int32_t y = y0 < 0 ? 0 : y0; y <= y1 && y < H; y++)
        for(int32_t x = x0 < 0 ? 0 : x0; x <= x1 && x < W; x++)
        {
          const double u = (x + 0.5 - cx0) / a, v = (y + 0.5 - cy0) / b;
          if(u * u + v * v <= 1.0)
          {
            tp[0][(size_t)y * W + x] = fill;
            tp[1][(size_t)(y >> 1) * cw + (x >> 1)] = fill;
            tp[2][(size_t)(y >> 1) * cw + (x >> 1)] = fill;
          }
        }
    }
  }
  return 0;
}

/* Float 4:4:4 pair in [0,1] for the differentiable loss workload: the 8-bit generator's
 * reference normalised by 255; the test is the reference with block shifts, noise of
 * standard deviation sigma and a per-channel offset in [-off, off]. */
int qs_generate_float444(const qs_params* p, float* ref, float* tst, double sigma, double off_range)
{
  const int32_t W = p->width, H = p->height;
  qs_params q = *p; q.bitdepth = 8; q.holes = 0; q.noise_sigma = 0.0; q.offset[0] = q.offset[1] = q.offset[2] = 0;
  const size_t area = (size_t)W * H, carea = area / 4;
  uint16_t* r = (uint16_t*)malloc(sizeof(uint16_t) * (area + 2 * carea));
  uint16_t* t = (uint16_t*)malloc(sizeof(uint16_t) * (area + 2 * carea));
  if(qs_generate_pair(&q, r, t) != 0) { free(r); free(t); return -1; }
  uint32_t s = mix(p->seed, 4u);
  double offs[3];
  for(int c = 0; c < 3; c++) offs[c] = off_range * (2.0 * uni(&s) - 1.0);
  for(int c = 0; c < 3; c++)
  {
    const uint16_t* rs = c == 0 ? r : r + area + (size_t)(c - 1) * carea;
    const uint16_t* ts = c == 0 ? t : t + area + (size_t)(c - 1) * carea;
    for(int32_t y = 0; y < H; y++)
    {
      uint32_t rs2 = mix(p->seed ^ 0x5151u * (uint32_t)(c + 1), (uint32_t)y);
      for(int32_t x = 0; x < W; x++)
      {
        const size_t si = c == 0 ? (size_t)y * W + x : (size_t)(y >> 1) * (W / 2) + (x >> 1);
        double n = 0.0;
        for(int i = 0; i < 12; i++) n += uni(&rs2);
        ref[(size_t)c * area + (size_t)y * W + x] = (float)(rs[si] / 255.0);
        tst[(size_t)c * area + (size_t)y * W + x] = (float)(ts[si] / 255.0 + sigma * (n - 6.0) + offs[c]);
      }
    }
  }
  free(r); free(t);
  return 0;
}
