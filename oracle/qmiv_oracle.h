/*
 * CPU restatement of the QMIV metric hot path (reference: libs/pmbb-ivqm) — TEST
 * INFRASTRUCTURE ONLY.
 *
 * This is the oracle the GPU path is checked against. Only tests/, the smoke check
 * in __graft_entry__.py and the CPU-baseline leg of bench.py may load it; the product
 * never links or calls it. Parity of this restatement is pinned against the reference
 * itself: tests compare it with the reference library built from source by
 * oracle/build_ref.sh (oracle/_ref/qmiv_ref_harness) on the bundled example pictures
 * (whose IV-PSNR / PSNR values the reference publishes in example/README.md:44-47,67-69)
 * and on seeded synthetic pictures, and with the golden fixtures in tests/golden/.
 *
 * Pictures are 4:4:4 planar uint16 with no margin; every window read clamps its
 * coordinates, which equals the reference's edge-replicated margin of
 * roundup4(search range) >= search range pixels (libs/pmbb-core/src/xPixelOpsSTD.cpp:210,
 * apps/QMIV/src/xAppQMIV.cpp:330).
 *
 * Integer results (GCD, CPS maps, SSE sums, shift-compensated pictures) are bit-exact
 * with the reference. FP64 results are computed in the reference's order of operations
 * with contraction disabled; they agree with the x86-64-v4 reference build to ~1e-15
 * (that build contracts some products into FMAs).
 */
#ifndef QMIV_ORACLE_H
#define QMIV_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oq_pic {
  int32_t width, height, bitdepth;
  const uint16_t* plane[3]; /* 4:4:4, row stride == width */
} oq_pic;

typedef struct oq_opts {
  int32_t search_range;      /* xCorrespPixelShift.h:32, default 2 */
  int32_t w_search[3];       /* xCorrespPixelShift.h:33, default 4:1:1 */
  int32_t w_avg[3];          /* default 4:1:1 */
  float   unnoticeable[3];   /* xGlobClrDiff.h:20, default 0.01 */
  int32_t use_ws;            /* equirectangular weighting for PSNR-family */
  int32_t lat_range_deg;     /* default 180 */
  int32_t ssim_window;       /* 0: reference 10x10 truncated window, 1: full 11x11 Gaussian */
  int32_t nthreads;          /* host threads used by the row loops (>=1) */
} oq_opts;

typedef struct oq_frame_result {
  int32_t gcd[3];            /* GCD_R2T as the application computes it */
  int32_t exact[3];          /* component identical in both pictures */
  double  psnr[3], wspsnr[3];
  double  ivpsnr, ivpsnr_r2t, ivpsnr_t2r;
  uint64_t sse_r2t[3], sse_t2r[3];
  double  ssim[3], msssim[3];
  double  ivssim, ivssim_r2t, ivssim_t2r;
} oq_frame_result;

void   oq_default_opts(oq_opts* o);

/* a1: packed 4:2:0 / 4:4:4 frame (1 or 2 bytes per sample, little endian) -> 4:4:4 planes */
int    oq_unpack_frame(const uint8_t* packed, int32_t w, int32_t h, int32_t bytes_per_sample,
                       int32_t chroma_format, uint16_t* out444);

/* a15: compensated sums */
double oq_kbns(const double* x, size_t n);

/* a3 */
void   oq_gcd(const oq_pic* p0, const oq_pic* p1, const float unc[3], int32_t gcd_r2t[3]);

/* a4/a5/a10: one CPS direction. For every pixel of tst (+gcd) search ref; outputs are optional. */
void   oq_cps_dir(const oq_pic* tst, const oq_pic* ref, const int32_t gcd[3], int32_t sr,
                  const int32_t w[3], uint64_t* row_sse /* h*3 */, int8_t* argmin /* w*h */,
                  int32_t* minerr /* w*h */, uint16_t* scp /* 3*w*h */, int32_t nthreads);

/* a6: one direction's picture quality from its per-row SSE */
double oq_quality_from_rows(const uint64_t* row_sse, int32_t h, int32_t area, int32_t bd,
                            const double* ws_weights, const int32_t w_avg[3]);

/* a9 helpers */
void   oq_ws_weights(int32_t h, int32_t lat_deg, double* w, double* correction);
double oq_psnr_from_ssd(double ssd, int32_t area, int32_t bd);

/* a8/a9 */
void   oq_psnr(const oq_pic* p0, const oq_pic* p1, double out[3], uint64_t ssd[3]);
void   oq_wspsnr(const oq_pic* p0, const oq_pic* p1, int32_t lat_deg, double out[3]);

/* a11/a12 */
void   oq_ssim_table(int32_t window, float table[11][11]);
double oq_ssim_plane(const uint16_t* t, const uint16_t* r, int32_t w, int32_t h, int32_t bd,
                     int32_t calc_l, int32_t window, int32_t nthreads);
void   oq_ssim(const oq_pic* t, const oq_pic* r, int32_t calc_l, int32_t window, int32_t nthreads, double out[3]);
/* a13 */
void   oq_downsample(const uint16_t* src, int32_t sw, int32_t sh, uint16_t* dst);
void   oq_msssim(const oq_pic* p0, const oq_pic* p1, int32_t window, int32_t nthreads, double out[3]);

/* the application's per-frame flow over all six metrics (xAppQMIV.cpp:661-751) */
void   oq_frame(const oq_pic* p0, const oq_pic* p1, const oq_opts* o, int32_t do_ssim, oq_frame_result* r);

/* masked variants (xIVPSNR.cpp:138-200, xGlobClrDiff.cpp:52-83, xPSNR.cpp:148) */
int32_t oq_count_nonzero(const uint16_t* m, int32_t w, int32_t h);
void   oq_gcd_masked(const oq_pic* p0, const oq_pic* p1, const uint16_t* mask, int32_t nnm, int32_t mask_bd,
                     const float unc[3], int32_t gcd_r2t[3]);
void   oq_psnr_masked(const oq_pic* p0, const oq_pic* p1, const uint16_t* mask, int32_t nnm, int32_t mask_bd,
                      const double* ws_weights, double ws_correction, double out[3]);
double oq_ivpsnr_masked(const oq_pic* p0, const oq_pic* p1, const uint16_t* mask, int32_t nnm, int32_t mask_bd,
                        const int32_t gcd_r2t[3], const oq_opts* o, const double* ws_weights,
                        double* r2t, double* t2r);

/* input-side operations: colour conversion (xColorSpaceSTD.cpp:195-272), range clip (xPixelOpsSTD.cpp:163-209) */
void    oq_color_matrix(int32_t space, int32_t to_ycbcr, int32_t m[3][3]);
void    oq_color_convert(const uint16_t* in, uint16_t* out, int32_t w, int32_t h, int32_t bd, int32_t space, int32_t to_ycbcr);
int64_t oq_range_clip(uint16_t* p, int32_t w, int32_t h, int32_t bd);

#ifdef __cplusplus
}
#endif
#endif
