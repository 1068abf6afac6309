/*
 * qmiv_gb300 — C ABI of the GB300 implementation of the QMIV metric path
 * (IV-PSNR, PSNR, WS-PSNR, SSIM, MS-SSIM, IV-SSIM; reference: jstankowski/ivpsnr,
 * libs/pmbb-ivqm).
 *
 * Plain pointers and sizes only. Every call returns a qmiv_status; nothing throws.
 * A handle is not thread-safe; several handles (one per host thread or stream) may be
 * used at once. The handle owns all device scratch, sized at qmiv_create for the
 * largest picture and batch it will see; the calc calls allocate nothing.
 *
 * Each entry point names the reference interface it replaces (file:line within the
 * reference project). Picture 0 / picture 1 are the application's two inputs
 * (-i0 / -i1 of apps/QMIV, read into m_PicInP[0] / m_PicInP[1]); every metric is
 * computed with the argument order the application uses (apps/QMIV/src/xAppQMIV.cpp:693-935).
 */
#ifndef QMIV_GB300_H
#define QMIV_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QMIV_ABI_VERSION 1

typedef enum qmiv_status {
  QMIV_OK             = 0,
  QMIV_BAD_ARG        = 1, /* null pointer, size out of range, stride < width, ... */
  QMIV_UNSUPPORTED    = 2, /* valid request this build does not implement (e.g. odd 4:2:0 sizes) */
  QMIV_CUDA_ERROR     = 3, /* a CUDA runtime call failed; qmiv_last_error() has the text */
  QMIV_DEVICE_TIMEOUT = 4, /* a bounded device-side wait gave up */
  QMIV_OUT_OF_MEMORY  = 5,
  QMIV_TOO_LARGE      = 6  /* picture or batch larger than the handle was created for */
} qmiv_status;

/* Metric selection bits (apps/QMIV/src/xAppQMIV.h:140-153, eMetric) */
enum {
  QMIV_M_PSNR   = 1u << 0,
  QMIV_M_WSPSNR = 1u << 1,
  QMIV_M_IVPSNR = 1u << 2,
  QMIV_M_SSIM   = 1u << 3,
  QMIV_M_MSSSIM = 1u << 4,
  QMIV_M_IVSSIM = 1u << 5,
  QMIV_M_ALL    = 0x3Fu
};

enum { QMIV_CF420 = 420, QMIV_CF444 = 444 };
enum { QMIV_SSIM_REF10 = 0 /* the reference's truncated 10x10 window */, QMIV_SSIM_GAUSS11 = 1 /* full 11x11 */ };

/* One picture: three planes of 8-bit or 16-bit samples (little endian), host or device.
 * For 4:2:0 the chroma planes are (width/2) x (height/2) and are upsampled by
 * nearest neighbour on the fly, as xSeq::xUnpackFrame does (libs/pmbb-core/src/xSeq.cpp:179-213).
 * For 4:4:4 the planes may be the reference's xPicP planes (xPic.h:18): pass the origin
 * pointers and the stride; the margin is not read (window reads clamp to the picture,
 * which equals the reference's edge-replicated margin). */
typedef struct qmiv_pic {
  const void* plane[3];    /* Y, Cb, Cr */
  int32_t     stride[3];   /* in samples */
  int32_t     width, height;
  int32_t     bitdepth;    /* 8..14; the sample type is set by sample_bytes */
  int32_t     sample_bytes;/* 1 (uint8) or 2 (uint16) */
  int32_t     chroma_format; /* QMIV_CF420 or QMIV_CF444 */
  int32_t     is_device;   /* 1: device pointers; 0: host pointers (copied by the call) */
} qmiv_pic;

/* Processor parameters (xCorrespPixelShift.h:28-45, xGlobClrDiff.h:17-25,
 * xWeightedSpherically.h:21, xPSNR.h:31, xWSPSNR.h:28). */
typedef struct qmiv_options {
  int32_t search_range;    /* default 2 */
  int32_t cmp_w_search[4]; /* default 4,1,1,0 */
  int32_t cmp_w_avg[4];    /* default 4,1,1,0 */
  float   unnoticeable[4]; /* default 0.01,0.01,0.01,0 */
  int32_t use_ws;          /* equirectangular weighting of the PSNR family (initWS) */
  int32_t lon_deg, lat_deg;/* default 360, 180 */
  int32_t fake_exact;      /* 1 (default): exact components report PSNR(SSD=1) as the application does */
  int32_t legacy_ws8;      /* setLegacyWS8bit (off by default, never set by the application) */
  int32_t ssim_window;     /* QMIV_SSIM_REF10 (default) or QMIV_SSIM_GAUSS11 */
  uint32_t scratch_metrics;/* metrics whose per-job device scratch qmiv_create reserves (default
                            * QMIV_M_ALL); the SSIM family needs shift-compensated pictures and the
                            * MS-SSIM pyramid for every job slot, so PSNR-only callers can skip it */
} qmiv_options;

/* Per-frame results. Per-component arrays hold Y, Cb, Cr (index 3 unused, 0). The *_pic
 * values are the application's 4:1:1 weighted per-picture values (xAppQMIV.h:245-251). */
typedef struct qmiv_frame_result {
  uint32_t metrics;        /* QMIV_M_* bits computed */
  int32_t  status;         /* device-side status of this frame (qmiv_status) */
  int32_t  gcd_r2t[4];     /* global colour difference, xGlobClrDiffProc::CalcGlobalColorDiff(P0,P1) */
  int32_t  exact[4];       /* component identical in both pictures */
  double   psnr[4], psnr_pic;
  double   wspsnr[4], wspsnr_pic;
  double   ivpsnr, ivpsnr_r2t, ivpsnr_t2r;
  uint64_t sse_r2t[4], sse_t2r[4]; /* exact CPS squared-error sums per component */
  double   ssim[4], ssim_pic;
  double   msssim[4], msssim_pic;
  double   ivssim, ivssim_r2t, ivssim_t2r;
} qmiv_frame_result;

/* Per-sequence averages (xMetricStat::calcAvgMetric, xAppQMIV.h:256-260). */
typedef struct qmiv_seq_result {
  int32_t  num_frames;
  uint32_t metrics;
  double   psnr[4], psnr_pic, wspsnr[4], wspsnr_pic, ivpsnr;
  double   ssim[4], ssim_pic, msssim[4], msssim_pic, ivssim;
} qmiv_seq_result;

/* One job of a batch: a picture pair plus the metrics to compute on it. Pictures of a
 * batch may differ in size, bit depth and chroma format; use_ws selects ERP weighting
 * per job (lat_deg from the options). Device pictures for qmiv_calc_batch, host pictures for
 * qmiv_calc_batch_host. */
typedef struct qmiv_job {
  qmiv_pic pic0, pic1;
  uint32_t metrics;
  int32_t  use_ws;
  /* optional device outputs of the shift-compensated pictures (4:4:4 uint16, stride in
   * samples; null to skip): scp0 is built from picture 0, scp1 from picture 1 */
  uint16_t* scp0[3];
  uint16_t* scp1[3];
  int32_t   scp_stride;
} qmiv_job;

typedef struct qmiv_handle qmiv_handle;
typedef struct CUstream_st* qmiv_stream; /* a cudaStream_t; 0 = legacy default stream */

/* --- version / errors ------------------------------------------------------------- */
int32_t     qmiv_abi_version(void);
const char* qmiv_status_str(qmiv_status s);
const char* qmiv_last_error(void); /* thread-local text of the last failure */

/* --- processors: create/destroy ------------------------------------------------------
 * Replaces the processor set-up of apps/QMIV/src/xAppQMIV.cpp:593-650 (xIVPSNR / xSSIM /
 * xIVSSIM ::create, setSearchRange, setCmpWeights*, setUnntcbCoef, initWS, initRowBuffers,
 * initThreadPool). max_jobs bounds qmiv_calc_batch. */
void        qmiv_default_options(qmiv_options* opt);
qmiv_status qmiv_create(qmiv_handle** out, const qmiv_options* opt, int32_t max_width, int32_t max_height,
                        int32_t max_jobs);
qmiv_status qmiv_destroy(qmiv_handle* h);
qmiv_status qmiv_set_options(qmiv_handle* h, const qmiv_options* opt);

/* --- per frame -----------------------------------------------------------------------
 * All metrics of one picture pair in one call: replaces the per-frame body of
 * xAppQMIV::processAllFrames (xAppQMIV.cpp:661-751): GCD (:693-697), SCP (:703), and
 * calcFrame____PSNR / __WSPSNR / __IVPSNR / ____SSIM / __MSSSIM / __IVSSIM (:831-935).
 * Enqueued on `stream`; returns once the results are in *out (synchronous, like the
 * reference's calcPic* calls). The frame is also added to the sequence statistics. */
qmiv_status qmiv_calc_frame(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, uint32_t metrics,
                            qmiv_frame_result* out, qmiv_stream stream);

/* Masked form: xPSNR::calcPicPSNRM (xPSNR.cpp:42), xWSPSNR::calcPicWSPSNRM (xWSPSNR.cpp:61),
 * xIVPSNRM::calcPicIVPSNRM (xIVPSNR.cpp:138-200) and xGlobClrDiff::CalcGlobalColorDiffM
 * (xGlobClrDiff.cpp:52-83), as the application runs them with -im (xAppQMIV.cpp:693-695,
 * 831-893). The mask is one luma-resolution plane (width x height of the pictures, its own bit
 * depth) weighting all three components; mask 0 excludes a pixel as a tested pixel and as a
 * search candidate. metrics: any of QMIV_M_PSNR, QMIV_M_WSPSNR, QMIV_M_IVPSNR; gcd_r2t holds the
 * masked GCD. Synchronous; the frame is added to the sequence statistics. */
typedef struct qmiv_mask {
  const void* plane;
  int32_t     stride;       /* in samples */
  int32_t     bitdepth;     /* the mask's peak is 2^bitdepth - 1 */
  int32_t     sample_bytes; /* 1 or 2 */
  int32_t     is_device;
} qmiv_mask;
qmiv_status qmiv_calc_frame_masked(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, const qmiv_mask* mask,
                                   uint32_t metrics, qmiv_frame_result* out, qmiv_stream stream);

/* Batched form: n jobs of mixed sizes in one launch sequence on `stream`, asynchronous.
 * results (n entries) must be device memory or host memory the device can write
 * (cudaHostAlloc'd); they are valid after the stream synchronises. Frames are not added
 * to the sequence statistics. */
qmiv_status qmiv_calc_batch(qmiv_handle* h, const qmiv_job* jobs, int32_t n, qmiv_frame_result* results,
                            qmiv_stream stream);

/* Batched form for host pictures (the pictures of every job in host memory, page-locked for the
 * copies to overlap): the handle uploads the jobs in consecutive groups of at most group_bytes
 * of packed planes (0: a sixteenth of the batch, and a quarter of that for the last eighth of the
 * batch, whose measurement no upload hides; never less than the largest job) into two device
 * buffers it owns, on an upload stream of its own, and measures each group on `stream` as
 * qmiv_calc_batch does while the next group uploads. Asynchronous: returns once everything is
 * enqueued; the host pictures must stay unchanged until `stream` synchronises, after which the
 * results (device memory, n entries) are valid. Groups hold at most max_jobs jobs. No reference
 * counterpart: it replaces the application's read-then-measure loop over many pictures. */
qmiv_status qmiv_calc_batch_host(qmiv_handle* h, const qmiv_job* jobs, int32_t n, qmiv_frame_result* results,
                                 size_t group_bytes, qmiv_stream stream);

/* A batch captured once as a CUDA graph and replayed: for a fixed set of device pictures whose
 * contents change between replays (video frames decoded into the same buffers). No
 * counterpart in the reference. create runs the batch once, then records its launches on
 * `stream` (a created stream, not the legacy default stream) with private copies of the job
 * tables and TMA descriptors; launch replays them on any stream. The graph uses the handle's
 * scratch: replays and other calls on the handle must not overlap (same stream or
 * serialised), and the handle must outlive the graph. Results land in `results` as for
 * qmiv_calc_batch. */
typedef struct qmiv_graph qmiv_graph;
qmiv_status qmiv_batch_graph_create(qmiv_handle* h, const qmiv_job* jobs, int32_t n, qmiv_frame_result* results,
                                    qmiv_stream stream, qmiv_graph** out);
qmiv_status qmiv_batch_graph_launch(qmiv_graph* g, qmiv_stream stream);
qmiv_status qmiv_batch_graph_destroy(qmiv_graph* g);

/* --- fine-grained calls (each synchronous; for the C++ processor shim) --------------- */
/* xGlobClrDiffProc::CalcGlobalColorDiff(P0, P1) (xGlobClrDiff.h:41 -> xGlobClrDiff.cpp:15) */
qmiv_status qmiv_gcd(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, int32_t gcd_r2t[4],
                     qmiv_stream stream);
/* xPSNR::calcPicPSNR (xPSNR.cpp:17) and xWSPSNR::calcPicWSPSNR (xWSPSNR.cpp:17) */
qmiv_status qmiv_psnr(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, double psnr[4],
                      double wspsnr[4], qmiv_stream stream);
/* PSNR and GCD_R2T of one pair of device pictures with no handle and no allocation. No
 * counterpart in the reference: it exists for callers that cannot allocate device memory
 * when they measure, such as code running inside an allocator or memory-pool callback,
 * where an allocation could re-enter the allocator, or a process whose device memory is
 * all handed to one caching allocator up front, and that have nowhere to keep a handle.
 * It runs a variant of the statistics kernel whose scratch (per-row sums, the block counter
 * and the result) is one static device array of about 385 KiB; pictures taller than 8192
 * rows or wider than 65536 samples are rejected with QMIV_TOO_LARGE, host pictures with
 * QMIV_BAD_ARG. opt may be null
 * (defaults); it supplies unnoticeable, cmp_w_avg and fake_exact. Fills out->psnr,
 * psnr_pic, gcd_r2t and exact; every other field is 0. Synchronous on `stream`.
 * The first call on each device looks up the static array's address. All callers on a
 * device share the one array: calls that overlap in time, from other threads or on other
 * streams, race and must be serialised. */
qmiv_status qmiv_psnr_static(const qmiv_pic* pic0, const qmiv_pic* pic1, const qmiv_options* opt,
                             qmiv_frame_result* out, qmiv_stream stream);
/* xIVPSNR::calcPicIVPSNR(Tst=P0, Ref=P1, GCD) (xIVPSNR.cpp:32-56); gcd_r2t may be null (computed) */
qmiv_status qmiv_ivpsnr(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, const int32_t* gcd_r2t,
                        double* ivpsnr, double* r2t, double* t2r, qmiv_stream stream);
/* xShftCompPic::GenShftCompPics(&SCP1, &SCP0, &P1, &P0, GCD) (xShftCompPic.cpp:12-20); outputs are
 * host or device 4:4:4 uint16 planes per scp_is_device */
qmiv_status qmiv_scp(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, const int32_t* gcd_r2t,
                     uint16_t* scp0[3], uint16_t* scp1[3], int32_t scp_stride, int32_t scp_is_device,
                     qmiv_stream stream);
/* The corresponding-pixel search itself, pixel by pixel: for every pixel of both directions the
 * window index (dy + B)(2B + 1) + (dx + B) of the candidate that
 * xCorrespPixelShift::xFindBestPixelWithinBlock returns (xCorrespPixelShift.cpp:48-85, the first
 * strict minimum in row-major order; R2T searches picture 1 for picture 0 + GCD, T2R picture 0
 * for picture 1 - GCD), as int16 maps of width x height with row pitch map_stride (host or device
 * per map_is_device). row_sse (host, may be null) receives the per-row squared errors at the
 * argmin, [2][height][3] for R2T then T2R and Y, Cb, Cr (xCorrespPixelShift::xCalcDistAsymmetricRow,
 * xCorrespPixelShift.cpp:20-46). gcd_r2t may be null (computed). Synchronous. Host outputs use a
 * device buffer of 4 * max_width * max_height bytes that the handle allocates on first use. */
qmiv_status qmiv_cps_maps(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, const int32_t* gcd_r2t,
                          int16_t* map_r2t, int16_t* map_t2r, int32_t map_stride, int32_t map_is_device,
                          uint64_t* row_sse, qmiv_stream stream);
/* xSSIM::calcPicSSIM(Tst, Ref, CalcL) (xSSIM.cpp:54) on any two pictures (e.g. P0 and SCP1) */
qmiv_status qmiv_ssim(qmiv_handle* h, const qmiv_pic* tst, const qmiv_pic* ref, int32_t calc_l, double ssim[4],
                      qmiv_stream stream);
/* xSSIM::calcPicMSSSIM (xSSIM.cpp:67-87) */
qmiv_status qmiv_msssim(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, double msssim[4],
                        qmiv_stream stream);
/* xIVSSIM::calcPicIVSSIM(P0, P1, SCP0, SCP1) (xSSIM.cpp:192-210), building the SCPs itself */
qmiv_status qmiv_ivssim(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, const int32_t* gcd_r2t,
                        double* ivssim, double* r2t, double* t2r, qmiv_stream stream);

/* --- differentiable IV-PSNR error and IV-SSIM ------------------------------------------
 * No counterpart in the reference (which takes integer samples and has no gradients). Inputs
 * are n pairs of FP32 4:4:4 pictures with values in [0, 1] (Max = 1), device memory laid out
 * [n][3][height][width], tst the picture being optimised and ref fixed. The reference's
 * definitions carry over without integer rounding (opt: search_range 1..4, cmp_w_search,
 * unnoticeable, ssim_window; null = defaults):
 *   GCD_c = clip(mean(ref_c - tst_c), +-unnoticeable_c)                          (xGlobClrDiff.cpp:15-48)
 *   direction 0 (R2T): each tested pixel + GCD searched in ref, first strict minimum of
 *     sum_c w_c d_c^2 in row-major order, borders clamped; SSE_c = sum of squared errors at the
 *     argmin (xIVPSNR.cpp:62-95); SSIM_c = SSIM(ref_c, SCP0_c), SCP0 = clip(tst[argmin T2R] + GCD, 0, 1)
 *   direction 1 (T2R): each ref pixel - GCD searched in tst; SSIM_c = SSIM(tst_c, SCP1_c),
 *     SCP1 = clip(ref[argmin R2T] - GCD, 0, 1)                                      (xSSIM.cpp:166-190)
 * so IV-PSNR = min over directions of the weighted 10 log10(W H / SSE_c) and IV-SSIM = min over
 * directions of the weighted SSIM_c, both formed by the caller from sse[n][2][3] and
 * ssim[n][2][3] (device FP64). Gradients: the argmin carries none (it is piecewise constant);
 * errors and SCP samples route to the pixel they were read from; clips pass gradient on their
 * closed interval; GCD contributes -1/(W H) per pixel while it is not clipped.
 * The workspace (device, 256-byte aligned, qmiv_loss_workspace_size bytes) is the caller's and
 * carries the forward state (GCD, argmin maps, SCP planes) to the backward call, which must
 * see the same inputs and options. g_sse and g_ssim (device FP64, [n][2][3]) are the upstream
 * gradients; g_tst (device FP32, like tst) receives d loss / d tst. Asynchronous on stream. */
qmiv_status qmiv_loss_workspace_size(int32_t n, int32_t width, int32_t height, const qmiv_options* opt,
                                     size_t* bytes);
qmiv_status qmiv_loss_forward(const float* tst, const float* ref, int32_t n, int32_t width, int32_t height,
                              const qmiv_options* opt, void* workspace, size_t workspace_bytes, double* sse,
                              double* ssim, qmiv_stream stream);
qmiv_status qmiv_loss_backward(const float* tst, const float* ref, int32_t n, int32_t width, int32_t height,
                               const qmiv_options* opt, void* workspace, size_t workspace_bytes,
                               const double* g_sse, const double* g_ssim, float* g_tst, qmiv_stream stream);

/* --- input side ------------------------------------------------------------------------
 * Range check and concealment (xPixelOps::CheckIfInRange / ClipToRange, libs/pmbb-core/src/
 * xPixelOpsSTD.cpp:163-209, as xAppQMIV::validateFrames applies them, apps/QMIV/src/
 * xAppQMIV.cpp:753-770): counts the samples of each component above 2^bitdepth - 1 in a device
 * picture; with conceal != 0 clips them in place (the planes must be writable). Synchronous. */
qmiv_status qmiv_check_range(const qmiv_pic* pic, int32_t conceal, int64_t out_of_range[3], qmiv_stream stream);
/* Fixed-point colour conversion of a device 4:4:4 picture (xColorSpace::ConvertRGB2YCbCr /
 * ConvertYCbCr2RGB, xColorSpaceSTD.cpp:195-272, as xAppQMIV::preprocessFrames uses it,
 * xAppQMIV.cpp:778-814): to_ycbcr 1 reads R, G, B planes and writes Y, Cb, Cr; 0 the reverse.
 * color_space: 0 BT.601, 1 BT.709, 2 SMPTE 240M, 3 BT.2020. dst: three device uint16 planes
 * with row pitch dst_stride (samples); they may be src's own planes (in place, as the application
 * converts) when src has 16-bit samples and dst_stride is its stride. Asynchronous on stream. */
qmiv_status qmiv_color_convert(const qmiv_pic* src, uint16_t* dst[3], int32_t dst_stride, int32_t to_ycbcr,
                               int32_t color_space, qmiv_stream stream);
/* Raw planar YUV files (xSeqBase, libs/pmbb-core/src/xSeq.cpp:179-250): 8-bit samples as bytes,
 * deeper ones as 16-bit little endian, chroma 420, 422 or 444. qmiv_yuv_read seeks frame,
 * reads it into pinned memory and uploads it on stream into one of two device buffers (frame
 * parity), returning a device qmiv_pic valid until the read of frame + 2; 4:2:2 chroma is
 * doubled horizontally on the device into 4:4:4 planes (UpsampleH), 4:2:0 stays native. */
typedef struct qmiv_yuv_reader qmiv_yuv_reader;
qmiv_status qmiv_yuv_open(qmiv_yuv_reader** out, const char* path, int32_t width, int32_t height, int32_t bitdepth,
                          int32_t chroma_format);
int64_t     qmiv_yuv_frames(const qmiv_yuv_reader* r);
qmiv_status qmiv_yuv_read(qmiv_yuv_reader* r, int64_t frame, qmiv_pic* out, qmiv_stream stream);
qmiv_status qmiv_yuv_close(qmiv_yuv_reader* r);

/* --- per sequence ----------------------------------------------------------------------
 * xMetricStat::calcAvgMetric (xAppQMIV.h:256-260): compensated mean over the frames passed
 * to qmiv_calc_frame since create or the last reset. */
qmiv_status qmiv_finish_sequence(qmiv_handle* h, qmiv_seq_result* out);
qmiv_status qmiv_reset_sequence(qmiv_handle* h);

/* --- introspection (tests, profiling) -------------------------------------------------- */
/* Number of kernels this handle has launched since creation. */
int64_t     qmiv_kernel_launches(const qmiv_handle* h);
/* CPS kernel variants (tile shape, search-window unrolling, key width): count, name, and
 * a per-handle override used by the autotuner and the tests (-1 restores the default
 * choice; a variant that does not fit a job falls back to the default for that job). */
int32_t     qmiv_cps_variant_count(void);
const char* qmiv_cps_variant_name(int32_t v);
qmiv_status qmiv_set_cps_variant(qmiv_handle* h, int32_t v);
/* Autotuner: times every compiled CPS variant that fits all IV-PSNR / IV-SSIM jobs of the batch
 * (reps timed runs each after one warm-up, CUDA events around the CPS launches) and keeps the
 * fastest as the handle's override. Runs the batch as qmiv_calc_batch does (results are
 * written). best_variant / best_ms (may be null) receive the choice and its CPS time. */
qmiv_status qmiv_autotune_cps(qmiv_handle* h, const qmiv_job* jobs, int32_t n, qmiv_frame_result* results,
                              int32_t reps, qmiv_stream stream, int32_t* best_variant, double* best_ms);
/* Test hook for the failure path of the bounded device-side waits (no counterpart in the
 * reference). With polls > 0 the first bulk-copy wait of every block of the TMA search kernels and
 * of the fused SSIM kernel polls, polls times, an mbarrier that no copy arrives on, gives up, and
 * takes the failure path: the block records QMIV_DEVICE_TIMEOUT in the frame's status, waits with
 * the full limit for its own copies in flight, and stops, so the call returns QMIV_DEVICE_TIMEOUT.
 * 0 restores normal waits; the handle stays usable. Only calls whose pictures the bulk copies can
 * stage (16-byte aligned device planes) reach these waits. */
qmiv_status qmiv_test_wait_timeout(qmiv_handle* h, uint32_t polls);
/* Per-kernel timing of the most recent calc call (CUDA events recorded on the call's
 * stream around each launch, when enabled). qmiv_kernel_times synchronises with those
 * events and returns up to max launches: names[i] (static strings) and ms[i]. */
qmiv_status qmiv_set_profiling(qmiv_handle* h, int32_t enable);
int32_t     qmiv_kernel_times(qmiv_handle* h, const char** names, double* ms, int32_t max);

#ifdef __cplusplus
}
#endif
#endif
