// Host side of the C ABI (include/qmiv_gb300.h): handles, argument validation, device
// scratch, job descriptors and launch sequencing. No host threads; every call is enqueued
// on the caller's stream. Calls on one handle must be issued on one stream (or serialised):
// they share the handle's device job tables.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <condition_variable>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <unistd.h>

#include <cuda.h>
#include <cuda_runtime.h>

#include "qmiv_internal.h"
#include "qmiv_io.h"
#include "qmiv_loss.h"
#include "qmiv_masked.h"
#include "qmiv_ssim.h"

using namespace qmiv;

namespace {

// All compiled CPS variants: index 0 is the generic kernel.
const std::vector<CpsVariant>& variants()
{
  static std::vector<CpsVariant> v = [] {
    std::vector<CpsVariant> out;
    int n = 0;
    const CpsVariant* a = cps_variants_staged(&n);
    out.insert(out.end(), a, a + n);
    a = cps_variants_tma(&n);
    out.insert(out.end(), a, a + n);
    return out;
  }();
  return v;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn()
{
  static EncodeTiledFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
       q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return (EncodeTiledFn)f;
  }();
  return fn;
}

thread_local std::string g_last_error;

qmiv_status fail(qmiv_status s, const char* fmt, ...)
{
  char buf[512];
  va_list ap; va_start(ap, fmt); vsnprintf(buf, sizeof(buf), fmt, ap); va_end(ap);
  g_last_error = buf;
  return s;
}

#define CUDA_TRY(expr)                                                                           \
  do {                                                                                           \
    cudaError_t e_ = (expr);                                                                     \
    if(e_ != cudaSuccess) return fail(QMIV_CUDA_ERROR, "%s: %s", #expr, cudaGetErrorString(e_)); \
  } while(0)

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

constexpr uint32_t kSsimMetrics = QMIV_M_SSIM | QMIV_M_MSSSIM | QMIV_M_IVSSIM;
constexpr int kSsimJobsPerFrame = 24;  // 3 SSIM + 15 MS-SSIM + 6 IV-SSIM
constexpr int kPyrStepsPerFrame = 6;   // per pyramid level: 2 pictures x 3 components

// Device slot for one job: scratch rows and scalars, tensor maps, SSIM scratch.
struct Slot {
  int64_t* stat_rows = nullptr;           // [max_h][6]
  unsigned long long* cps_rows = nullptr; // [2][max_h][3]
  JobScalars* sc = nullptr;
  // encoded tensor-map sets of the last kTmapSets picture layouts this slot ran (up to
  // kTmapMaps x 128 B each, device: six for the CPS kernel, twelve for the fused SSIM kernel),
  // so that a batch repeated over alternating buffers finds its maps without a copy
  static constexpr int kTmapSets = 16, kTmapMaps = 12, kKey = 32;
  uint8_t* d_tmaps = nullptr;
  uint64_t tmap_key[kTmapSets][kKey] = { { 0 } };
  uint64_t tmap_stamp[kTmapSets] = { 0 };
  bool tmap_valid[kTmapSets] = { false };
  uint16_t* scp = nullptr;                // 2 pictures x 3 planes x max_w*max_h (IV-SSIM)
  uint16_t* pyr = nullptr;                // MS-SSIM levels 1..4, 2 pictures x 3 components
  float* partial = nullptr;               // SSIM per-tile row sums of all the frame's SSIM jobs
  double* vals = nullptr;                 // kSsimVals picture means
};

struct SeqAcc { std::vector<double> v[18]; };

// Per-call tables uploaded to the device in one copy, from a ring of pinned buffers so that
// a table is never rewritten while an earlier call's copy of it may still be pending.
struct CallTables {
  size_t jobs_off, ssim_off, pyr_off, frames_off, bytes;
};

}  // namespace

struct qmiv_handle {
  qmiv_options opt;
  Params params;
  int max_w = 0, max_h = 0, max_jobs = 0;
  int device = 0, num_sms = 0;
  int cps_variant_override = -1;
  uint32_t test_wait_polls = 0;           // qmiv_test_wait_timeout
  std::vector<Slot> slots;
  void* slot_mem = nullptr;
  void* ssim_mem = nullptr;
  size_t slot_partial_floats = 0;
  qmiv_frame_result* d_results = nullptr;
  qmiv_frame_result* h_results = nullptr; // pinned
  // call tables
  CallTables tab;
  uint8_t* d_tab = nullptr;
  static constexpr int kRing = 4;
  uint8_t* h_tab[kRing] = { nullptr };      // page-locked, mapped
  uint8_t* h_tab_dev[kRing] = { nullptr };  // their device addresses
  cudaEvent_t tab_ev[kRing] = { nullptr };
  bool tab_used[kRing] = { false };
  int tab_next = 0;
  // host-side working copies of the tables
  std::vector<DevJob> jobs;
  std::vector<SsimJob> sjobs;
  std::vector<SsimQuadJob> qjobs;         // fused full-resolution SSIM family (IV-SSIM frames)
  std::vector<PyrStep> steps[4];
  std::vector<SsimFrame> frames;
  // staging for host pictures (2 pictures, planar, up to uint16 4:4:4)
  uint16_t* d_stage[2] = { nullptr, nullptr };
  // qmiv_calc_batch_host: its upload stream, two device group buffers and their events
  cudaStream_t up_stream = nullptr;
  uint8_t* d_up[2] = { nullptr, nullptr };
  size_t up_cap = 0;
  cudaEvent_t up_done[2] = { nullptr, nullptr }, up_free[2] = { nullptr, nullptr };
  bool up_recorded[2] = { false, false };
  // pinned staging ring of encoded tensor maps (6 per entry), so that re-encoding a job's maps
  // never waits for the stream: an entry is rewritten only after its copy has run
  uint8_t* h_tmaps = nullptr;
  std::vector<cudaEvent_t> tmap_ev;
  std::vector<char> tmap_used;
  int tmap_next = 0;
  uint64_t tmap_clock = 0;                // LRU stamps of the slots' tensor-map sets
  // masked frames: per-row sums, counters / count / GCD, host-mask staging
  int64_t* mask_rows = nullptr;
  uint8_t* mask_small = nullptr;
  uint16_t* mask_stage = nullptr;
  // qmiv_cps_maps with host outputs: both directions' argmin maps (sized on first use)
  int16_t* d_maps = nullptr;
  std::map<std::pair<int, int>, std::pair<double*, double>> ws_cache;
  SeqAcc seq;
  int64_t launches = 0;
  struct Prof { cudaEvent_t a = nullptr, b = nullptr; const char* name = ""; };
  bool profiling = false;
  std::vector<Prof> prof;
  int prof_n = 0;
};

namespace {

int pow2_log2(uint64_t v) { if(v == 0 || (v & (v - 1))) return -1; int l = 0; while((1ull << l) < v) l++; return l; }

// One past the largest window index: (2B+1)^2 for the row-major numbering, or 2B*P + 2B + 1
// with the power-of-two row pitch P >= 2B+1 of the TMA kernels (the larger of the two).
uint64_t window_index_bound(int sr)
{
  uint64_t pitch = 1;
  while(pitch < (uint64_t)(2 * sr + 1)) pitch <<= 1;
  const uint64_t a = (uint64_t)(2 * sr + 1) * (2 * sr + 1), b = 2ull * sr * pitch + 2ull * sr + 1;
  return a > b ? a : b;
}
int32_t rne_f32(float v) { return (int32_t)std::nearbyint(v); }

void derive_params(qmiv_handle* h)
{
  const qmiv_options& o = h->opt;
  Params& p = h->params;
  std::memset(&p, 0, sizeof(p));
  p.sr = o.search_range;
  for(int c = 0; c < 3; c++) { p.w_search[c] = o.cmp_w_search[c]; p.w_avg[c] = o.cmp_w_avg[c]; }
  for(int bd = 0; bd <= 14; bd++)
    for(int c = 0; c < 3; c++)
    { // xGlobClrDiff.cpp:21: xRoundFltToInt32(CmpUnntcbCoef * (flt32)MaxValue)
      const float mx = (float)((1 << bd) - 1);
      p.maxdiff_for_bd[bd][c] = rne_f32(o.unnoticeable[c] * mx);
    }
  p.fake_exact = o.fake_exact;
  p.legacy_ws8 = o.legacy_ws8;
  // CPS key: M*E + k with (s*d)^2 = M*w0*d^2, s = w0*m, M = w0*m^2, and M above every window
  // index k; the TMA kernels number the window with a power-of-two row pitch, so k < N
  const uint64_t N = window_index_bound(o.search_range);
  const uint64_t w0 = (uint64_t)std::max(o.cmp_w_search[0], 1);
  uint64_t m = 1;
  while(w0 * m * m < N) m <<= 1;
  p.key_m = (uint32_t)(w0 * m * m);
  p.key_m_log2 = pow2_log2(p.key_m);
  p.luma_scale = (int32_t)(w0 * m);
  p.luma_scale_log2 = pow2_log2((uint64_t)p.luma_scale);
  p.one = 1;
  p.first_wait_test_polls = h->test_wait_polls;
}

// Does the 32-bit packed key hold for this bit depth? The 32-bit TMA search evaluates keys
// relative to the tested sample's square in signed 32-bit arithmetic, so the key must stay
// below 2^31 (with room for the window-index offset) and the scaled samples' squares too.
bool key32_ok(const qmiv_handle* h, int bd)
{
  const Params& p = h->params;
  int md = 0;
  for(int c = 0; c < 3; c++) md = std::max(md, p.maxdiff_for_bd[bd][c]);
  const uint64_t D = (uint64_t)((1 << bd) - 1) + (uint64_t)md;
  const uint64_t wsum = (uint64_t)p.w_search[0] + p.w_search[1] + p.w_search[2];
  const uint64_t N = window_index_bound(p.sr);
  const uint64_t kmax = (uint64_t)p.key_m * wsum * D * D + N;
  return kmax + 64 < (1ull << 31) && (uint64_t)p.luma_scale * D < 46340ull;
}

// Can the TMA kernels stage this job? 16-byte aligned planes and row pitches.
bool tma_ok(const DevJob& j)
{
  if(!j.cshift || !encode_fn()) return false;
  for(int c = 0; c < 3; c++)
  {
    if((((uintptr_t)j.p0[c]) | ((uintptr_t)j.p1[c])) & 15) return false;
    if(((j.stride0[c] * j.sbytes) | (j.stride1[c] * j.sbytes)) & 15) return false;
  }
  return true;
}

// Can compiled variant v run job j? (its search range, key width, staging kind and sample size)
bool cps_variant_fits(const qmiv_handle* h, const DevJob& j, int v)
{
  const auto& V = variants();
  if(v <= 0 || v >= (int)V.size()) return false;
  const int sr = h->params.sr;
  if(!j.cshift || h->opt.cmp_w_search[0] < 1 || sr < 1 || sr > 4) return false;
  const CpsVariant& c = V[v];
  if(c.sr != sr || c.key64 != !key32_ok(h, j.bd)) return false;
  if(c.kind == 2 && (!tma_ok(j) || c.sbytes != j.sbytes)) return false;
  return c.kind != 0;
}

int pick_cps_variant(const qmiv_handle* h, const DevJob& j)
{
  const auto& V = variants();
  const int sr = h->params.sr;
  if(!j.cshift || h->opt.cmp_w_search[0] < 1 || sr < 1 || sr > 4) return 0; // generic
  if(h->cps_variant_override == 0) return 0;
  if(cps_variant_fits(h, j, h->cps_variant_override)) return h->cps_variant_override;
  // default: at search range <= 2 the TMA kernel with 16-row strips and 4 warps (more resident
  // blocks), above it the one with 32-row strips and 8 warps (measured faster at range 4 on
  // 8K frames); else the staged-load kernel
  const char* first = sr <= 2 ? "_q4_w2" : "_q4_w4";
  const char* second = sr <= 2 ? "_q4_w4" : "_q4_w2";
  for(const char* shape : { first, second })
    for(int v = 1; v < (int)V.size(); v++)
      if(cps_variant_fits(h, j, v) && V[v].kind == 2 && std::strstr(V[v].name, shape)) return v;
  for(int v = 1; v < (int)V.size(); v++)
    if(cps_variant_fits(h, j, v) && V[v].kind == 1 && std::strstr(V[v].name, "rpt8_nwg2")) return v;
  return 0;
}

qmiv_status check_pic(const qmiv_handle* h, const qmiv_pic* p, const char* name)
{
  if(!p) return fail(QMIV_BAD_ARG, "%s is null", name);
  if(p->width < 1 || p->height < 1) return fail(QMIV_BAD_ARG, "%s: size %dx%d", name, p->width, p->height);
  if(p->width > h->max_w || p->height > h->max_h)
    return fail(QMIV_TOO_LARGE, "%s: %dx%d exceeds the handle's %dx%d", name, p->width, p->height, h->max_w, h->max_h);
  if(p->bitdepth < 1 || p->bitdepth > 14) return fail(QMIV_BAD_ARG, "%s: bit depth %d (1..14)", name, p->bitdepth);
  if(p->sample_bytes != 1 && p->sample_bytes != 2) return fail(QMIV_BAD_ARG, "%s: sample_bytes %d", name, p->sample_bytes);
  if(p->sample_bytes == 1 && p->bitdepth > 8) return fail(QMIV_BAD_ARG, "%s: %d-bit samples in 8-bit storage", name, p->bitdepth);
  if(p->chroma_format != QMIV_CF420 && p->chroma_format != QMIV_CF444)
    return fail(QMIV_UNSUPPORTED, "%s: chroma format %d", name, p->chroma_format);
  if(p->chroma_format == QMIV_CF420 && ((p->width | p->height) & 1))
    return fail(QMIV_UNSUPPORTED, "%s: 4:2:0 needs even sizes (%dx%d)", name, p->width, p->height);
  for(int c = 0; c < 3; c++)
  {
    if(!p->plane[c]) return fail(QMIV_BAD_ARG, "%s: plane %d is null", name, c);
    const int w = (c && p->chroma_format == QMIV_CF420) ? p->width / 2 : p->width;
    if(p->stride[c] < w) return fail(QMIV_BAD_ARG, "%s: stride[%d]=%d < width %d", name, c, p->stride[c], w);
  }
  return QMIV_OK;
}

qmiv_status check_pair(const qmiv_handle* h, const qmiv_pic* a, const qmiv_pic* b)
{
  qmiv_status s;
  if((s = check_pic(h, a, "pic0")) != QMIV_OK) return s;
  if((s = check_pic(h, b, "pic1")) != QMIV_OK) return s;
  if(a->width != b->width || a->height != b->height || a->bitdepth != b->bitdepth ||
     a->chroma_format != b->chroma_format || a->sample_bytes != b->sample_bytes || a->is_device != b->is_device)
    return fail(QMIV_BAD_ARG, "pic0 and pic1 differ in size, bit depth, format, sample size or location");
  return QMIV_OK;
}

qmiv_status check_metrics(const qmiv_handle* h, uint32_t metrics, int W, int H)
{
  if(metrics & ~QMIV_M_ALL) return fail(QMIV_BAD_ARG, "metrics 0x%x", metrics);
  if(metrics & ~h->opt.scratch_metrics)
    return fail(QMIV_UNSUPPORTED, "metrics 0x%x need scratch the handle did not reserve (scratch_metrics 0x%x)",
                metrics, h->opt.scratch_metrics);
  if((metrics & QMIV_M_MSSSIM) && (W < 16 || H < 16))
    return fail(QMIV_UNSUPPORTED, "MS-SSIM needs at least 16x16 (four halvings), got %dx%d", W, H);
  return QMIV_OK;
}

qmiv_status ws_weights(qmiv_handle* h, int H, const double** d_w, double* corr)
{
  const auto key = std::make_pair(H, h->opt.lat_deg);
  auto it = h->ws_cache.find(key);
  if(it == h->ws_cache.end())
  { // xWeightedSpherically::initWS (xWeightedSpherically.cpp:13-29), FP64 on the host
    std::vector<double> w(H);
    const double he = 180.0 * (double)H / (double)h->opt.lat_deg;
    const double off = (he - H) / 2.0;
    const double pi = 3.14159265358979323846;
    for(int y = 0; y < H; y++) w[y] = std::cos((y + off - (he / 2 - 0.5)) * pi / he);
    double s = w[0], c = 0.0; // xKBNS::Accumulate
    for(int y = 1; y < H; y++)
    {
      const double t = s + w[y];
      if(std::fabs(s) >= std::fabs(w[y])) c += ((s - t) + w[y]); else c += ((w[y] - t) + s);
      s = t;
    }
    double* d = nullptr;
    CUDA_TRY(cudaMalloc(&d, sizeof(double) * H));
    CUDA_TRY(cudaMemcpy(d, w.data(), sizeof(double) * H, cudaMemcpyHostToDevice));
    it = h->ws_cache.emplace(key, std::make_pair(d, H / (s + c))).first;
  }
  *d_w = it->second.first;
  *corr = it->second.second;
  return QMIV_OK;
}

// Fill a job from two validated device pictures.
void fill_job(qmiv_handle* h, DevJob& j, const qmiv_pic* a, const qmiv_pic* b, uint32_t metrics, int slot)
{
  std::memset(&j, 0, sizeof(j));
  for(int c = 0; c < 3; c++)
  {
    j.p0[c] = a->plane[c]; j.p1[c] = b->plane[c];
    j.stride0[c] = a->stride[c]; j.stride1[c] = b->stride[c];
  }
  j.W = a->width; j.H = a->height; j.bd = a->bitdepth; j.sbytes = a->sample_bytes;
  j.cshift = a->chroma_format == QMIV_CF420 ? 1 : 0;
  j.metrics = metrics;
  j.slot = slot;
  j.stat_rows = h->slots[slot].stat_rows;
  j.cps_rows = h->slots[slot].cps_rows;
  j.sc = h->slots[slot].sc;
  j.result = h->d_results + slot;
}

// Grid decomposition of a set of jobs for the stats and CPS kernels.
void plan_grid(qmiv_handle* h, DevJob* jobs, int n, const std::vector<int>& variant)
{
  int sbase = 0;
  long long strips_total = 0;
  for(int i = 0; i < n; i++)
  {
    DevJob& j = jobs[i];
    j.stat_blocks = ((j.H + 1) / 2 + 7) / 8; // 8 row pairs (one per warp) per block
    j.stat_base = sbase;
    sbase += j.stat_blocks;
    const int rows = variants()[variant[i]].rows;
    j.cps_strips = (j.H + rows - 1) / rows;
    strips_total += j.cps_strips;
  }
  const long long target = 8ll * h->num_sms;
  for(int i = 0; i < n; i++)
  {
    DevJob& j = jobs[i];
    if(variant[i] == 0)
    { // generic: 32 x 4 pixel tiles
      j.cps_segs = (j.W + 31) / 32;
      j.cps_seg_chunks = 1;
      continue;
    }
    const int nchunks = (j.W + 63) / 64;
    int segs = (int)std::min<long long>(nchunks, std::max<long long>(1, (target + strips_total - 1) / std::max(1ll, strips_total)));
    // per-thread 32-bit SSE accumulators: 2 pixels per chunk, each < (Max + maxdiff)^2
    int md = 0; for(int c = 0; c < 3; c++) md = std::max(md, h->params.maxdiff_for_bd[j.bd][c]);
    const double D = (double)((1 << j.bd) - 1 + md);
    const int max_chunks = std::max(1, (int)std::floor(4294967295.0 / (2.0 * D * D)));
    int seg_chunks = (nchunks + segs - 1) / segs;
    if(seg_chunks > max_chunks) seg_chunks = max_chunks;
    // at most 16 chunks (1024 columns) per block: the last wave of a launch stays short
    if(seg_chunks > 16) seg_chunks = 16;
    j.cps_seg_chunks = seg_chunks;
    j.cps_segs = (nchunks + seg_chunks - 1) / seg_chunks;
  }
}

// Device bytes of a host picture packed as stage_pic lays it out.
size_t stage_bytes(const qmiv_pic* p)
{
  size_t off = 0;
  const int sb = p->sample_bytes;
  for(int c = 0; c < 3; c++)
  {
    const int w = (c && p->chroma_format == QMIV_CF420) ? p->width / 2 : p->width;
    const int hh = (c && p->chroma_format == QMIV_CF420) ? p->height / 2 : p->height;
    off = (off + 255) & ~(size_t)255;
    off += (size_t)(((w * sb + 15) & ~15)) * hh;
  }
  return (off + 255) & ~(size_t)255;
}

// Host picture -> packed device copy at base (same sample size, planes back to back and
// 256-byte aligned, rows padded to 16-byte multiples so that the TMA kernels can take them).
// A plane whose rows are contiguous on both sides goes as one linear copy, and planes stored
// back to back on both sides (a picture held as one Y-Cb-Cr buffer) as one copy: the copy
// engine pays a fixed cost per copy and moves short pitched rows well below its linear rate.
// The merged range is exactly the planes' bytes; if the runtime refuses it (the planes are
// separate page-locked allocations that happen to touch), the planes go one by one.
qmiv_status stage_pic(const qmiv_pic* src, uint8_t* base, qmiv_pic* dst, cudaStream_t st)
{
  *dst = *src;
  const int sb = src->sample_bytes;
  size_t off = 0;
  struct Run { const uint8_t* s; uint8_t* d; size_t bytes; };
  Run runs[3];
  int nr = 0;
  for(int c = 0; c < 3; c++)
  {
    const int w = (c && src->chroma_format == QMIV_CF420) ? src->width / 2 : src->width;
    const int hh = (c && src->chroma_format == QMIV_CF420) ? src->height / 2 : src->height;
    const int pitch = ((w * sb + 15) & ~15) / sb;
    off = (off + 255) & ~(size_t)255;
    const uint8_t* sp = static_cast<const uint8_t*>(src->plane[c]);
    if(src->stride[c] == w && pitch == w)
      runs[nr++] = { sp, base + off, (size_t)w * hh * sb };
    else
      CUDA_TRY(cudaMemcpy2DAsync(base + off, (size_t)pitch * sb, sp, (size_t)src->stride[c] * sb,
                                 (size_t)w * sb, hh, cudaMemcpyHostToDevice, st));
    dst->plane[c] = base + off;
    dst->stride[c] = pitch;
    off += (size_t)pitch * hh * sb;
  }
  int k = 0;
  while(k < nr)
  {
    int e = k;
    size_t bytes = runs[k].bytes;
    while(e + 1 < nr && runs[e + 1].s == runs[k].s + bytes && runs[e + 1].d == runs[k].d + bytes) bytes += runs[++e].bytes;
    if(e > k && cudaMemcpyAsync(runs[k].d, runs[k].s, bytes, cudaMemcpyHostToDevice, st) == cudaSuccess) { k = e + 1; continue; }
    if(e > k) (void)cudaGetLastError();  // refused merge: clear it and copy plane by plane
    for(int i = k; i <= e; i++) CUDA_TRY(cudaMemcpyAsync(runs[i].d, runs[i].s, runs[i].bytes, cudaMemcpyHostToDevice, st));
    k = e + 1;
  }
  dst->is_device = 1;
  return QMIV_OK;
}

qmiv_status upload_pic(qmiv_handle* h, const qmiv_pic* src, int idx, qmiv_pic* dst, cudaStream_t st)
{
  *dst = *src;
  if(src->is_device) return QMIV_OK;
  return stage_pic(src, reinterpret_cast<uint8_t*>(h->d_stage[idx]), dst, st);
}

cudaError_t prof_mark(qmiv_handle* h, const char* name, cudaStream_t st, bool begin)
{
  if(!h->profiling) return cudaSuccess;
  if(begin)
  {
    if(h->prof_n == (int)h->prof.size())
    {
      qmiv_handle::Prof p;
      cudaError_t e = cudaEventCreate(&p.a); if(e != cudaSuccess) return e;
      e = cudaEventCreate(&p.b); if(e != cudaSuccess) return e;
      h->prof.push_back(p);
    }
    h->prof[h->prof_n].name = name;
    return cudaEventRecord(h->prof[h->prof_n].a, st);
  }
  return cudaEventRecord(h->prof[h->prof_n++].b, st);
}

// One 2-D tensor map over a plane of `sb`-byte samples (no swizzle, zeros outside).
bool encode_plane(CUtensorMap* m, const void* base, int w, int hgt, int stride, int sb, uint32_t bw, uint32_t bh)
{
  EncodeTiledFn enc = encode_fn();
  if(!enc) return false;
  const cuuint64_t dims[2] = { (cuuint64_t)w, (cuuint64_t)hgt };
  const cuuint64_t strides[1] = { (cuuint64_t)stride * sb };
  const cuuint32_t box[2] = { bw, bh };
  const cuuint32_t estr[2] = { 1, 1 };
  return enc(m, sb == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, const_cast<void*>(base), dims,
             strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The slot's device copy of the tensor-map set identified by `key` (nmaps maps). A set seen
// before is reused; a new one is encoded by `encode` into a pinned staging entry and copied
// over the least recently used set. The copy is stream-ordered after every earlier launch of
// the handle, so no kernel still reads the set it overwrites.
template <typename Enc>
qmiv_status slot_tmaps(qmiv_handle* h, Slot& S, const uint64_t (&key)[Slot::kKey], int nmaps, Enc encode,
                       cudaStream_t st, const void** out)
{
  int e = -1, victim = 0;
  for(int t = 0; t < Slot::kTmapSets; t++)
  {
    if(S.tmap_valid[t] && std::memcmp(key, S.tmap_key[t], sizeof(key)) == 0) { e = t; break; }
    if(!S.tmap_valid[victim]) continue;
    if(!S.tmap_valid[t] || S.tmap_stamp[t] < S.tmap_stamp[victim]) victim = t;
  }
  S.tmap_stamp[e >= 0 ? e : victim] = ++h->tmap_clock;
  if(e < 0)
  {
    e = victim;
    const int nr = (int)h->tmap_ev.size();
    const int k = h->tmap_next;
    h->tmap_next = (k + 1) % nr;
    if(h->tmap_used[k]) CUDA_TRY(cudaEventSynchronize(h->tmap_ev[k]));
    CUtensorMap* maps = reinterpret_cast<CUtensorMap*>(h->h_tmaps + (size_t)k * Slot::kTmapMaps * sizeof(CUtensorMap));
    S.tmap_valid[e] = false;
    if(!encode(maps)) return fail(QMIV_CUDA_ERROR, "cuTensorMapEncodeTiled failed");
    CUDA_TRY(cudaMemcpyAsync(S.d_tmaps + (size_t)e * Slot::kTmapMaps * sizeof(CUtensorMap), maps,
                             (size_t)nmaps * sizeof(CUtensorMap), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaEventRecord(h->tmap_ev[k], st));
    h->tmap_used[k] = 1;
    std::memcpy(S.tmap_key[e], key, sizeof(key));
    S.tmap_valid[e] = true;
  }
  *out = S.d_tmaps + (size_t)e * Slot::kTmapMaps * sizeof(CUtensorMap);
  return QMIV_OK;
}

// Encode (or reuse) the six tensor maps a TMA variant reads for one job's planes.
qmiv_status ensure_tmaps(qmiv_handle* h, DevJob& j, const CpsVariant& v, cudaStream_t st)
{
  Slot& S = h->slots[j.slot];
  const int sb = j.sbytes, XA = 16 / sb, R = v.rows, SR = v.sr, CS = (SR + 1) / 2;
  const int fd = (R - 1 + SR) / 2;
  const uint32_t RW = 64 + 2 * XA, TH = R + 2 * SR, CRW = 32 + 2 * XA, CTH = fd + CS + 1;
  uint64_t key[Slot::kKey] = { 0 };
  key[0] = 1;  // CPS set
  for(int c = 0; c < 3; c++)
  {
    key[1 + c] = (uint64_t)(uintptr_t)j.p0[c]; key[4 + c] = (uint64_t)(uintptr_t)j.p1[c];
    key[7 + c] = ((uint64_t)(uint32_t)j.stride0[c] << 32) | (uint32_t)j.stride1[c];
  }
  key[10] = ((uint64_t)(uint32_t)j.W << 32) | (uint32_t)j.H;
  key[11] = ((uint64_t)RW << 48) | ((uint64_t)TH << 32) | ((uint64_t)CRW << 16) | CTH;
  key[12] = (uint64_t)sb;
  auto encode = [&](CUtensorMap* maps) {
    for(int pic = 0; pic < 2; pic++)
      for(int c = 0; c < 3; c++)
      {
        const void* base = pic == 0 ? j.p0[c] : j.p1[c];
        const int stride = pic == 0 ? j.stride0[c] : j.stride1[c];
        if(!encode_plane(&maps[pic * 3 + c], base, c ? j.W / 2 : j.W, c ? j.H / 2 : j.H, stride, sb, c ? CRW : RW, c ? CTH : TH))
          return false;
      }
    return true;
  };
  return slot_tmaps(h, S, key, 6, encode, st, &j.tmaps);
}

// Can a tensor map describe this plane? 16-byte aligned base and pitch, 8/16-bit samples.
bool plane_tma_ok(const SsimPlane& p)
{
  return p.ptr && (p.sbytes == 1 || p.sbytes == 2) && ((uintptr_t)p.ptr & 15) == 0 && ((size_t)p.stride * p.sbytes) % 16 == 0;
}

// Tensor maps of a frame's three fused-SSIM jobs (four planes each), or null maps for a frame
// whose planes a tensor map cannot describe (the kernel then stages them with plain loads).
qmiv_status ensure_quad_tmaps(qmiv_handle* h, Slot& S, SsimQuadJob* q, cudaStream_t st)
{
  bool ok = encode_fn() != nullptr;
  for(int c = 0; c < 3 && ok; c++)
    ok = plane_tma_ok(q[c].p0) && plane_tma_ok(q[c].p1) && plane_tma_ok(q[c].scp1) && plane_tma_ok(q[c].scp0) &&
         q[c].scp1.sbytes == 2 && q[c].scp1.shift == 0 && q[c].scp0.sbytes == 2 && q[c].scp0.shift == 0;
  if(!ok) { for(int c = 0; c < 3; c++) q[c].tmaps = nullptr; return QMIV_OK; }
  const int win = h->opt.ssim_window;
  uint64_t key[Slot::kKey] = { 0 };
  key[0] = 2;  // fused-SSIM set
  key[1] = ((uint64_t)(uint32_t)q[0].W << 32) | (uint32_t)q[0].H;
  key[2] = ((uint64_t)(uint32_t)win << 32) | ((uint32_t)q[0].p0.sbytes << 8);
  for(int c = 0; c < 3; c++)
  {
    const SsimPlane* pl[4] = { &q[c].p0, &q[c].p1, &q[c].scp1, &q[c].scp0 };
    for(int k = 0; k < 4; k++)
    {
      key[3 + c * 8 + 2 * k] = (uint64_t)(uintptr_t)pl[k]->ptr;
      key[4 + c * 8 + 2 * k] = ((uint64_t)(uint32_t)pl[k]->stride << 8) | (uint64_t)(uint8_t)pl[k]->shift;
    }
  }
  auto encode = [&](CUtensorMap* maps) {
    for(int c = 0; c < 3; c++)
    {
      const SsimPlane* pl[4] = { &q[c].p0, &q[c].p1, &q[c].scp1, &q[c].scp0 };
      for(int k = 0; k < 4; k++)
      {
        const SsimPlane& P = *pl[k];
        const int wp = P.shift ? q[c].W / 2 : q[c].W, hp = P.shift ? q[c].H / 2 : q[c].H;
        if(!encode_plane(&maps[c * 4 + k], P.ptr, wp, hp, P.stride, P.sbytes, (uint32_t)quad_box_w(P.sbytes, P.shift),
                         (uint32_t)quad_box_h(win, P.shift)))
          return false;
      }
    }
    return true;
  };
  const void* d = nullptr;
  qmiv_status s = slot_tmaps(h, S, key, 12, encode, st, &d);
  if(s != QMIV_OK) return s;
  for(int c = 0; c < 3; c++) q[c].tmaps = static_cast<const uint8_t*>(d) + (size_t)c * 4 * sizeof(CUtensorMap);
  return QMIV_OK;
}

// ------------------------------------------------------------------------------------
// SSIM-family planning
// ------------------------------------------------------------------------------------
SsimPlane plane_of(const void* p, int stride, int sbytes, int shift)
{
  SsimPlane s;
  s.ptr = p; s.stride = stride; s.sbytes = (int8_t)sbytes; s.shift = (int8_t)shift; s.pad = 0;
  return s;
}

void add_ssim_job(qmiv_handle* h, const SsimPlane& a, const SsimPlane& b, int W, int H, int bd, int calc_l,
                  float*& partial, double* out)
{
  SsimJob s;
  std::memset(&s, 0, sizeof(s));
  s.a = a; s.b = b; s.W = W; s.H = H; s.calc_l = calc_l;
  const double mx = (double)((1 << bd) - 1);
  s.c1 = (float)((0.01 * mx) * (0.01 * mx)); // xSSIM.cpp:21-23
  s.c2 = (float)((0.03 * mx) * (0.03 * mx));
  s.tiles_x = ssim_tiles_x(W, h->opt.ssim_window);
  s.tiles_y = ssim_tiles_y(H);
  s.partial = partial;
  s.out = out;
  partial += (size_t)std::max(0, H - 10) * s.tiles_x;
  h->sjobs.push_back(s);
}

// SSIM jobs, pyramid steps and the combine entry of one frame (a job with SSIM metrics).
qmiv_status plan_ssim(qmiv_handle* h, const DevJob& j, cudaStream_t st)
{
  Slot& S = h->slots[j.slot];
  const int W = j.W, H = j.H, bd = j.bd, sb = j.sbytes, cs = j.cshift;
  float* part = S.partial;
  const SsimPlane P0[3] = { plane_of(j.p0[0], j.stride0[0], sb, 0), plane_of(j.p0[1], j.stride0[1], sb, cs), plane_of(j.p0[2], j.stride0[2], sb, cs) };
  const SsimPlane P1[3] = { plane_of(j.p1[0], j.stride1[0], sb, 0), plane_of(j.p1[1], j.stride1[1], sb, cs), plane_of(j.p1[2], j.stride1[2], sb, cs) };
  if(j.metrics & QMIV_M_IVSSIM)
  { // one fused pass per component: SSIM(P0,P1), CS(P0,P1) (MS-SSIM scale 0), and the IV-SSIM
    // directions T2R = SSIM(P0, SCP1), R2T = SSIM(P1, SCP0) (xSSIM.cpp:197-198); each output is
    // finalised by an SsimJob entry without tiles of its own
    const double mx = (double)((1 << bd) - 1);
    for(int c = 0; c < 3; c++)
    {
      SsimQuadJob q;
      std::memset(&q, 0, sizeof(q));
      q.p0 = P0[c]; q.p1 = P1[c];
      q.scp1 = plane_of(j.scp1[c], j.scp_stride, 2, 0);
      q.scp0 = plane_of(j.scp0[c], j.scp_stride, 2, 0);
      q.W = W; q.H = H;
      q.c1 = (float)((0.01 * mx) * (0.01 * mx)); // xSSIM.cpp:21-23
      q.c2 = (float)((0.03 * mx) * (0.03 * mx));
      q.tiles_x = ssim_tiles_x(W, h->opt.ssim_window);
      q.tiles_y = ssim_quad_tiles_y(H);
      q.outs = ((j.metrics & QMIV_M_SSIM) ? 1u : 0u) | ((j.metrics & QMIV_M_MSSSIM) ? 2u : 0u) | 12u;
      double* outs[4] = { S.vals + c, S.vals + 3 + c, S.vals + 18 + c, S.vals + 21 + c };
      for(int k = 0; k < 4; k++)
      {
        if(!(q.outs & (1u << k))) continue;
        q.partial[k] = part;
        add_ssim_job(h, P0[c], P1[c], W, H, bd, 1, part, outs[k]);
        h->sjobs.back().tiles_y = 0;  // finalisation only
      }
      q.status = reinterpret_cast<int32_t*>(reinterpret_cast<char*>(j.result) + offsetof(qmiv_frame_result, status));
      h->qjobs.push_back(q);
    }
    qmiv_status ts = ensure_quad_tmaps(h, S, &h->qjobs[h->qjobs.size() - 3], st);
    if(ts != QMIV_OK) return ts;
  }
  else if(j.metrics & QMIV_M_SSIM)   // xAppQMIV.cpp:907: calcPicSSIM(P0, P1)
    for(int c = 0; c < 3; c++) add_ssim_job(h, P0[c], P1[c], W, H, bd, 1, part, S.vals + c);
  if(j.metrics & QMIV_M_MSSSIM) // xSSIM.cpp:67-87
  {
    if(!(j.metrics & QMIV_M_IVSSIM))
      for(int c = 0; c < 3; c++) add_ssim_job(h, P0[c], P1[c], W, H, bd, 0, part, S.vals + 3 + c);
    // pyramid: level s of picture p, component c lives at pyr + off(s) + (p*3+c)*cap(s)
    size_t off = 0;
    SsimPlane prev[2][3];
    for(int p = 0; p < 2; p++)
      for(int c = 0; c < 3; c++) prev[p][c] = p == 0 ? plane_of(j.p0[c], j.stride0[c], sb, 0) : plane_of(j.p1[c], j.stride1[c], sb, 0);
    int w = W, hh = H;
    for(int s = 1; s <= 4; s++)
    {
      const int dw = w >> 1, dh = hh >> 1;
      const size_t cap = (size_t)(h->max_w >> s) * (h->max_h >> s);
      SsimPlane cur[2][3];
      for(int p = 0; p < 2; p++)
        for(int c = 0; c < 3; c++)
        {
          if(s == 1 && c > 0 && cs)
          { // 4:2:0: the 2x2 mean of the nearest-neighbour upsampled chroma is the native plane
            cur[p][c] = p == 0 ? plane_of(j.p0[c], j.stride0[c], sb, 0) : plane_of(j.p1[c], j.stride1[c], sb, 0);
            continue;
          }
          uint16_t* dst = S.pyr + off + (size_t)(p * 3 + c) * cap;
          PyrStep st;
          st.src = prev[p][c]; st.dst = dst; st.dst_stride = dw; st.dw = dw; st.dh = dh;
          h->steps[s - 1].push_back(st);
          cur[p][c] = plane_of(dst, dw, 2, 0);
        }
      off += 6 * cap;
      for(int c = 0; c < 3; c++) add_ssim_job(h, cur[0][c], cur[1][c], dw, dh, bd, s != 4, part, S.vals + 3 + 3 * s + c);
      for(int p = 0; p < 2; p++) for(int c = 0; c < 3; c++) prev[p][c] = cur[p][c];
      w = dw; hh = dh;
    }
  }
  SsimFrame f;
  f.metrics = j.metrics & kSsimMetrics; f.pad = 0; f.result = j.result; f.vals = S.vals;
  h->frames.push_back(f);
  return QMIV_OK;
}

// Lays out the call tables of h->jobs / sjobs / steps / frames and copies them to the device.
// Host image of the per-call tables (jobs, SSIM jobs, pyramid steps, SSIM frames), each
// section 256-byte aligned; returns its size, or 0 if it would exceed `cap`.
size_t pack_tables(const qmiv_handle* h, uint8_t* dst, size_t cap)
{
  size_t pos = 0;
  bool ok = true;
  auto put = [&](const void* src, size_t bytes) {
    if(pos + bytes > cap) { ok = false; return; }
    if(bytes) std::memcpy(dst + pos, src, bytes);
    pos += align256(bytes);
  };
  put(h->jobs.data(), sizeof(DevJob) * h->jobs.size());
  put(h->sjobs.data(), sizeof(SsimJob) * h->sjobs.size());
  for(int s = 0; s < 4; s++) put(h->steps[s].data(), sizeof(PyrStep) * h->steps[s].size());
  put(h->frames.data(), sizeof(SsimFrame) * h->frames.size());
  put(h->qjobs.data(), sizeof(SsimQuadJob) * h->qjobs.size());
  return ok ? pos : 0;
}

qmiv_status upload_tables(qmiv_handle* h, cudaStream_t st)
{
  CallTables& t = h->tab;
  const int k = h->tab_next;
  h->tab_next = (k + 1) % qmiv_handle::kRing;
  if(h->tab_used[k]) CUDA_TRY(cudaEventSynchronize(h->tab_ev[k]));
  const size_t pos = pack_tables(h, h->h_tab[k], t.bytes);
  if(!pos) return fail(QMIV_TOO_LARGE, "call tables exceed %zu B", t.bytes);
  CUDA_TRY(launch_copy_table(h->h_tab_dev[k], h->d_tab, pos, st));
  h->launches++;
  CUDA_TRY(cudaEventRecord(h->tab_ev[k], st));
  h->tab_used[k] = true;
  return QMIV_OK;
}

// The launch plan of the jobs in h->jobs: their CPS variants (sorted so that each variant's
// jobs are contiguous), grid decomposition, tensor maps and the SSIM-family tables.
struct LaunchPlan {
  std::vector<int> sv;   // CPS variant per (sorted) job, -1: none
  bool any_stats = false;
};

qmiv_status plan_jobs(qmiv_handle* h, LaunchPlan& P, cudaStream_t st)
{
  const int n = (int)h->jobs.size();
  std::vector<int> var(n);
  P.any_stats = false;
  for(int i = 0; i < n; i++)
  {
    DevJob& j = h->jobs[i];
    var[i] = (j.metrics & (QMIV_M_IVPSNR | QMIV_M_IVSSIM)) ? pick_cps_variant(h, j) : -1;
    P.any_stats |= (j.metrics & (QMIV_M_PSNR | QMIV_M_WSPSNR | QMIV_M_IVPSNR | QMIV_M_IVSSIM)) != 0;
  }
  std::vector<int> order(n);
  for(int i = 0; i < n; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return var[a] < var[b]; });
  std::vector<DevJob> sorted(n);
  std::vector<int> svar(n);
  P.sv.assign(n, -1);
  for(int i = 0; i < n; i++) { sorted[i] = h->jobs[order[i]]; P.sv[i] = var[order[i]]; svar[i] = P.sv[i] < 0 ? 0 : P.sv[i]; }
  plan_grid(h, sorted.data(), n, svar);
  int first = 0;
  while(first < n)
  {
    int last = first;
    while(last + 1 < n && P.sv[last + 1] == P.sv[first]) last++;
    int base = 0;
    for(int i = first; i <= last; i++) { sorted[i].cps_base = base; base += P.sv[i] < 0 ? 0 : sorted[i].cps_strips * sorted[i].cps_segs; }
    first = last + 1;
  }
  for(int i = 0; i < n; i++)
  {
    if(P.sv[i] > 0 && variants()[P.sv[i]].kind == 2)
    {
      qmiv_status ts = ensure_tmaps(h, sorted[i], variants()[P.sv[i]], st);
      if(ts != QMIV_OK) return ts;
    }
  }
  h->jobs = sorted;
  h->sjobs.clear(); h->frames.clear(); h->qjobs.clear();
  for(int s = 0; s < 4; s++) h->steps[s].clear();
  for(int i = 0; i < n; i++)
    if(h->jobs[i].metrics & kSsimMetrics) { qmiv_status ps = plan_ssim(h, h->jobs[i], st); if(ps != QMIV_OK) return ps; }
  int tb = 0;
  for(auto& s : h->sjobs) { s.tile_base = tb; tb += s.tiles_x * s.tiles_y; }
  tb = 0;
  for(auto& q : h->qjobs) { q.tile_base = tb; tb += q.tiles_x * q.tiles_y; }
  return QMIV_OK;
}

// Tiles of the SSIM tile kernel in a job table (0: it is not launched).
int ssim_tiles(const std::vector<SsimJob>& sj)
{
  int t = 0;
  for(const SsimJob& j : sj) t = std::max(t, j.tile_base + j.tiles_x * j.tiles_y);
  return t;
}

// Every launch of a plan, reading its tables from d_tab (laid out by pack_tables).
qmiv_status launch_jobs(qmiv_handle* h, const LaunchPlan& P, const uint8_t* d_tab, cudaStream_t st)
{
  const int n = (int)h->jobs.size();
  const DevJob* d_jobs = reinterpret_cast<const DevJob*>(d_tab);
  h->prof_n = 0;
  CUDA_TRY(launch_init_results(d_jobs, n, st));
  h->launches++;
  if(P.any_stats)
  {
    CUDA_TRY(prof_mark(h, "k_stats", st, true));
    CUDA_TRY(launch_stats(d_jobs, h->jobs.data(), n, h->params, st));
    CUDA_TRY(prof_mark(h, "k_stats", st, false));
    h->launches++;
  }
  int first = 0;
  while(first < n)
  {
    int last = first;
    while(last + 1 < n && P.sv[last + 1] == P.sv[first]) last++;
    if(P.sv[first] >= 0)
    {
      const CpsVariant& cv = variants()[P.sv[first]];
      int blocks = 0;
      bool maps = false;
      for(int i = first; i <= last; i++)
      {
        blocks = h->jobs[i].cps_base + h->jobs[i].cps_strips * h->jobs[i].cps_segs;
        maps = maps || h->jobs[i].cps_map[0] || h->jobs[i].cps_map[1];
      }
      CUDA_TRY(prof_mark(h, cv.name, st, true));
      if(blocks > 0) CUDA_TRY((maps ? cv.launch_map : cv.launch)(d_jobs + first, last - first + 1, blocks, h->params, st));
      CUDA_TRY(prof_mark(h, nullptr, st, false));
      h->launches++;
    }
    first = last + 1;
  }
  if(!h->sjobs.empty())
  {
    size_t pos = align256(sizeof(DevJob) * n) + align256(sizeof(SsimJob) * h->sjobs.size());
    for(int s = 0; s < 4; s++)
    {
      const PyrStep* d_steps = reinterpret_cast<const PyrStep*>(d_tab + pos);
      if(!h->steps[s].empty())
      {
        CUDA_TRY(prof_mark(h, "k_downsample", st, true));
        CUDA_TRY(launch_downsample(d_steps, h->steps[s].data(), (int)h->steps[s].size(), st));
        CUDA_TRY(prof_mark(h, nullptr, st, false));
        h->launches++;
      }
      pos += align256(sizeof(PyrStep) * h->steps[s].size());
    }
    const SsimFrame* d_frames = reinterpret_cast<const SsimFrame*>(d_tab + pos);
    pos += align256(sizeof(SsimFrame) * h->frames.size());
    if(!h->qjobs.empty())
    {
      const SsimQuadJob* d_q = reinterpret_cast<const SsimQuadJob*>(d_tab + pos);
      CUDA_TRY(prof_mark(h, h->opt.ssim_window == QMIV_SSIM_GAUSS11 ? "k_ssim_quad<11>" : "k_ssim_quad<10>", st, true));
      CUDA_TRY(launch_ssim_quad(d_q, h->qjobs.data(), (int)h->qjobs.size(), h->opt.ssim_window,
                                h->params.first_wait_test_polls, st));
      CUDA_TRY(prof_mark(h, nullptr, st, false));
      h->launches++;
    }
    const SsimJob* d_sjobs = reinterpret_cast<const SsimJob*>(d_tab + align256(sizeof(DevJob) * n));
    CUDA_TRY(prof_mark(h, h->opt.ssim_window == QMIV_SSIM_GAUSS11 ? "k_ssim<11>" : "k_ssim<10>", st, true));
    CUDA_TRY(launch_ssim(d_sjobs, h->sjobs.data(), (int)h->sjobs.size(), h->opt.ssim_window, st));
    CUDA_TRY(prof_mark(h, nullptr, st, false));
    h->launches += 2 + (ssim_tiles(h->sjobs) > 0 ? 1 : 0);  // the tile kernel (if any tiles), two finalisation passes
    CUDA_TRY(launch_ssim_combine(d_frames, (int)h->frames.size(), h->params, st));
    h->launches++;
  }
  return QMIV_OK;
}

// Runs every metric of the jobs in h->jobs (each bound to its slot).
qmiv_status run_jobs(qmiv_handle* h, cudaStream_t st)
{
  LaunchPlan P;
  qmiv_status s = plan_jobs(h, P, st);
  if(s != QMIV_OK) return s;
  if((s = upload_tables(h, st)) != QMIV_OK) return s;
  return launch_jobs(h, P, h->d_tab + h->tab.jobs_off, st);
}

// Window constants of the separable SSIM (the factor of the reference's coefficient table).
cudaError_t set_ssim_constants()
{
  double g[11], s = 0.0;
  for(int i = 0; i < 11; i++) { const double k = i - 5; g[i] = std::exp(-(k * k) / (2.0 * 1.5 * 1.5)); s += g[i]; }
  float gf[11];
  for(int i = 0; i < 11; i++) gf[i] = (float)(g[i] / s);
  double s10 = 0.0, s11 = 0.0;
  for(int i = 0; i < 10; i++) s10 += (double)gf[i];
  s11 = s10 + (double)gf[10];
  const double w0[2] = { s10 * s10, s11 * s11 };
  return ssim_set_window_constants(gf, w0);
}

void seq_add(qmiv_handle* h, uint32_t metrics, const qmiv_frame_result* r)
{ // xMetricStat::setPerCmpMeric / setPerPicMeric (xAppQMIV.h:245-252)
  SeqAcc& q = h->seq;
  if(metrics & QMIV_M_PSNR)   { for(int c = 0; c < 3; c++) q.v[c].push_back(r->psnr[c]); q.v[3].push_back(r->psnr_pic); }
  if(metrics & QMIV_M_WSPSNR) { for(int c = 0; c < 3; c++) q.v[4 + c].push_back(r->wspsnr[c]); q.v[7].push_back(r->wspsnr_pic); }
  if(metrics & QMIV_M_IVPSNR) q.v[8].push_back(r->ivpsnr);
  if(metrics & QMIV_M_SSIM)   { for(int c = 0; c < 3; c++) q.v[9 + c].push_back(r->ssim[c]); q.v[12].push_back(r->ssim_pic); }
  if(metrics & QMIV_M_MSSSIM) { for(int c = 0; c < 3; c++) q.v[13 + c].push_back(r->msssim[c]); q.v[16].push_back(r->msssim_pic); }
  if(metrics & QMIV_M_IVSSIM) q.v[17].push_back(r->ivssim);
}

}  // namespace

// =====================================================================================
// C ABI
// =====================================================================================
extern "C" {

int32_t qmiv_abi_version(void) { return QMIV_ABI_VERSION; }

const char* qmiv_status_str(qmiv_status s)
{
  switch(s)
  {
    case QMIV_OK: return "ok";
    case QMIV_BAD_ARG: return "bad argument";
    case QMIV_UNSUPPORTED: return "unsupported";
    case QMIV_CUDA_ERROR: return "CUDA error";
    case QMIV_DEVICE_TIMEOUT: return "device timeout";
    case QMIV_OUT_OF_MEMORY: return "out of memory";
    case QMIV_TOO_LARGE: return "too large for handle";
  }
  return "unknown";
}

const char* qmiv_last_error(void) { return g_last_error.c_str(); }

void qmiv_default_options(qmiv_options* o)
{
  if(!o) return;
  std::memset(o, 0, sizeof(*o));
  o->search_range = 2;
  o->cmp_w_search[0] = 4; o->cmp_w_search[1] = 1; o->cmp_w_search[2] = 1; o->cmp_w_search[3] = 0;
  o->cmp_w_avg[0] = 4; o->cmp_w_avg[1] = 1; o->cmp_w_avg[2] = 1; o->cmp_w_avg[3] = 0;
  o->unnoticeable[0] = o->unnoticeable[1] = o->unnoticeable[2] = 0.01f; o->unnoticeable[3] = 0.0f;
  o->use_ws = 0; o->lon_deg = 360; o->lat_deg = 180;
  o->fake_exact = 1; o->legacy_ws8 = 0; o->ssim_window = QMIV_SSIM_REF10;
  o->scratch_metrics = QMIV_M_ALL;
}

static qmiv_status check_options(const qmiv_options* o)
{
  if(!o) return fail(QMIV_BAD_ARG, "options are null");
  if(o->search_range < 0 || o->search_range > kMaxSR) return fail(QMIV_BAD_ARG, "search_range %d (0..%d)", o->search_range, kMaxSR);
  for(int c = 0; c < 3; c++)
  {
    if(o->cmp_w_search[c] < 0 || o->cmp_w_search[c] > 1024) return fail(QMIV_BAD_ARG, "cmp_w_search[%d]=%d", c, o->cmp_w_search[c]);
    if(o->cmp_w_avg[c] < 0) return fail(QMIV_BAD_ARG, "cmp_w_avg[%d]=%d", c, o->cmp_w_avg[c]);
  }
  if(o->cmp_w_avg[0] + o->cmp_w_avg[1] + o->cmp_w_avg[2] <= 0) return fail(QMIV_BAD_ARG, "cmp_w_avg sums to 0");
  if(o->lat_deg <= 0 || o->lat_deg > 180) return fail(QMIV_BAD_ARG, "lat_deg %d", o->lat_deg);
  if(o->ssim_window != QMIV_SSIM_REF10 && o->ssim_window != QMIV_SSIM_GAUSS11) return fail(QMIV_BAD_ARG, "ssim_window %d", o->ssim_window);
  if(o->scratch_metrics & ~QMIV_M_ALL) return fail(QMIV_BAD_ARG, "scratch_metrics 0x%x", o->scratch_metrics);
  return QMIV_OK;
}

qmiv_status qmiv_create(qmiv_handle** out, const qmiv_options* opt, int32_t max_w, int32_t max_h, int32_t max_jobs)
{
  if(!out) return fail(QMIV_BAD_ARG, "out is null");
  *out = nullptr;
  qmiv_options defaults;
  qmiv_default_options(&defaults);
  if(!opt) opt = &defaults;
  qmiv_status s = check_options(opt);
  if(s != QMIV_OK) return s;
  if(max_w < 2 || max_h < 2 || max_w > 65536 || max_h > 65536) return fail(QMIV_BAD_ARG, "max size %dx%d", max_w, max_h);
  if(max_jobs < 1 || max_jobs > 65536) return fail(QMIV_BAD_ARG, "max_jobs %d", max_jobs);

  qmiv_handle* h = new qmiv_handle();
  h->opt = *opt;
  h->max_w = max_w; h->max_h = max_h; h->max_jobs = max_jobs;
  derive_params(h);
  auto cleanup = [&](qmiv_status st) { qmiv_destroy(h); return st; };
  if(cudaGetDevice(&h->device) != cudaSuccess) return cleanup(fail(QMIV_CUDA_ERROR, "no CUDA device"));
  cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
  if(set_ssim_constants() != cudaSuccess) return cleanup(fail(QMIV_CUDA_ERROR, "SSIM window constants"));

  // per-slot scratch of the PSNR family
  const size_t rows_b = align256((size_t)max_h * 6 * sizeof(int64_t));
  const size_t cps_b = align256((size_t)2 * max_h * 3 * sizeof(unsigned long long));
  const size_t sc_b = align256(sizeof(JobScalars));
  const size_t tm_b = align256((size_t)Slot::kTmapSets * Slot::kTmapMaps * 128);
  const size_t per = rows_b + cps_b + sc_b + tm_b;
  if(cudaMalloc(&h->slot_mem, per * max_jobs) != cudaSuccess) return cleanup(fail(QMIV_OUT_OF_MEMORY, "slot scratch %zu B", per * max_jobs));
  if(cudaMemset(h->slot_mem, 0, per * max_jobs) != cudaSuccess) return cleanup(fail(QMIV_CUDA_ERROR, "memset"));
  h->slots.resize(max_jobs);
  for(int i = 0; i < max_jobs; i++)
  {
    uint8_t* b = (uint8_t*)h->slot_mem + per * i;
    h->slots[i].stat_rows = (int64_t*)b; b += rows_b;
    h->slots[i].cps_rows = (unsigned long long*)b; b += cps_b;
    h->slots[i].sc = (JobScalars*)b; b += sc_b;
    h->slots[i].d_tmaps = b;
  }
  h->tmap_clock = 0;
  // per-slot scratch of the SSIM family, for the metrics the caller reserves
  const uint32_t sm = opt->scratch_metrics;
  size_t scp_b = 0, pyr_b = 0, part_floats = 0;
  if(sm & QMIV_M_IVSSIM) scp_b = align256((size_t)6 * max_w * max_h * sizeof(uint16_t));
  if(sm & QMIV_M_MSSSIM)
    for(int sc = 1; sc <= 4; sc++) pyr_b += (size_t)6 * (max_w >> sc) * (max_h >> sc) * sizeof(uint16_t);
  pyr_b = align256(pyr_b);
  if(sm & kSsimMetrics)
  {
    // sized for the 11-tap window, whose narrower tiles give the most tiles per row
    const size_t full = (size_t)max_h * ssim_tiles_x(max_w, QMIV_SSIM_GAUSS11);
    part_floats = 12 * full;
    for(int sc = 1; sc <= 4; sc++) part_floats += 3 * (size_t)(max_h >> sc) * ssim_tiles_x(max_w >> sc, QMIV_SSIM_GAUSS11);
  }
  h->slot_partial_floats = part_floats;
  const size_t part_b = align256(part_floats * sizeof(float) + 16);
  const size_t vals_b = (sm & kSsimMetrics) ? align256(kSsimVals * sizeof(double)) : 0;
  const size_t sper = scp_b + pyr_b + part_b + vals_b;
  if(sper > 256 && (sm & kSsimMetrics))
  {
    if(cudaMalloc(&h->ssim_mem, sper * max_jobs) != cudaSuccess) return cleanup(fail(QMIV_OUT_OF_MEMORY, "SSIM scratch %zu B", sper * max_jobs));
    for(int i = 0; i < max_jobs; i++)
    {
      uint8_t* b = (uint8_t*)h->ssim_mem + sper * i;
      if(scp_b) { h->slots[i].scp = (uint16_t*)b; b += scp_b; }
      if(pyr_b) { h->slots[i].pyr = (uint16_t*)b; b += pyr_b; }
      h->slots[i].partial = (float*)b; b += part_b;
      h->slots[i].vals = (double*)b;
    }
  }
  if(cudaMalloc(&h->d_results, sizeof(qmiv_frame_result) * max_jobs) != cudaSuccess) return cleanup(fail(QMIV_OUT_OF_MEMORY, "results"));
  if(cudaMallocHost(&h->h_results, sizeof(qmiv_frame_result) * max_jobs) != cudaSuccess) return cleanup(fail(QMIV_OUT_OF_MEMORY, "pinned results"));
  // call tables
  CallTables& t = h->tab;
  t.jobs_off = 0;
  t.bytes = align256(sizeof(DevJob) * max_jobs) + align256(sizeof(SsimJob) * kSsimJobsPerFrame * max_jobs) +
            4 * align256(sizeof(PyrStep) * kPyrStepsPerFrame * max_jobs) + align256(sizeof(SsimFrame) * max_jobs) +
            align256(sizeof(SsimQuadJob) * 3 * max_jobs);
  if(cudaMalloc(&h->d_tab, t.bytes) != cudaSuccess) return cleanup(fail(QMIV_OUT_OF_MEMORY, "call tables"));
  for(int k = 0; k < qmiv_handle::kRing; k++)
  {
    if(cudaHostAlloc((void**)&h->h_tab[k], t.bytes, cudaHostAllocMapped) != cudaSuccess ||
       cudaHostGetDevicePointer((void**)&h->h_tab_dev[k], h->h_tab[k], 0) != cudaSuccess)
      return cleanup(fail(QMIV_OUT_OF_MEMORY, "pinned call tables"));
    if(cudaEventCreateWithFlags(&h->tab_ev[k], cudaEventDisableTiming) != cudaSuccess) return cleanup(fail(QMIV_CUDA_ERROR, "event"));
  }
  for(int i = 0; i < 2; i++)
  { // staging for host pictures: up to 3 full planes of 16-bit samples with 16-byte row pitch
    const size_t e = (size_t)((max_w + 7) & ~7) * max_h * 3 + 512;
    if(cudaMalloc(&h->d_stage[i], e * sizeof(uint16_t)) != cudaSuccess) return cleanup(fail(QMIV_OUT_OF_MEMORY, "staging"));
  }
  {
    const int nr = 2 * max_jobs + 4;
    if(cudaMallocHost(&h->h_tmaps, (size_t)nr * Slot::kTmapMaps * sizeof(CUtensorMap)) != cudaSuccess) return cleanup(fail(QMIV_OUT_OF_MEMORY, "pinned tensor maps"));
    h->tmap_ev.assign(nr, nullptr);
    h->tmap_used.assign(nr, 0);
    for(int k = 0; k < nr; k++)
      if(cudaEventCreateWithFlags(&h->tmap_ev[k], cudaEventDisableTiming) != cudaSuccess) return cleanup(fail(QMIV_CUDA_ERROR, "event"));
  }
  if(cudaMalloc(&h->mask_rows, sizeof(int64_t) * kMaskRowVals * max_h) != cudaSuccess ||
     cudaMalloc(&h->mask_small, 256) != cudaSuccess || cudaMemset(h->mask_small, 0, 256) != cudaSuccess ||
     cudaMalloc(&h->mask_stage, sizeof(uint16_t) * (size_t)max_w * max_h) != cudaSuccess)
    return cleanup(fail(QMIV_OUT_OF_MEMORY, "mask scratch"));
  if(cudaDeviceSynchronize() != cudaSuccess) return cleanup(fail(QMIV_CUDA_ERROR, "create sync"));
  *out = h;
  return QMIV_OK;
}

qmiv_status qmiv_destroy(qmiv_handle* h)
{
  if(!h) return QMIV_OK;
  cudaFree(h->slot_mem);
  cudaFree(h->ssim_mem);
  cudaFree(h->d_results);
  cudaFreeHost(h->h_results);
  cudaFree(h->d_tab);
  for(int k = 0; k < qmiv_handle::kRing; k++) { cudaFreeHost(h->h_tab[k]); if(h->tab_ev[k]) cudaEventDestroy(h->tab_ev[k]); }
  for(int i = 0; i < 2; i++) cudaFree(h->d_stage[i]);
  if(h->up_stream) cudaStreamSynchronize(h->up_stream);
  for(int i = 0; i < 2; i++)
  {
    cudaFree(h->d_up[i]);
    if(h->up_done[i]) cudaEventDestroy(h->up_done[i]);
    if(h->up_free[i]) cudaEventDestroy(h->up_free[i]);
  }
  if(h->up_stream) cudaStreamDestroy(h->up_stream);
  for(auto e : h->tmap_ev) if(e) cudaEventDestroy(e);
  cudaFreeHost(h->h_tmaps);
  cudaFree(h->mask_rows);
  cudaFree(h->mask_small);
  cudaFree(h->mask_stage);
  cudaFree(h->d_maps);
  for(auto& kv : h->ws_cache) cudaFree(kv.second.first);
  for(auto& p : h->prof) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
  delete h;
  return QMIV_OK;
}

qmiv_status qmiv_set_options(qmiv_handle* h, const qmiv_options* opt)
{
  if(!h) return fail(QMIV_BAD_ARG, "handle is null");
  qmiv_status s = check_options(opt);
  if(s != QMIV_OK) return s;
  if((opt->scratch_metrics & ~h->opt.scratch_metrics) != 0)
    return fail(QMIV_UNSUPPORTED, "scratch_metrics can only shrink after qmiv_create");
  if(opt->lat_deg != h->opt.lat_deg) { for(auto& kv : h->ws_cache) cudaFree(kv.second.first); h->ws_cache.clear(); }
  h->opt = *opt;
  derive_params(h);
  return QMIV_OK;
}

int64_t qmiv_kernel_launches(const qmiv_handle* h) { return h ? h->launches : 0; }

int32_t qmiv_cps_variant_count(void) { return (int32_t)variants().size(); }
const char* qmiv_cps_variant_name(int32_t v) { return (v >= 0 && v < (int32_t)variants().size()) ? variants()[v].name : ""; }

qmiv_status qmiv_set_profiling(qmiv_handle* h, int32_t enable)
{
  if(!h) return fail(QMIV_BAD_ARG, "handle is null");
  h->profiling = enable != 0;
  h->prof_n = 0;
  return QMIV_OK;
}

int32_t qmiv_kernel_times(qmiv_handle* h, const char** names, double* ms, int32_t max)
{
  if(!h) return -1;
  int n = 0;
  for(int i = 0; i < h->prof_n && n < max; i++, n++)
  {
    float t = 0.f;
    if(cudaEventSynchronize(h->prof[i].b) != cudaSuccess) return -1;
    if(cudaEventElapsedTime(&t, h->prof[i].a, h->prof[i].b) != cudaSuccess) return -1;
    if(names) names[n] = h->prof[i].name;
    if(ms) ms[n] = t;
  }
  return n;
}

qmiv_status qmiv_test_wait_timeout(qmiv_handle* h, uint32_t polls)
{
  if(!h) return fail(QMIV_BAD_ARG, "handle is null");
  h->test_wait_polls = polls;
  h->params.first_wait_test_polls = polls;
  return QMIV_OK;
}

qmiv_status qmiv_set_cps_variant(qmiv_handle* h, int32_t v)
{
  if(!h) return fail(QMIV_BAD_ARG, "handle is null");
  if(v < -1 || v >= (int32_t)variants().size()) return fail(QMIV_BAD_ARG, "variant %d", v);
  h->cps_variant_override = v;
  return QMIV_OK;
}

// ------------------------------------------------------------------------------------
// per frame
// ------------------------------------------------------------------------------------
static qmiv_status frame_common(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, uint32_t metrics,
                                const int32_t* gcd_given, uint16_t* const* scp0, uint16_t* const* scp1, int32_t scp_stride,
                                qmiv_frame_result* out, cudaStream_t st, int16_t* map_r2t = nullptr,
                                int16_t* map_t2r = nullptr, int32_t map_stride = 0)
{
  if(!h) return fail(QMIV_BAD_ARG, "handle is null");
  qmiv_status s = check_pair(h, pic0, pic1);
  if(s != QMIV_OK) return s;
  if((s = check_metrics(h, metrics, pic0->width, pic0->height)) != QMIV_OK) return s;
  qmiv_pic a, b;
  if((s = upload_pic(h, pic0, 0, &a, st)) != QMIV_OK) return s;
  if((s = upload_pic(h, pic1, 1, &b, st)) != QMIV_OK) return s;
  h->jobs.assign(1, DevJob());
  DevJob& j = h->jobs[0];
  fill_job(h, j, &a, &b, metrics, 0);
  j.use_ws = h->opt.use_ws;
  if(j.use_ws) { if((s = ws_weights(h, j.H, &j.ws, &j.ws_corr)) != QMIV_OK) return s; }
  if(scp0 && scp1) { for(int c = 0; c < 3; c++) { j.scp0[c] = scp0[c]; j.scp1[c] = scp1[c]; } j.scp_stride = scp_stride; }
  else if(metrics & QMIV_M_IVSSIM)
  {
    const size_t area = (size_t)h->max_w * h->max_h;
    for(int c = 0; c < 3; c++) { j.scp0[c] = h->slots[0].scp + c * area; j.scp1[c] = h->slots[0].scp + (3 + c) * area; }
    j.scp_stride = j.W;
  }
  j.cps_map[0] = map_r2t;
  j.cps_map[1] = map_t2r;
  j.map_stride = map_stride;
  if(gcd_given)
  {
    int32_t g[4] = { gcd_given[0], gcd_given[1], gcd_given[2], 0 };
    CUDA_TRY(cudaMemcpyAsync(h->slots[0].sc->gcd, g, sizeof(g), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st)); // `g` lives on this stack frame
    j.gcd_given = 1;
  }
  CUDA_TRY(cudaMemsetAsync(h->d_results, 0, sizeof(qmiv_frame_result), st));
  if((s = run_jobs(h, st)) != QMIV_OK) return s;
  CUDA_TRY(cudaMemcpyAsync(h->h_results, h->d_results, sizeof(qmiv_frame_result), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  *out = h->h_results[0];
  out->metrics = metrics;
  if(out->status != QMIV_OK) return fail((qmiv_status)out->status, "device-side wait gave up");
  return QMIV_OK;
}

qmiv_status qmiv_calc_frame(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, uint32_t metrics,
                            qmiv_frame_result* out, qmiv_stream stream)
{
  if(!out) return fail(QMIV_BAD_ARG, "out is null");
  qmiv_status s = frame_common(h, pic0, pic1, metrics, nullptr, nullptr, nullptr, 0, out, (cudaStream_t)stream);
  if(s != QMIV_OK) return s;
  seq_add(h, metrics, out);
  return QMIV_OK;
}

qmiv_status qmiv_calc_frame_masked(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, const qmiv_mask* mask,
                                   uint32_t metrics, qmiv_frame_result* out, qmiv_stream stream)
{
  if(!h || !out) return fail(QMIV_BAD_ARG, "handle or out is null");
  const cudaStream_t st = (cudaStream_t)stream;
  qmiv_status s = check_pair(h, pic0, pic1);
  if(s != QMIV_OK) return s;
  if(metrics & ~(QMIV_M_PSNR | QMIV_M_WSPSNR | QMIV_M_IVPSNR))
    return fail(QMIV_UNSUPPORTED, "masked metrics are PSNR, WS-PSNR and IV-PSNR (requested 0x%x)", metrics);
  if(!mask || !mask->plane) return fail(QMIV_BAD_ARG, "mask is null");
  if(mask->sample_bytes != 1 && mask->sample_bytes != 2) return fail(QMIV_BAD_ARG, "mask sample_bytes %d", mask->sample_bytes);
  if(mask->bitdepth < 1 || mask->bitdepth > 8 * mask->sample_bytes) return fail(QMIV_BAD_ARG, "mask bit depth %d", mask->bitdepth);
  if(mask->stride < pic0->width) return fail(QMIV_BAD_ARG, "mask stride %d < width %d", mask->stride, pic0->width);
  qmiv_pic a, b;
  if((s = upload_pic(h, pic0, 0, &a, st)) != QMIV_OK) return s;
  if((s = upload_pic(h, pic1, 1, &b, st)) != QMIV_OK) return s;
  MaskJob j;
  std::memset(&j, 0, sizeof(j));
  for(int c = 0; c < 3; c++) { j.p0[c] = a.plane[c]; j.p1[c] = b.plane[c]; j.s0[c] = a.stride[c]; j.s1[c] = b.stride[c]; }
  j.W = a.width; j.H = a.height; j.bd = a.bitdepth; j.sbytes = a.sample_bytes;
  j.cshift = a.chroma_format == QMIV_CF420 ? 1 : 0;
  if(mask->is_device) { j.mask = mask->plane; j.mstride = mask->stride; }
  else
  {
    CUDA_TRY(cudaMemcpy2DAsync(h->mask_stage, (size_t)j.W * mask->sample_bytes, mask->plane,
                               (size_t)mask->stride * mask->sample_bytes, (size_t)j.W * mask->sample_bytes, j.H,
                               cudaMemcpyHostToDevice, st));
    j.mask = h->mask_stage; j.mstride = j.W;
  }
  j.msbytes = mask->sample_bytes; j.mbd = mask->bitdepth;
  j.metrics = metrics;
  j.use_ws = h->opt.use_ws;
  if(j.use_ws) { if((s = ws_weights(h, j.H, &j.ws, &j.ws_corr)) != QMIV_OK) return s; }
  j.fake_exact = h->opt.fake_exact;
  j.sr = h->opt.search_range;
  for(int c = 0; c < 3; c++)
  {
    j.w_search[c] = h->opt.cmp_w_search[c]; j.w_avg[c] = h->opt.cmp_w_avg[c];
    j.maxdiff[c] = h->params.maxdiff_for_bd[j.bd][c];
  }
  {
    uint64_t bound = 0;
    for(int c = 0; c < 3; c++)
    {
      const uint64_t d = (uint64_t)((1 << j.bd) - 1) + (uint64_t)std::abs(j.maxdiff[c]);
      bound += d * d * (uint64_t)j.w_search[c];
    }
    j.fits32 = bound < (uint64_t)INT32_MAX;
  }
  j.counters = reinterpret_cast<uint32_t*>(h->mask_small);
  j.nnm = reinterpret_cast<long long*>(h->mask_small + 16);
  j.gcd = reinterpret_cast<int32_t*>(h->mask_small + 32);
  j.rows = h->mask_rows;
  j.cps_rows = h->slots[0].cps_rows;
  j.result = h->d_results;
  CUDA_TRY(cudaMemsetAsync(h->d_results, 0, sizeof(qmiv_frame_result), st));
  CUDA_TRY(launch_masked(j, st));
  h->launches += (metrics & QMIV_M_IVPSNR) ? 2 : 1;
  CUDA_TRY(cudaMemcpyAsync(h->h_results, h->d_results, sizeof(qmiv_frame_result), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  *out = h->h_results[0];
  out->metrics = metrics;
  seq_add(h, metrics, out);
  return QMIV_OK;
}

qmiv_status qmiv_gcd(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, int32_t gcd[4], qmiv_stream stream)
{
  if(!gcd) return fail(QMIV_BAD_ARG, "gcd is null");
  qmiv_frame_result r;
  qmiv_status s = frame_common(h, pic0, pic1, QMIV_M_PSNR, nullptr, nullptr, nullptr, 0, &r, (cudaStream_t)stream);
  if(s != QMIV_OK) return s;
  for(int c = 0; c < 4; c++) gcd[c] = r.gcd_r2t[c];
  return QMIV_OK;
}

qmiv_status qmiv_psnr(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, double psnr[4], double wspsnr[4], qmiv_stream stream)
{
  qmiv_frame_result r;
  qmiv_status s = frame_common(h, pic0, pic1, QMIV_M_PSNR | QMIV_M_WSPSNR, nullptr, nullptr, nullptr, 0, &r, (cudaStream_t)stream);
  if(s != QMIV_OK) return s;
  for(int c = 0; c < 4; c++) { if(psnr) psnr[c] = r.psnr[c]; if(wspsnr) wspsnr[c] = r.wspsnr[c]; }
  return QMIV_OK;
}

// PSNR and GCD without a handle: the statistics kernel's static-scratch variant. Nothing is
// allocated here (no device, pinned or managed memory); the only device memory written is
// the static array of k_stats.cu and the caller's *out through one copy.
qmiv_status qmiv_psnr_static(const qmiv_pic* pic0, const qmiv_pic* pic1, const qmiv_options* opt,
                             qmiv_frame_result* out, qmiv_stream stream)
{
  if(!pic0 || !pic1 || !out) return fail(QMIV_BAD_ARG, "pic0, pic1 and out must not be null");
  qmiv_options o;
  if(opt) o = *opt; else qmiv_default_options(&o);
  qmiv_status s = check_options(&o);
  if(s != QMIV_OK) return s;
  const qmiv_pic* pics[2] = { pic0, pic1 };
  for(int i = 0; i < 2; i++)
  {
    const qmiv_pic* p = pics[i];
    if(!p->is_device) return fail(QMIV_BAD_ARG, "pic%d: qmiv_psnr_static takes device pictures only", i);
    if(p->width < 1 || p->height < 1) return fail(QMIV_BAD_ARG, "pic%d: size %dx%d", i, p->width, p->height);
    if(p->height > kStaticMaxRows)
      return fail(QMIV_TOO_LARGE, "pic%d: height %d exceeds the static scratch limit of %d rows", i, p->height, kStaticMaxRows);
    if(p->width > kStaticMaxWidth)
      return fail(QMIV_TOO_LARGE, "pic%d: width %d exceeds the limit of %d samples per row", i, p->width, kStaticMaxWidth);
    if(p->bitdepth < 1 || p->bitdepth > 14) return fail(QMIV_BAD_ARG, "pic%d: bit depth %d (1..14)", i, p->bitdepth);
    if(p->sample_bytes != 1 && p->sample_bytes != 2) return fail(QMIV_BAD_ARG, "pic%d: sample_bytes %d", i, p->sample_bytes);
    if(p->sample_bytes == 1 && p->bitdepth > 8) return fail(QMIV_BAD_ARG, "pic%d: %d-bit samples in 8-bit storage", i, p->bitdepth);
    if(p->chroma_format != QMIV_CF420 && p->chroma_format != QMIV_CF444)
      return fail(QMIV_UNSUPPORTED, "pic%d: chroma format %d", i, p->chroma_format);
    if(p->chroma_format == QMIV_CF420 && ((p->width | p->height) & 1))
      return fail(QMIV_UNSUPPORTED, "pic%d: 4:2:0 needs even sizes (%dx%d)", i, p->width, p->height);
    for(int c = 0; c < 3; c++)
    {
      if(!p->plane[c]) return fail(QMIV_BAD_ARG, "pic%d: plane %d is null", i, c);
      const int w = (c && p->chroma_format == QMIV_CF420) ? p->width / 2 : p->width;
      if(p->stride[c] < w) return fail(QMIV_BAD_ARG, "pic%d: stride[%d]=%d < width %d", i, c, p->stride[c], w);
    }
  }
  if(pic0->width != pic1->width || pic0->height != pic1->height || pic0->bitdepth != pic1->bitdepth ||
     pic0->chroma_format != pic1->chroma_format || pic0->sample_bytes != pic1->sample_bytes)
    return fail(QMIV_BAD_ARG, "pic0 and pic1 differ in size, bit depth, format or sample size");

  StaticStatsScratch ss;
  CUDA_TRY(stats_static_scratch(&ss));
  Params p;
  std::memset(&p, 0, sizeof(p));
  for(int c = 0; c < 3; c++) p.w_avg[c] = o.cmp_w_avg[c];
  for(int bd = 0; bd <= 14; bd++)
    for(int c = 0; c < 3; c++) p.maxdiff_for_bd[bd][c] = rne_f32(o.unnoticeable[c] * (float)((1 << bd) - 1));
  p.fake_exact = o.fake_exact;
  DevJob j;
  std::memset(&j, 0, sizeof(j));
  for(int c = 0; c < 3; c++)
  {
    j.p0[c] = pic0->plane[c]; j.p1[c] = pic1->plane[c];
    j.stride0[c] = pic0->stride[c]; j.stride1[c] = pic1->stride[c];
  }
  j.W = pic0->width; j.H = pic0->height; j.bd = pic0->bitdepth; j.sbytes = pic0->sample_bytes;
  j.cshift = pic0->chroma_format == QMIV_CF420 ? 1 : 0;
  j.metrics = QMIV_M_PSNR;
  j.stat_rows = ss.stat_rows;
  j.sc = ss.sc;
  j.result = ss.result;
  j.stat_blocks = ((j.H + 1) / 2 + 7) / 8;
  const cudaStream_t st = (cudaStream_t)stream;
  // the block counter must start at zero; the result is cleared so fields not computed read 0
  CUDA_TRY(cudaMemsetAsync(ss.sc, 0, sizeof(JobScalars), st));
  CUDA_TRY(cudaMemsetAsync(ss.result, 0, sizeof(qmiv_frame_result), st));
  CUDA_TRY(launch_stats_static(j, p, st));
  CUDA_TRY(cudaMemcpyAsync(out, ss.result, sizeof(qmiv_frame_result), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  out->metrics = QMIV_M_PSNR;
  if(out->status != 0) return fail(QMIV_CUDA_ERROR, "device status %d", out->status);
  return QMIV_OK;
}

qmiv_status qmiv_ivpsnr(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, const int32_t* gcd,
                        double* iv, double* r2t, double* t2r, qmiv_stream stream)
{
  qmiv_frame_result r;
  qmiv_status s = frame_common(h, pic0, pic1, QMIV_M_IVPSNR, gcd, nullptr, nullptr, 0, &r, (cudaStream_t)stream);
  if(s != QMIV_OK) return s;
  if(iv) *iv = r.ivpsnr;
  if(r2t) *r2t = r.ivpsnr_r2t;
  if(t2r) *t2r = r.ivpsnr_t2r;
  return QMIV_OK;
}

qmiv_status qmiv_scp(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, const int32_t* gcd,
                     uint16_t* scp0[3], uint16_t* scp1[3], int32_t scp_stride, int32_t scp_is_device, qmiv_stream stream)
{
  if(!h) return fail(QMIV_BAD_ARG, "handle is null");
  if(!scp0 || !scp1) return fail(QMIV_BAD_ARG, "scp outputs are null");
  for(int c = 0; c < 3; c++) if(!scp0[c] || !scp1[c]) return fail(QMIV_BAD_ARG, "scp plane %d is null", c);
  if(!pic0) return fail(QMIV_BAD_ARG, "pic0 is null");
  if(scp_stride < pic0->width) return fail(QMIV_BAD_ARG, "scp_stride %d < width %d", scp_stride, pic0->width);
  cudaStream_t st = (cudaStream_t)stream;
  qmiv_frame_result r;
  // the SCP pictures come out of the CPS kernel, which runs for IV-PSNR
  if(scp_is_device) return frame_common(h, pic0, pic1, QMIV_M_IVPSNR, gcd, scp0, scp1, scp_stride, &r, st);
  if(!h->slots[0].scp) return fail(QMIV_UNSUPPORTED, "host SCP outputs need IV-SSIM scratch (scratch_metrics)");
  const size_t area = (size_t)h->max_w * h->max_h;
  uint16_t* d0[3]; uint16_t* d1[3];
  for(int c = 0; c < 3; c++) { d0[c] = h->slots[0].scp + c * area; d1[c] = h->slots[0].scp + (3 + c) * area; }
  qmiv_status s = frame_common(h, pic0, pic1, QMIV_M_IVPSNR, gcd, d0, d1, pic0->width, &r, st);
  if(s != QMIV_OK) return s;
  for(int c = 0; c < 3; c++)
  {
    CUDA_TRY(cudaMemcpy2DAsync(scp0[c], (size_t)scp_stride * 2, d0[c], (size_t)pic0->width * 2, (size_t)pic0->width * 2, pic0->height, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpy2DAsync(scp1[c], (size_t)scp_stride * 2, d1[c], (size_t)pic0->width * 2, (size_t)pic0->width * 2, pic0->height, cudaMemcpyDeviceToHost, st));
  }
  CUDA_TRY(cudaStreamSynchronize(st));
  return QMIV_OK;
}

qmiv_status qmiv_cps_maps(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, const int32_t* gcd,
                          int16_t* map_r2t, int16_t* map_t2r, int32_t map_stride, int32_t map_is_device, uint64_t* row_sse,
                          qmiv_stream stream)
{
  if(!h) return fail(QMIV_BAD_ARG, "handle is null");
  if(!map_r2t || !map_t2r) return fail(QMIV_BAD_ARG, "map outputs are null");
  if(!pic0) return fail(QMIV_BAD_ARG, "pic0 is null");
  if(map_stride < pic0->width) return fail(QMIV_BAD_ARG, "map_stride %d < width %d", map_stride, pic0->width);
  cudaStream_t st = (cudaStream_t)stream;
  qmiv_frame_result r;
  qmiv_status s;
  const int W = pic0->width, H = pic0->height;
  if(map_is_device) s = frame_common(h, pic0, pic1, QMIV_M_IVPSNR, gcd, nullptr, nullptr, 0, &r, st, map_r2t, map_t2r, map_stride);
  else
  {
    if(!h->d_maps) CUDA_TRY(cudaMalloc(&h->d_maps, (size_t)2 * h->max_w * h->max_h * sizeof(int16_t)));
    int16_t* d0 = h->d_maps;
    int16_t* d1 = h->d_maps + (size_t)h->max_w * h->max_h;
    s = frame_common(h, pic0, pic1, QMIV_M_IVPSNR, gcd, nullptr, nullptr, 0, &r, st, d0, d1, W);
    if(s != QMIV_OK) return s;
    CUDA_TRY(cudaMemcpy2DAsync(map_r2t, (size_t)map_stride * 2, d0, (size_t)W * 2, (size_t)W * 2, H, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpy2DAsync(map_t2r, (size_t)map_stride * 2, d1, (size_t)W * 2, (size_t)W * 2, H, cudaMemcpyDeviceToHost, st));
  }
  if(s != QMIV_OK) return s;
  if(row_sse)
    CUDA_TRY(cudaMemcpyAsync(row_sse, h->slots[0].cps_rows, (size_t)2 * H * 3 * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return QMIV_OK;
}

static qmiv_status fill_batch(qmiv_handle* h, const qmiv_job* jobs, int32_t n, qmiv_frame_result* results)
{
  if(!h) return fail(QMIV_BAD_ARG, "handle is null");
  if(!jobs || n < 1) return fail(QMIV_BAD_ARG, "no jobs");
  if(n > h->max_jobs) return fail(QMIV_TOO_LARGE, "%d jobs > max_jobs %d", n, h->max_jobs);
  if(!results) return fail(QMIV_BAD_ARG, "results is null");
  h->jobs.assign(n, DevJob());
  for(int i = 0; i < n; i++)
  {
    const qmiv_job& jb = jobs[i];
    qmiv_status s = check_pair(h, &jb.pic0, &jb.pic1);
    if(s != QMIV_OK) return fail(s, "job %d: %s", i, g_last_error.c_str());
    if(!jb.pic0.is_device) return fail(QMIV_BAD_ARG, "job %d: batch pictures must be device pointers", i);
    if((s = check_metrics(h, jb.metrics, jb.pic0.width, jb.pic0.height)) != QMIV_OK) return fail(s, "job %d: %s", i, g_last_error.c_str());
    DevJob& j = h->jobs[i];
    fill_job(h, j, &jb.pic0, &jb.pic1, jb.metrics, i);
    j.result = results + i;
    j.use_ws = jb.use_ws;
    if(j.use_ws) { s = ws_weights(h, j.H, &j.ws, &j.ws_corr); if(s != QMIV_OK) return s; }
    if(jb.scp0[0] && jb.scp1[0]) { for(int c = 0; c < 3; c++) { j.scp0[c] = jb.scp0[c]; j.scp1[c] = jb.scp1[c]; } j.scp_stride = jb.scp_stride; }
    else if(jb.metrics & QMIV_M_IVSSIM)
    {
      const size_t area = (size_t)h->max_w * h->max_h;
      for(int c = 0; c < 3; c++) { j.scp0[c] = h->slots[i].scp + c * area; j.scp1[c] = h->slots[i].scp + (3 + c) * area; }
      j.scp_stride = j.W;
    }
  }
  return QMIV_OK;
}

qmiv_status qmiv_calc_batch(qmiv_handle* h, const qmiv_job* jobs, int32_t n, qmiv_frame_result* results, qmiv_stream stream)
{
  qmiv_status s = fill_batch(h, jobs, n, results);
  if(s != QMIV_OK) return s;
  return run_jobs(h, (cudaStream_t)stream);
}

// ---- a batch of host pictures, uploaded in groups overlapped with the measurement ------------
qmiv_status qmiv_calc_batch_host(qmiv_handle* h, const qmiv_job* jobs, int32_t n, qmiv_frame_result* results,
                                 size_t group_bytes, qmiv_stream stream)
{
  if(!h) return fail(QMIV_BAD_ARG, "handle is null");
  if(!jobs || n < 1) return fail(QMIV_BAD_ARG, "no jobs");
  if(!results) return fail(QMIV_BAD_ARG, "results is null");
  const cudaStream_t st = (cudaStream_t)stream;
  std::vector<size_t> bytes(n);
  size_t largest = 0, total = 0;
  for(int i = 0; i < n; i++)
  {
    qmiv_status s = check_pair(h, &jobs[i].pic0, &jobs[i].pic1);
    if(s != QMIV_OK) return fail(s, "job %d: %s", i, g_last_error.c_str());
    if(jobs[i].pic0.is_device) return fail(QMIV_BAD_ARG, "job %d: qmiv_calc_batch_host takes host pictures", i);
    bytes[i] = stage_bytes(&jobs[i].pic0) + stage_bytes(&jobs[i].pic1);
    largest = std::max(largest, bytes[i]);
    total += bytes[i];
  }
  const bool taper = group_bytes == 0;
  if(group_bytes == 0) group_bytes = (total + 15) / 16;
  group_bytes = std::max(group_bytes, largest);
  // consecutive jobs per group, bounded by group_bytes and max_jobs. With the default size the
  // last two group sizes' worth of pictures go in quarter-size groups: the measurement of the
  // last group is the one part that no upload hides.
  std::vector<int> first(1, 0);
  {
    size_t acc = 0, done = 0, budget = group_bytes;
    for(int i = 0; i < n; i++)
    {
      if(i > first.back() && (acc + bytes[i] > budget || i - first.back() >= h->max_jobs))
      {
        first.push_back(i);
        done += acc;
        acc = 0;
        if(taper && total - done <= 2 * group_bytes) budget = std::max(largest, group_bytes / 4);
      }
      acc += bytes[i];
    }
  }
  first.push_back(n);
  const int groups = (int)first.size() - 1;
  if(!h->up_stream)
  {
    CUDA_TRY(cudaStreamCreateWithFlags(&h->up_stream, cudaStreamNonBlocking));
    for(int i = 0; i < 2; i++)
    {
      CUDA_TRY(cudaEventCreateWithFlags(&h->up_done[i], cudaEventDisableTiming));
      CUDA_TRY(cudaEventCreateWithFlags(&h->up_free[i], cudaEventDisableTiming));
    }
  }
  size_t need = 0;
  for(int g = 0; g < groups; g++)
  {
    size_t b = 0;
    for(int i = first[g]; i < first[g + 1]; i++) b += bytes[i];
    need = std::max(need, b);
  }
  if(need > h->up_cap)
  { // grow: earlier work on either buffer must have finished
    CUDA_TRY(cudaStreamSynchronize(h->up_stream));
    CUDA_TRY(cudaStreamSynchronize(st));
    for(int i = 0; i < 2; i++)
    {
      cudaFree(h->d_up[i]);
      h->d_up[i] = nullptr;
      h->up_recorded[i] = false;
    }
    h->up_cap = 0;
    for(int i = 0; i < 2; i++)
      if(cudaMalloc(&h->d_up[i], need) != cudaSuccess) return fail(QMIV_OUT_OF_MEMORY, "host-batch group buffers 2 x %zu B", need);
    h->up_cap = need;
  }
  std::vector<std::vector<qmiv_job>> staged(groups);
  auto upload = [&](int g) -> qmiv_status {
    const int b = g & 1;
    if(h->up_recorded[b]) CUDA_TRY(cudaStreamWaitEvent(h->up_stream, h->up_free[b], 0));
    size_t off = 0;
    staged[g].assign(jobs + first[g], jobs + first[g + 1]);
    for(int i = first[g]; i < first[g + 1]; i++)
    {
      qmiv_job& d = staged[g][i - first[g]];
      qmiv_status s = stage_pic(&jobs[i].pic0, h->d_up[b] + off, &d.pic0, h->up_stream);
      if(s != QMIV_OK) return s;
      off += stage_bytes(&jobs[i].pic0);
      if((s = stage_pic(&jobs[i].pic1, h->d_up[b] + off, &d.pic1, h->up_stream)) != QMIV_OK) return s;
      off += stage_bytes(&jobs[i].pic1);
    }
    CUDA_TRY(cudaEventRecord(h->up_done[b], h->up_stream));
    return QMIV_OK;
  };
  qmiv_status s = upload(0);
  for(int g = 0; g < groups && s == QMIV_OK; g++)
  {
    if(g + 1 < groups && (s = upload(g + 1)) != QMIV_OK) break;  // the next group uploads while this one runs
    const int b = g & 1;
    CUDA_TRY(cudaStreamWaitEvent(st, h->up_done[b], 0));
    if((s = fill_batch(h, staged[g].data(), first[g + 1] - first[g], results + first[g])) != QMIV_OK) break;
    if((s = run_jobs(h, st)) != QMIV_OK) break;
    CUDA_TRY(cudaEventRecord(h->up_free[b], st));
    h->up_recorded[b] = true;
  }
  return s;
}

// ---- a batch captured once as a CUDA graph ----------------------------------------------------
struct qmiv_graph {
  qmiv_handle* h = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint8_t* d_tab = nullptr;     // the batch's own tables
  uint8_t* d_tmaps = nullptr;   // the batch's own tensor maps (6 per job, 4 per fused-SSIM job)
  int64_t launches = 0;         // kernels per replay
};

qmiv_status qmiv_batch_graph_destroy(qmiv_graph* g)
{
  if(!g) return QMIV_OK;
  if(g->exec) cudaGraphExecDestroy(g->exec);
  if(g->graph) cudaGraphDestroy(g->graph);
  if(g->d_tab) cudaFree(g->d_tab);
  if(g->d_tmaps) cudaFree(g->d_tmaps);
  delete g;
  return QMIV_OK;
}

qmiv_status qmiv_batch_graph_create(qmiv_handle* h, const qmiv_job* jobs, int32_t n, qmiv_frame_result* results,
                                    qmiv_stream stream, qmiv_graph** out)
{
  if(!out) return fail(QMIV_BAD_ARG, "out is null");
  *out = nullptr;
  const cudaStream_t st = (cudaStream_t)stream;
  if(st == nullptr) return fail(QMIV_BAD_ARG, "graph capture needs a created stream, not the legacy default stream");
  qmiv_status s = fill_batch(h, jobs, n, results);
  if(s != QMIV_OK) return s;
  // one ordinary run first: validates the batch and performs every one-time set-up
  if((s = run_jobs(h, st)) != QMIV_OK) return s;
  CUDA_TRY(cudaStreamSynchronize(st));
  if((s = fill_batch(h, jobs, n, results)) != QMIV_OK) return s;
  LaunchPlan P;
  if((s = plan_jobs(h, P, st)) != QMIV_OK) return s;
  qmiv_graph* g = new qmiv_graph;
  g->h = h;
  auto bail = [&](qmiv_status e) { qmiv_batch_graph_destroy(g); return e; };
  // private copies of the tensor maps and tables: later calls on the handle rewrite the slots'
  const size_t nq = h->qjobs.size();
  if(cudaMalloc(&g->d_tmaps, ((size_t)n * 6 + nq * 4) * sizeof(CUtensorMap)) != cudaSuccess) return bail(fail(QMIV_OUT_OF_MEMORY, "graph tensor maps"));
  for(int i = 0; i < n; i++)
  {
    DevJob& j = h->jobs[i];
    if(!j.tmaps) continue;
    uint8_t* dst = g->d_tmaps + (size_t)i * 6 * sizeof(CUtensorMap);
    if(cudaMemcpyAsync(dst, j.tmaps, 6 * sizeof(CUtensorMap), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      return bail(fail(QMIV_CUDA_ERROR, "graph tensor maps copy"));
    j.tmaps = dst;
  }
  for(size_t i = 0; i < nq; i++)
  {
    SsimQuadJob& q = h->qjobs[i];
    if(!q.tmaps) continue;
    uint8_t* dst = g->d_tmaps + ((size_t)n * 6 + i * 4) * sizeof(CUtensorMap);
    if(cudaMemcpyAsync(dst, q.tmaps, 4 * sizeof(CUtensorMap), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      return bail(fail(QMIV_CUDA_ERROR, "graph tensor maps copy"));
    q.tmaps = dst;
  }
  std::vector<uint8_t> img(h->tab.bytes);
  const size_t bytes = pack_tables(h, img.data(), img.size());
  if(!bytes) return bail(fail(QMIV_TOO_LARGE, "call tables exceed %zu B", h->tab.bytes));
  if(cudaMalloc(&g->d_tab, bytes) != cudaSuccess) return bail(fail(QMIV_OUT_OF_MEMORY, "graph tables"));
  if(cudaMemcpyAsync(g->d_tab, img.data(), bytes, cudaMemcpyHostToDevice, st) != cudaSuccess ||
     cudaStreamSynchronize(st) != cudaSuccess)
    return bail(fail(QMIV_CUDA_ERROR, "graph tables copy"));
  const bool prof = h->profiling;
  h->profiling = false;
  const int64_t l0 = h->launches;
  if(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
  { h->profiling = prof; return bail(fail(QMIV_CUDA_ERROR, "cudaStreamBeginCapture")); }
  s = launch_jobs(h, P, g->d_tab, st);
  const cudaError_t ce = cudaStreamEndCapture(st, &g->graph);
  h->profiling = prof;
  g->launches = h->launches - l0;
  h->launches = l0;
  if(s != QMIV_OK) return bail(s);
  if(ce != cudaSuccess) return bail(fail(QMIV_CUDA_ERROR, "cudaStreamEndCapture: %s", cudaGetErrorString(ce)));
  if(cudaGraphInstantiate(&g->exec, g->graph, 0) != cudaSuccess) return bail(fail(QMIV_CUDA_ERROR, "cudaGraphInstantiate"));
  *out = g;
  return QMIV_OK;
}

qmiv_status qmiv_batch_graph_launch(qmiv_graph* g, qmiv_stream stream)
{
  if(!g || !g->exec) return fail(QMIV_BAD_ARG, "graph is null");
  CUDA_TRY(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
  g->h->launches += g->launches;
  return QMIV_OK;
}

// ---- CPS variant autotuner ---------------------------------------------------------------
qmiv_status qmiv_autotune_cps(qmiv_handle* h, const qmiv_job* jobs, int32_t n, qmiv_frame_result* results,
                              int32_t reps, qmiv_stream stream, int32_t* best_variant, double* best_ms)
{
  if(!h) return fail(QMIV_BAD_ARG, "handle is null");
  const cudaStream_t st = (cudaStream_t)stream;
  if(reps < 1) reps = 3;
  qmiv_status s = fill_batch(h, jobs, n, results);
  if(s != QMIV_OK) return s;
  std::vector<int> cand;
  for(int v = 1; v < (int)variants().size(); v++)
  {
    bool all = true, any = false;
    for(const DevJob& j : h->jobs)
    {
      if(!(j.metrics & (QMIV_M_IVPSNR | QMIV_M_IVSSIM))) continue;
      any = true;
      all = all && cps_variant_fits(h, j, v);
    }
    if(any && all) cand.push_back(v);
  }
  const int saved = h->cps_variant_override;
  const bool prof = h->profiling;
  if(!prof) { s = (qmiv_status)qmiv_set_profiling(h, 1); if(s != QMIV_OK) return s; }
  int best = saved;
  double best_t = 1e300;
  for(int v : cand)
  {
    h->cps_variant_override = v;
    double tmin = 1e300;
    for(int r = 0; r < reps + 1; r++)  // the first run of a variant is a warm-up
    {
      if((s = fill_batch(h, jobs, n, results)) != QMIV_OK || (s = run_jobs(h, st)) != QMIV_OK) break;
      const char* names[64];
      double ms[64];
      const int k = qmiv_kernel_times(h, names, ms, 64);
      double t = 0;
      for(int i = 0; i < k; i++)
        if(names[i] && std::strcmp(names[i], "k_stats") && std::strcmp(names[i], "k_downsample") && std::strncmp(names[i], "k_ssim", 6))
          t += ms[i];
      if(r > 0 && t < tmin) tmin = t;
    }
    if(s != QMIV_OK) break;
    if(tmin < best_t) { best_t = tmin; best = v; }
  }
  if(!prof) qmiv_set_profiling(h, 0);
  if(s != QMIV_OK) { h->cps_variant_override = saved; return s; }
  h->cps_variant_override = cand.empty() ? saved : best;
  if(best_variant) *best_variant = h->cps_variant_override;
  if(best_ms) *best_ms = cand.empty() ? 0.0 : best_t;
  return QMIV_OK;
}

qmiv_status qmiv_ssim(qmiv_handle* h, const qmiv_pic* tst, const qmiv_pic* ref, int32_t calc_l, double ssim[4], qmiv_stream stream)
{ // xSSIM::calcPicSSIM(Tst, Ref, CalcL) on any two pictures, no other metric
  if(!h) return fail(QMIV_BAD_ARG, "handle is null");
  if(!ssim) return fail(QMIV_BAD_ARG, "ssim is null");
  qmiv_status s = check_pair(h, tst, ref);
  if(s != QMIV_OK) return s;
  if(!h->slots[0].vals) return fail(QMIV_UNSUPPORTED, "SSIM needs SSIM scratch (scratch_metrics)");
  cudaStream_t st = (cudaStream_t)stream;
  qmiv_pic a, b;
  if((s = upload_pic(h, tst, 0, &a, st)) != QMIV_OK) return s;
  if((s = upload_pic(h, ref, 1, &b, st)) != QMIV_OK) return s;
  const int cs = a.chroma_format == QMIV_CF420 ? 1 : 0, sb = a.sample_bytes;
  h->jobs.clear(); h->sjobs.clear(); h->frames.clear();
  for(int k = 0; k < 4; k++) h->steps[k].clear();
  float* part = h->slots[0].partial;
  for(int c = 0; c < 3; c++)
    add_ssim_job(h, plane_of(a.plane[c], a.stride[c], sb, c ? cs : 0), plane_of(b.plane[c], b.stride[c], sb, c ? cs : 0),
                 a.width, a.height, a.bitdepth, calc_l ? 1 : 0, part, h->slots[0].vals + c);
  int tb = 0;
  for(auto& sj : h->sjobs) { sj.tile_base = tb; tb += sj.tiles_x * sj.tiles_y; }
  if((s = upload_tables(h, st)) != QMIV_OK) return s;
  // no picture-pair jobs in this call: the SSIM jobs start the table
  const SsimJob* d_sjobs = reinterpret_cast<const SsimJob*>(h->d_tab + h->tab.jobs_off);
  h->prof_n = 0;
  CUDA_TRY(launch_ssim(d_sjobs, h->sjobs.data(), 3, h->opt.ssim_window, st));
  h->launches += 2 + (ssim_tiles(h->sjobs) > 0 ? 1 : 0);
  double v[3];
  CUDA_TRY(cudaMemcpyAsync(v, h->slots[0].vals, sizeof(v), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  for(int c = 0; c < 3; c++) ssim[c] = v[c];
  ssim[3] = 0.0;
  return QMIV_OK;
}

qmiv_status qmiv_msssim(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, double msssim[4], qmiv_stream stream)
{
  if(!msssim) return fail(QMIV_BAD_ARG, "msssim is null");
  qmiv_frame_result r;
  qmiv_status s = frame_common(h, pic0, pic1, QMIV_M_MSSSIM, nullptr, nullptr, nullptr, 0, &r, (cudaStream_t)stream);
  if(s != QMIV_OK) return s;
  for(int c = 0; c < 4; c++) msssim[c] = r.msssim[c];
  return QMIV_OK;
}

qmiv_status qmiv_ivssim(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, const int32_t* gcd,
                        double* iv, double* r2t, double* t2r, qmiv_stream stream)
{
  qmiv_frame_result r;
  qmiv_status s = frame_common(h, pic0, pic1, QMIV_M_IVSSIM, gcd, nullptr, nullptr, 0, &r, (cudaStream_t)stream);
  if(s != QMIV_OK) return s;
  if(iv) *iv = r.ivssim;
  if(r2t) *r2t = r.ivssim_r2t;
  if(t2r) *t2r = r.ivssim_t2r;
  return QMIV_OK;
}

qmiv_status qmiv_finish_sequence(qmiv_handle* h, qmiv_seq_result* out)
{
  if(!h || !out) return fail(QMIV_BAD_ARG, "null argument");
  std::memset(out, 0, sizeof(*out));
  auto avg = [](const std::vector<double>& v) -> double {
    if(v.empty()) return std::nan("");
    double s = v[0], c = 0.0; // xKBNS::Accumulate / NumFrames (xAppQMIV.h:256-260)
    for(size_t i = 1; i < v.size(); i++)
    {
      const double t = s + v[i];
      if(std::fabs(s) >= std::fabs(v[i])) c += ((s - t) + v[i]); else c += ((v[i] - t) + s);
      s = t;
    }
    return (s + c) / (double)v.size();
  };
  const SeqAcc& q = h->seq;
  size_t nf = 0;
  for(int k = 0; k < 18; k++) nf = std::max(nf, q.v[k].size());
  out->num_frames = (int32_t)nf;
  for(int c = 0; c < 3; c++)
  {
    out->psnr[c] = avg(q.v[c]); out->wspsnr[c] = avg(q.v[4 + c]);
    out->ssim[c] = avg(q.v[9 + c]); out->msssim[c] = avg(q.v[13 + c]);
  }
  out->psnr_pic = avg(q.v[3]); out->wspsnr_pic = avg(q.v[7]); out->ivpsnr = avg(q.v[8]);
  out->ssim_pic = avg(q.v[12]); out->msssim_pic = avg(q.v[16]); out->ivssim = avg(q.v[17]);
  if(!q.v[3].empty()) out->metrics |= QMIV_M_PSNR;
  if(!q.v[7].empty()) out->metrics |= QMIV_M_WSPSNR;
  if(!q.v[8].empty()) out->metrics |= QMIV_M_IVPSNR;
  if(!q.v[12].empty()) out->metrics |= QMIV_M_SSIM;
  if(!q.v[16].empty()) out->metrics |= QMIV_M_MSSSIM;
  if(!q.v[17].empty()) out->metrics |= QMIV_M_IVSSIM;
  return QMIV_OK;
}

qmiv_status qmiv_reset_sequence(qmiv_handle* h)
{
  if(!h) return fail(QMIV_BAD_ARG, "handle is null");
  for(auto& v : h->seq.v) v.clear();
  return QMIV_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------
// Differentiable IV-PSNR error and IV-SSIM on FP32 4:4:4 pictures (k_loss.cu)
// ------------------------------------------------------------------------------------
namespace {

std::mutex g_const_mu;
bool g_const_set[kStaticMaxDevices] = { false };

qmiv_status loss_args(const float* tst, const float* ref, int32_t n, int32_t w, int32_t h, const qmiv_options* opt,
                      void* ws, size_t ws_bytes, LossArgs& a)
{
  qmiv_options o;
  if(opt) o = *opt; else qmiv_default_options(&o);
  qmiv_status s = check_options(&o);
  if(s != QMIV_OK) return s;
  if(n < 1 || w < 1 || h < 1) return fail(QMIV_BAD_ARG, "loss: n %d, size %dx%d", n, w, h);
  if(o.search_range < 1 || o.search_range > kLossMaxSR)
    return fail(QMIV_UNSUPPORTED, "loss: search_range %d (1..%d)", o.search_range, kLossMaxSR);
  if(!tst || !ref) return fail(QMIV_BAD_ARG, "loss: null picture");
  a.tst = tst; a.ref = ref; a.n = n; a.W = w; a.H = h; a.sr = o.search_range;
  for(int c = 0; c < 3; c++) { a.w_search[c] = (float)o.cmp_w_search[c]; a.unc[c] = o.unnoticeable[c]; }
  a.window = o.ssim_window;
  a.L = loss_layout(n, w, h, o.ssim_window);
  a.ws = (uint8_t*)ws;
  if(ws_bytes < a.L.bytes) return fail(QMIV_BAD_ARG, "loss: workspace %zu B < %zu B", ws_bytes, a.L.bytes);
  if(!ws || ((uintptr_t)ws & 255)) return fail(QMIV_BAD_ARG, "loss: workspace must be 256-byte aligned device memory");
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  if(dev < 0 || dev >= kStaticMaxDevices) return fail(QMIV_CUDA_ERROR, "loss: device %d", dev);
  std::lock_guard<std::mutex> lock(g_const_mu);
  if(!g_const_set[dev])
  {
    CUDA_TRY(set_ssim_constants());
    g_const_set[dev] = true;
  }
  return QMIV_OK;
}

}  // namespace

qmiv_status qmiv_loss_workspace_size(int32_t n, int32_t width, int32_t height, const qmiv_options* opt, size_t* bytes)
{
  if(!bytes || n < 1 || width < 1 || height < 1) return fail(QMIV_BAD_ARG, "loss workspace: bad arguments");
  qmiv_options o;
  if(opt) o = *opt; else qmiv_default_options(&o);
  *bytes = loss_layout(n, width, height, o.ssim_window).bytes;
  return QMIV_OK;
}

qmiv_status qmiv_loss_forward(const float* tst, const float* ref, int32_t n, int32_t width, int32_t height,
                              const qmiv_options* opt, void* workspace, size_t workspace_bytes, double* sse,
                              double* ssim, qmiv_stream stream)
{
  LossArgs a;
  qmiv_status s = loss_args(tst, ref, n, width, height, opt, workspace, workspace_bytes, a);
  if(s != QMIV_OK) return s;
  if(!sse || !ssim) return fail(QMIV_BAD_ARG, "loss: null outputs");
  CUDA_TRY(loss_forward(a, sse, ssim, (cudaStream_t)stream));
  return QMIV_OK;
}

qmiv_status qmiv_loss_backward(const float* tst, const float* ref, int32_t n, int32_t width, int32_t height,
                               const qmiv_options* opt, void* workspace, size_t workspace_bytes, const double* g_sse,
                               const double* g_ssim, float* g_tst, qmiv_stream stream)
{
  LossArgs a;
  qmiv_status s = loss_args(tst, ref, n, width, height, opt, workspace, workspace_bytes, a);
  if(s != QMIV_OK) return s;
  if(!g_sse || !g_ssim || !g_tst) return fail(QMIV_BAD_ARG, "loss: null gradients");
  CUDA_TRY(loss_backward(a, g_sse, g_ssim, g_tst, (cudaStream_t)stream));
  return QMIV_OK;
}

// ------------------------------------------------------------------------------------
// Input side: range check / concealment, colour conversion, raw YUV reader
// ------------------------------------------------------------------------------------
static int device_sms()
{
  int dev = 0, sms = 0;
  if(cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  return sms;
}

static qmiv_status check_device_pic(const qmiv_pic* p, const char* name)
{
  if(!p) return fail(QMIV_BAD_ARG, "%s is null", name);
  if(!p->is_device) return fail(QMIV_BAD_ARG, "%s must be in device memory", name);
  if(p->width < 1 || p->height < 1) return fail(QMIV_BAD_ARG, "%s: size %dx%d", name, p->width, p->height);
  if(p->bitdepth < 1 || p->bitdepth > 16) return fail(QMIV_BAD_ARG, "%s: bit depth %d", name, p->bitdepth);
  if(p->sample_bytes != 1 && p->sample_bytes != 2) return fail(QMIV_BAD_ARG, "%s: sample_bytes %d", name, p->sample_bytes);
  if(p->chroma_format != QMIV_CF420 && p->chroma_format != QMIV_CF444) return fail(QMIV_UNSUPPORTED, "%s: chroma format %d", name, p->chroma_format);
  for(int c = 0; c < 3; c++)
  {
    const int w = (c && p->chroma_format == QMIV_CF420) ? p->width / 2 : p->width;
    if(!p->plane[c] || p->stride[c] < w) return fail(QMIV_BAD_ARG, "%s: plane %d null or stride < width", name, c);
  }
  return QMIV_OK;
}

// Counters of qmiv_check_range: per calling thread and device, 3 device counters and their
// pinned host copy, made on the first call and kept (a call is synchronous, so a thread's
// calls never overlap; other threads have their own).
struct RangeCounters {
  unsigned long long* d[kStaticMaxDevices] = {};
  unsigned long long* h[kStaticMaxDevices] = {};
  ~RangeCounters()
  {
    for(int i = 0; i < kStaticMaxDevices; i++)
    {
      if(d[i]) cudaFree(d[i]);
      if(h[i]) cudaFreeHost(h[i]);
    }
  }
};

qmiv_status qmiv_check_range(const qmiv_pic* pic, int32_t conceal, int64_t out_of_range[3], qmiv_stream stream)
{
  qmiv_status s = check_device_pic(pic, "pic");
  if(s != QMIV_OK) return s;
  if(!out_of_range) return fail(QMIV_BAD_ARG, "out_of_range is null");
  const cudaStream_t st = (cudaStream_t)stream;
  thread_local RangeCounters rc;
  int slot = 0;
  CUDA_TRY(cudaGetDevice(&slot));
  if(slot < 0 || slot >= kStaticMaxDevices) return fail(QMIV_UNSUPPORTED, "device %d: at most %d devices", slot, kStaticMaxDevices);
  if(!rc.d[slot])
  {
    CUDA_TRY(cudaMalloc((void**)&rc.d[slot], 3 * sizeof(unsigned long long)));
    CUDA_TRY(cudaHostAlloc((void**)&rc.h[slot], 3 * sizeof(unsigned long long), cudaHostAllocDefault));
  }
  unsigned long long* d_cnt = rc.d[slot];
  CUDA_TRY(cudaMemsetAsync(d_cnt, 0, 3 * sizeof(unsigned long long), st));
  const int maxv = pic->bitdepth >= 16 ? 65535 : (1 << pic->bitdepth) - 1;
  RangeJob j;
  std::memset(&j, 0, sizeof(j));
  for(int c = 0; c < 3; c++)
  {
    const bool sub = c && pic->chroma_format == QMIV_CF420;
    j.plane[c] = const_cast<void*>(pic->plane[c]);
    j.stride[c] = pic->stride[c];
    j.w[c] = sub ? pic->width / 2 : pic->width;
    j.h[c] = sub ? pic->height / 2 : pic->height;
  }
  j.sbytes = pic->sample_bytes; j.maxv = maxv; j.conceal = conceal ? 1 : 0; j.count = d_cnt;
  CUDA_TRY(launch_range(j, device_sms(), st));
  unsigned long long* h = rc.h[slot];
  CUDA_TRY(cudaMemcpyAsync(h, d_cnt, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  for(int c = 0; c < 3; c++) out_of_range[c] = (int64_t)h[c];
  return QMIV_OK;
}

qmiv_status qmiv_color_convert(const qmiv_pic* src, uint16_t* dst[3], int32_t dst_stride, int32_t to_ycbcr,
                               int32_t color_space, qmiv_stream stream)
{
  qmiv_status s = check_device_pic(src, "src");
  if(s != QMIV_OK) return s;
  if(src->chroma_format != QMIV_CF444) return fail(QMIV_UNSUPPORTED, "colour conversion works on 4:4:4 pictures");
  if(src->bitdepth > 14) return fail(QMIV_UNSUPPORTED, "colour conversion: bit depth %d (at most 14)", src->bitdepth);
  if(color_space < 0 || color_space > 3) return fail(QMIV_BAD_ARG, "colour space %d (0 BT.601, 1 BT.709, 2 SMPTE 240M, 3 BT.2020)", color_space);
  if(!dst || !dst[0] || !dst[1] || !dst[2] || dst_stride < src->width) return fail(QMIV_BAD_ARG, "dst planes or stride");
  if(src->stride[0] != src->stride[1] || src->stride[0] != src->stride[2]) return fail(QMIV_UNSUPPORTED, "src planes must share one stride");
  ColorJob j;
  std::memset(&j, 0, sizeof(j));
  for(int c = 0; c < 3; c++) { j.src[c] = src->plane[c]; j.dst[c] = dst[c]; }
  j.sbytes = src->sample_bytes; j.sstride = src->stride[0]; j.dstride = dst_stride;
  j.W = src->width; j.H = src->height; j.bd = src->bitdepth; j.to_ycbcr = to_ycbcr ? 1 : 0;
  color_matrix(color_space, to_ycbcr != 0, j.m);
  CUDA_TRY(launch_color(j, (cudaStream_t)stream));
  return QMIV_OK;
}

// A frame is read by a few threads at once (pread of consecutive slices into the pinned
// buffer): one thread copying out of the page cache reaches a fraction of the host memory
// bandwidth. The workers persist for the reader's lifetime and wait for a generation number.
struct YuvPool {
  std::vector<std::thread> workers;
  std::mutex m;
  std::condition_variable cv, done_cv;
  int fd = -1;
  uint8_t* dst = nullptr;
  int64_t off = 0, bytes = 0;
  uint64_t gen = 0;
  int pending = 0;
  bool stop = false, failed = false;

  void run(int id, int n)
  {
    uint64_t seen = 0;
    for(;;)
    {
      uint8_t* d; int64_t o, b;
      {
        std::unique_lock<std::mutex> lk(m);
        cv.wait(lk, [&] { return stop || gen != seen; });
        if(stop) return;
        seen = gen; d = dst; o = off; b = bytes;
      }
      // slice id of n, 4 KiB aligned
      const int64_t per = ((b + n - 1) / n + 4095) & ~(int64_t)4095;
      const int64_t s0 = std::min(b, per * id), s1 = std::min(b, s0 + per);
      bool ok = true;
      for(int64_t p = s0; p < s1 && ok;)
      {
        const ssize_t got = ::pread(fd, d + p, (size_t)(s1 - p), (off_t)(o + p));
        if(got <= 0) ok = false; else p += got;
      }
      std::lock_guard<std::mutex> lk(m);
      if(!ok) failed = true;
      if(--pending == 0) done_cv.notify_all();
    }
  }
  bool read(uint8_t* d, int64_t o, int64_t b)
  {
    std::unique_lock<std::mutex> lk(m);
    dst = d; off = o; bytes = b; failed = false; pending = (int)workers.size(); gen++;
    cv.notify_all();
    done_cv.wait(lk, [&] { return pending == 0; });
    return !failed;
  }
  ~YuvPool()
  {
    { std::lock_guard<std::mutex> lk(m); stop = true; }
    cv.notify_all();
    for(auto& t : workers) t.join();
  }
};

struct qmiv_yuv_reader {
  FILE* f = nullptr;
  int32_t w = 0, h = 0, bd = 8, cf = 420, bps = 1;
  int64_t frame_bytes = 0, frames = 0;
  uint8_t* h_buf[2] = { nullptr, nullptr };   // pinned, one per device slot
  uint8_t* d_raw[2] = { nullptr, nullptr };   // the raw frame as read
  uint8_t* d_444[2] = { nullptr, nullptr };   // 4:2:2 chroma upsampled to 4:4:4
  cudaEvent_t ev[2] = { nullptr, nullptr };
  bool used[2] = { false, false };
  std::unique_ptr<YuvPool> pool;              // frames of 1 MiB and more
};

qmiv_status qmiv_yuv_close(qmiv_yuv_reader* r)
{
  if(!r) return QMIV_OK;
  r->pool.reset();
  if(r->f) std::fclose(r->f);
  for(int i = 0; i < 2; i++)
  {
    if(r->ev[i]) { cudaEventSynchronize(r->ev[i]); cudaEventDestroy(r->ev[i]); }
    cudaFreeHost(r->h_buf[i]); cudaFree(r->d_raw[i]); cudaFree(r->d_444[i]);
  }
  delete r;
  return QMIV_OK;
}

qmiv_status qmiv_yuv_open(qmiv_yuv_reader** out, const char* path, int32_t width, int32_t height, int32_t bitdepth,
                          int32_t chroma_format)
{
  if(!out || !path) return fail(QMIV_BAD_ARG, "out or path is null");
  *out = nullptr;
  if(width < 1 || height < 1 || bitdepth < 1 || bitdepth > 16) return fail(QMIV_BAD_ARG, "size %dx%d, bit depth %d", width, height, bitdepth);
  if(chroma_format != 420 && chroma_format != 422 && chroma_format != 444) return fail(QMIV_UNSUPPORTED, "chroma format %d (420, 422, 444)", chroma_format);
  if((chroma_format != 444 && (width & 1)) || (chroma_format == 420 && (height & 1))) return fail(QMIV_UNSUPPORTED, "odd size for %d", chroma_format);
  qmiv_yuv_reader* r = new qmiv_yuv_reader;
  auto bail = [&](qmiv_status e) { qmiv_yuv_close(r); return e; };
  r->w = width; r->h = height; r->bd = bitdepth; r->cf = chroma_format; r->bps = bitdepth > 8 ? 2 : 1;
  const int64_t area = (int64_t)width * height;
  const int64_t csz = chroma_format == 420 ? area / 4 : (chroma_format == 422 ? area / 2 : area);
  r->frame_bytes = (area + 2 * csz) * r->bps;
  r->f = std::fopen(path, "rb");
  if(!r->f) return bail(fail(QMIV_BAD_ARG, "cannot open %s", path));
  std::fseek(r->f, 0, SEEK_END);
  const long long bytes = std::ftell(r->f);
  r->frames = bytes / r->frame_bytes;  // xSeqBase counts whole frames
  if(r->frame_bytes >= (1 << 20))
  {
    const unsigned hc = std::thread::hardware_concurrency();
    const int n = (int)std::max(1u, std::min(4u, hc ? hc : 1u));
    r->pool.reset(new YuvPool);
    r->pool->fd = fileno(r->f);
    for(int i = 0; i < n; i++) r->pool->workers.emplace_back([p = r->pool.get(), i, n] { p->run(i, n); });
  }
  for(int i = 0; i < 2; i++)
  {
    if(cudaMallocHost((void**)&r->h_buf[i], r->frame_bytes) != cudaSuccess ||
       cudaMalloc((void**)&r->d_raw[i], r->frame_bytes) != cudaSuccess ||
       cudaEventCreateWithFlags(&r->ev[i], cudaEventDisableTiming) != cudaSuccess)
      return bail(fail(QMIV_OUT_OF_MEMORY, "YUV reader buffers"));
    if(chroma_format == 422 && cudaMalloc((void**)&r->d_444[i], 2 * area * r->bps) != cudaSuccess)
      return bail(fail(QMIV_OUT_OF_MEMORY, "YUV reader 4:4:4 chroma"));
  }
  *out = r;
  return QMIV_OK;
}

int64_t qmiv_yuv_frames(const qmiv_yuv_reader* r) { return r ? r->frames : 0; }

qmiv_status qmiv_yuv_read(qmiv_yuv_reader* r, int64_t frame, qmiv_pic* out, qmiv_stream stream)
{
  if(!r || !out) return fail(QMIV_BAD_ARG, "reader or out is null");
  if(frame < 0 || frame >= r->frames) return fail(QMIV_BAD_ARG, "frame %lld of %lld", (long long)frame, (long long)r->frames);
  const cudaStream_t st = (cudaStream_t)stream;
  const int k = (int)(frame & 1);
  if(r->used[k]) CUDA_TRY(cudaEventSynchronize(r->ev[k]));  // the slot's previous upload has finished
  if(r->pool)
  {
    if(!r->pool->read(r->h_buf[k], frame * r->frame_bytes, r->frame_bytes))
      return fail(QMIV_BAD_ARG, "short read of frame %lld", (long long)frame);
  }
  else if(std::fseek(r->f, (long)(frame * r->frame_bytes), SEEK_SET) != 0 ||
          std::fread(r->h_buf[k], 1, (size_t)r->frame_bytes, r->f) != (size_t)r->frame_bytes)
    return fail(QMIV_BAD_ARG, "short read of frame %lld", (long long)frame);
  CUDA_TRY(cudaMemcpyAsync(r->d_raw[k], r->h_buf[k], (size_t)r->frame_bytes, cudaMemcpyHostToDevice, st));
  const int64_t area = (int64_t)r->w * r->h;
  const int bps = r->bps;
  std::memset(out, 0, sizeof(*out));
  out->width = r->w; out->height = r->h; out->bitdepth = r->bd; out->sample_bytes = bps; out->is_device = 1;
  out->plane[0] = r->d_raw[k]; out->stride[0] = r->w;
  if(r->cf == 420)
  {
    out->chroma_format = QMIV_CF420;
    out->plane[1] = r->d_raw[k] + area * bps; out->plane[2] = r->d_raw[k] + (area + area / 4) * bps;
    out->stride[1] = out->stride[2] = r->w / 2;
  }
  else if(r->cf == 444)
  {
    out->chroma_format = QMIV_CF444;
    out->plane[1] = r->d_raw[k] + area * bps; out->plane[2] = r->d_raw[k] + 2 * area * bps;
    out->stride[1] = out->stride[2] = r->w;
  }
  else
  { // 4:2:2: chroma doubled horizontally into 4:4:4 planes (xSeq.cpp:219-233)
    for(int c = 0; c < 2; c++)
      CUDA_TRY(launch_upsample_h(r->d_raw[k] + (area + c * area / 2) * bps, bps, r->w / 2, r->d_444[k] + c * area * bps,
                                 r->w, r->h, st));
    out->chroma_format = QMIV_CF444;
    out->plane[1] = r->d_444[k]; out->plane[2] = r->d_444[k] + area * bps;
    out->stride[1] = out->stride[2] = r->w;
  }
  CUDA_TRY(cudaEventRecord(r->ev[k], st));
  r->used[k] = true;
  return QMIV_OK;
}
