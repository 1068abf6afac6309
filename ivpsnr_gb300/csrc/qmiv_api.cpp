// Host side of the C ABI (include/qmiv_gb300.h): handles, argument validation, device
// scratch, job descriptors and launch sequencing. No host threads; every call is enqueued
// on the caller's stream.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include <cuda.h>
#include <cuda_runtime.h>

#include "qmiv_internal.h"

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

// Device slot for one job: scratch rows and scalars, plus the tensor maps of its planes.
struct Slot {
  int64_t* stat_rows = nullptr;          // [max_h][6]
  unsigned long long* cps_rows = nullptr; // [2][max_h][3]
  JobScalars* sc = nullptr;
  void* d_tmaps = nullptr;               // 6 x 128 B in device memory
  uint64_t tmap_key[16] = { 0 };         // what the maps were encoded for
  bool tmap_valid = false;
};

struct SeqAcc { std::vector<double> v[16]; };

}  // namespace

struct qmiv_handle {
  qmiv_options opt;
  Params params;
  int max_w = 0, max_h = 0, max_jobs = 0;
  int device = 0, num_sms = 0;
  int cps_variant_override = -1;         // set by the autotuner / tests
  std::vector<Slot> slots;
  void* slot_mem = nullptr;
  DevJob* d_jobs = nullptr;              // device job table
  DevJob* h_jobs = nullptr;              // pinned host job table
  qmiv_frame_result* d_results = nullptr;
  qmiv_frame_result* h_results = nullptr; // pinned
  // staging for host pictures (2 pictures, planar, uint16 worst case)
  uint16_t* d_stage[2] = { nullptr, nullptr };
  size_t stage_elems = 0;
  // shift-compensated pictures for the per-frame IV-SSIM path
  uint16_t* d_scp[2] = { nullptr, nullptr };
  // equirectangular row weights, cached per (height, lat)
  std::map<std::pair<int, int>, std::pair<double*, double>> ws_cache;
  SeqAcc seq;
  int64_t launches = 0;
  // optional per-launch timing
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
}

// Does the 32-bit packed key hold for this bit depth?
bool key32_ok(const qmiv_handle* h, int bd)
{
  const Params& p = h->params;
  int md = 0;
  for(int c = 0; c < 3; c++) md = std::max(md, p.maxdiff_for_bd[bd][c]);
  const uint64_t D = (uint64_t)((1 << bd) - 1) + (uint64_t)md;
  const uint64_t wsum = (uint64_t)p.w_search[0] + p.w_search[1] + p.w_search[2];
  const uint64_t N = window_index_bound(p.sr);
  const uint64_t kmax = (uint64_t)p.key_m * wsum * D * D + N;
  return kmax < (1ull << 32) && (uint64_t)p.luma_scale * D < 46340ull;
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

int pick_cps_variant(const qmiv_handle* h, const DevJob& j)
{
  const auto& V = variants();
  const int sr = h->params.sr;
  if(!j.cshift || h->opt.cmp_w_search[0] < 1 || sr < 1 || sr > 4) return 0; // generic
  if(h->cps_variant_override == 0) return 0;
  const bool k64 = !key32_ok(h, j.bd);
  const bool tma = tma_ok(j);
  auto fits = [&](int v) {
    const CpsVariant& c = V[v];
    if(c.sr != sr || c.key64 != k64) return false;
    if(c.kind == 2 && (!tma || c.sbytes != j.sbytes)) return false;
    return c.kind != 0;
  };
  if(h->cps_variant_override > 0 && h->cps_variant_override < (int)V.size() && fits(h->cps_variant_override))
    return h->cps_variant_override;
  // default: the TMA kernel with 32-row strips and 8 warps, else the staged-load kernel
  for(int v = 1; v < (int)V.size(); v++)
    if(fits(v) && V[v].kind == 2 && V[v].rows == 32 && std::strstr(V[v].name, "_q4_w4")) return v;
  for(int v = 1; v < (int)V.size(); v++)
    if(fits(v) && V[v].kind == 1 && std::strstr(V[v].name, "rpt8_nwg2")) return v;
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

// Fill the device-independent part of a job from two validated pictures (device pointers).
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
    int segs = (int)std::min<long long>(nchunks, std::max<long long>(1, (target + strips_total - 1) / strips_total));
    // per-thread 32-bit SSE accumulators: 2 pixels per chunk, each < (Max + maxdiff)^2
    int md = 0; for(int c = 0; c < 3; c++) md = std::max(md, h->params.maxdiff_for_bd[j.bd][c]);
    const double D = (double)((1 << j.bd) - 1 + md);
    const int max_chunks = std::max(1, (int)std::floor(4294967295.0 / (2.0 * D * D)));
    int seg_chunks = (nchunks + segs - 1) / segs;
    if(seg_chunks > max_chunks) seg_chunks = max_chunks;
    j.cps_seg_chunks = seg_chunks;
    j.cps_segs = (nchunks + seg_chunks - 1) / seg_chunks;
  }
}

qmiv_status upload_pic(qmiv_handle* h, const qmiv_pic* src, int idx, qmiv_pic* dst, cudaStream_t st)
{ // host picture -> packed device staging (same sample size, planes back to back)
  *dst = *src;
  if(src->is_device) return QMIV_OK;
  const int sb = src->sample_bytes;
  uint8_t* base = reinterpret_cast<uint8_t*>(h->d_stage[idx]);
  size_t off = 0;
  for(int c = 0; c < 3; c++)
  {
    const int w = (c && src->chroma_format == QMIV_CF420) ? src->width / 2 : src->width;
    const int hh = (c && src->chroma_format == QMIV_CF420) ? src->height / 2 : src->height;
    off = (off + 15) & ~(size_t)15;
    CUDA_TRY(cudaMemcpy2DAsync(base + off, (size_t)w * sb, src->plane[c], (size_t)src->stride[c] * sb,
                               (size_t)w * sb, hh, cudaMemcpyHostToDevice, st));
    dst->plane[c] = base + off;
    dst->stride[c] = w;
    off += (size_t)w * hh * sb;
  }
  dst->is_device = 1;
  return QMIV_OK;
}

// Event pair around one launch when profiling is enabled.
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

// Encode (or reuse) the six tensor maps a TMA variant reads for one job's planes.
qmiv_status ensure_tmaps(qmiv_handle* h, int slot, DevJob& j, const CpsVariant& v, cudaStream_t st)
{
  Slot& S = h->slots[slot];
  const int sb = j.sbytes, XA = 16 / sb, R = v.rows, SR = v.sr, CS = (SR + 1) / 2;
  const int fd = (R - 1 + SR) >= 0 ? (R - 1 + SR) / 2 : -((-(R - 1 + SR) + 1) / 2);
  const uint32_t RW = 64 + 2 * XA, TH = R + 2 * SR, CRW = 32 + 2 * XA, CTH = fd + CS + 1;
  uint64_t key[16] = { 0 };
  for(int c = 0; c < 3; c++)
  {
    key[c] = (uint64_t)(uintptr_t)j.p0[c]; key[3 + c] = (uint64_t)(uintptr_t)j.p1[c];
    key[6 + c] = ((uint64_t)(uint32_t)j.stride0[c] << 32) | (uint32_t)j.stride1[c];
  }
  key[9] = ((uint64_t)(uint32_t)j.W << 32) | (uint32_t)j.H;
  key[10] = ((uint64_t)RW << 48) | ((uint64_t)TH << 32) | ((uint64_t)CRW << 16) | CTH;
  key[11] = (uint64_t)sb;
  j.tmaps = S.d_tmaps;
  if(S.tmap_valid && std::memcmp(key, S.tmap_key, sizeof(key)) == 0) return QMIV_OK;
  EncodeTiledFn enc = encode_fn();
  if(!enc) return fail(QMIV_CUDA_ERROR, "cuTensorMapEncodeTiled unavailable");
  alignas(64) CUtensorMap maps[6];
  for(int pic = 0; pic < 2; pic++)
    for(int c = 0; c < 3; c++)
    {
      const void* base = pic == 0 ? j.p0[c] : j.p1[c];
      const int stride = pic == 0 ? j.stride0[c] : j.stride1[c];
      const cuuint64_t dims[2] = { (cuuint64_t)(c ? j.W / 2 : j.W), (cuuint64_t)(c ? j.H / 2 : j.H) };
      const cuuint64_t strides[1] = { (cuuint64_t)stride * sb };
      const cuuint32_t box[2] = { c ? CRW : RW, c ? CTH : TH };
      const cuuint32_t estr[2] = { 1, 1 };
      CUresult r = enc(&maps[pic * 3 + c], sb == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 2,
                       const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                       CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      if(r != CUDA_SUCCESS) { S.tmap_valid = false; return fail(QMIV_CUDA_ERROR, "cuTensorMapEncodeTiled failed (%d)", (int)r); }
    }
  CUDA_TRY(cudaMemcpyAsync(S.d_tmaps, maps, sizeof(maps), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaStreamSynchronize(st)); // `maps` lives on this stack frame
  std::memcpy(S.tmap_key, key, sizeof(key));
  S.tmap_valid = true;
  return QMIV_OK;
}

// Run stats + CPS for n jobs already in h->h_jobs[0..n) (slots 0..n).
qmiv_status run_psnr_family(qmiv_handle* h, int n, cudaStream_t st)
{
  std::vector<int> var(n);
  for(int i = 0; i < n; i++) var[i] = (h->h_jobs[i].metrics & (QMIV_M_IVPSNR | QMIV_M_IVSSIM)) ? pick_cps_variant(h, h->h_jobs[i]) : -1;
  // order jobs by CPS variant so each variant's jobs are contiguous
  std::vector<int> order(n);
  for(int i = 0; i < n; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return var[a] < var[b]; });
  std::vector<DevJob> sorted(n);
  std::vector<int> svar(n);
  for(int i = 0; i < n; i++) { sorted[i] = h->h_jobs[order[i]]; svar[i] = var[order[i]] < 0 ? 0 : var[order[i]]; }
  plan_grid(h, sorted.data(), n, svar);
  // CPS bases per variant group
  int first = 0;
  while(first < n)
  {
    int last = first;
    while(last + 1 < n && var[order[last + 1]] == var[order[first]]) last++;
    int base = 0;
    for(int i = first; i <= last; i++) { sorted[i].cps_base = base; base += (var[order[i]] < 0) ? 0 : sorted[i].cps_strips * sorted[i].cps_segs; }
    first = last + 1;
  }
  for(int i = 0; i < n; i++)
  {
    if(var[order[i]] > 0 && variants()[var[order[i]]].kind == 2)
    {
      qmiv_status ts = ensure_tmaps(h, order[i], sorted[i], variants()[var[order[i]]], st);
      if(ts != QMIV_OK) return ts;
    }
  }
  std::memcpy(h->h_jobs, sorted.data(), sizeof(DevJob) * n);
  CUDA_TRY(cudaMemcpyAsync(h->d_jobs, h->h_jobs, sizeof(DevJob) * n, cudaMemcpyHostToDevice, st));
  h->prof_n = 0;
  CUDA_TRY(prof_mark(h, "k_stats", st, true));
  CUDA_TRY(launch_stats(h->d_jobs, h->h_jobs, n, h->params, st));
  CUDA_TRY(prof_mark(h, "k_stats", st, false));
  h->launches++;
  first = 0;
  while(first < n)
  {
    int last = first;
    while(last + 1 < n && var[order[last + 1]] == var[order[first]]) last++;
    if(var[order[first]] >= 0)
    {
      const CpsVariant& cv = variants()[var[order[first]]];
      int blocks = 0;
      for(int i = first; i <= last; i++) blocks = h->h_jobs[i].cps_base + h->h_jobs[i].cps_strips * h->h_jobs[i].cps_segs;
      CUDA_TRY(prof_mark(h, cv.name, st, true));
      if(blocks > 0) CUDA_TRY(cv.launch(h->d_jobs + first, last - first + 1, blocks, h->params, st));
      CUDA_TRY(prof_mark(h, nullptr, st, false));
      h->launches++;
    }
    first = last + 1;
  }
  return QMIV_OK;
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

  const size_t rows_b = (size_t)max_h * 6 * sizeof(int64_t);
  const size_t cps_b = (size_t)2 * max_h * 3 * sizeof(unsigned long long);
  const size_t sc_b = (sizeof(JobScalars) + 255) & ~(size_t)255;
  const size_t tm_b = 6 * 128;
  const size_t per = ((rows_b + 255) & ~(size_t)255) + ((cps_b + 255) & ~(size_t)255) + sc_b + tm_b;
  if(cudaMalloc(&h->slot_mem, per * max_jobs) != cudaSuccess) return cleanup(fail(QMIV_OUT_OF_MEMORY, "slot scratch %zu B", per * max_jobs));
  if(cudaMemset(h->slot_mem, 0, per * max_jobs) != cudaSuccess) return cleanup(fail(QMIV_CUDA_ERROR, "memset"));
  h->slots.resize(max_jobs);
  for(int i = 0; i < max_jobs; i++)
  {
    uint8_t* b = (uint8_t*)h->slot_mem + per * i;
    h->slots[i].stat_rows = (int64_t*)b; b += (rows_b + 255) & ~(size_t)255;
    h->slots[i].cps_rows = (unsigned long long*)b; b += (cps_b + 255) & ~(size_t)255;
    h->slots[i].sc = (JobScalars*)b; b += sc_b;
    h->slots[i].d_tmaps = b;
  }
  if(cudaMalloc(&h->d_jobs, sizeof(DevJob) * max_jobs) != cudaSuccess) return cleanup(fail(QMIV_OUT_OF_MEMORY, "job table"));
  if(cudaMallocHost(&h->h_jobs, sizeof(DevJob) * max_jobs) != cudaSuccess) return cleanup(fail(QMIV_OUT_OF_MEMORY, "pinned job table"));
  if(cudaMalloc(&h->d_results, sizeof(qmiv_frame_result) * max_jobs) != cudaSuccess) return cleanup(fail(QMIV_OUT_OF_MEMORY, "results"));
  if(cudaMallocHost(&h->h_results, sizeof(qmiv_frame_result) * max_jobs) != cudaSuccess) return cleanup(fail(QMIV_OUT_OF_MEMORY, "pinned results"));
  h->stage_elems = (size_t)max_w * max_h * 3 + 64;
  for(int i = 0; i < 2; i++)
  {
    if(cudaMalloc(&h->d_stage[i], h->stage_elems * sizeof(uint16_t)) != cudaSuccess) return cleanup(fail(QMIV_OUT_OF_MEMORY, "staging"));
    if(cudaMalloc(&h->d_scp[i], (size_t)max_w * max_h * 3 * sizeof(uint16_t)) != cudaSuccess) return cleanup(fail(QMIV_OUT_OF_MEMORY, "scp"));
  }
  if(cudaDeviceSynchronize() != cudaSuccess) return cleanup(fail(QMIV_CUDA_ERROR, "create sync"));
  *out = h;
  return QMIV_OK;
}

qmiv_status qmiv_destroy(qmiv_handle* h)
{
  if(!h) return QMIV_OK;
  cudaFree(h->slot_mem);
  cudaFree(h->d_jobs);
  cudaFreeHost(h->h_jobs);
  cudaFree(h->d_results);
  cudaFreeHost(h->h_results);
  for(int i = 0; i < 2; i++) { cudaFree(h->d_stage[i]); cudaFree(h->d_scp[i]); }
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
                                const int32_t* gcd_given, uint16_t* scp0[3], uint16_t* scp1[3], int32_t scp_stride,
                                qmiv_frame_result* out, cudaStream_t st)
{
  if(!h) return fail(QMIV_BAD_ARG, "handle is null");
  qmiv_status s = check_pair(h, pic0, pic1);
  if(s != QMIV_OK) return s;
  if(metrics & ~QMIV_M_ALL) return fail(QMIV_BAD_ARG, "metrics 0x%x", metrics);
  qmiv_pic a, b;
  if((s = upload_pic(h, pic0, 0, &a, st)) != QMIV_OK) return s;
  if((s = upload_pic(h, pic1, 1, &b, st)) != QMIV_OK) return s;
  DevJob& j = h->h_jobs[0];
  fill_job(h, j, &a, &b, metrics | QMIV_M_PSNR, 0);
  j.use_ws = h->opt.use_ws;
  if(j.use_ws) { if((s = ws_weights(h, j.H, &j.ws, &j.ws_corr)) != QMIV_OK) return s; }
  for(int c = 0; c < 3; c++) { j.scp0[c] = scp0 ? scp0[c] : nullptr; j.scp1[c] = scp1 ? scp1[c] : nullptr; }
  j.scp_stride = scp_stride;
  if(gcd_given)
  {
    JobScalars tmp;
    std::memset(&tmp, 0, sizeof(tmp));
    for(int c = 0; c < 3; c++) tmp.gcd[c] = gcd_given[c];
    CUDA_TRY(cudaMemcpyAsync(h->slots[0].sc->gcd, tmp.gcd, sizeof(tmp.gcd), cudaMemcpyHostToDevice, st));
    j.gcd_given = 1;
  }
  CUDA_TRY(cudaMemsetAsync(h->d_results, 0, sizeof(qmiv_frame_result), st));
  if((s = run_psnr_family(h, 1, st)) != QMIV_OK) return s;
  CUDA_TRY(cudaMemcpyAsync(h->h_results, h->d_results, sizeof(qmiv_frame_result), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  *out = h->h_results[0];
  out->metrics = metrics;
  return QMIV_OK;
}

qmiv_status qmiv_calc_frame(qmiv_handle* h, const qmiv_pic* pic0, const qmiv_pic* pic1, uint32_t metrics,
                            qmiv_frame_result* out, qmiv_stream stream)
{
  if(!out) return fail(QMIV_BAD_ARG, "out is null");
  cudaStream_t st = (cudaStream_t)stream;
  const bool need_scp = (metrics & QMIV_M_IVSSIM) != 0;
  uint16_t* s0[3] = { nullptr, nullptr, nullptr };
  uint16_t* s1[3] = { nullptr, nullptr, nullptr };
  int32_t sstride = 0;
  if(need_scp && pic0)
  {
    const size_t area = (size_t)pic0->width * pic0->height;
    for(int c = 0; c < 3; c++) { s0[c] = h->d_scp[0] + c * area; s1[c] = h->d_scp[1] + c * area; }
    sstride = pic0->width;
  }
  qmiv_status s = frame_common(h, pic0, pic1, metrics, nullptr, need_scp ? s0 : nullptr, need_scp ? s1 : nullptr, sstride, out, st);
  if(s != QMIV_OK) return s;
  // sequence statistics (xMetricStat::setPerCmpMeric / setPerPicMeric)
  SeqAcc& q = h->seq;
  if(metrics & QMIV_M_PSNR)   { for(int c = 0; c < 3; c++) q.v[c].push_back(out->psnr[c]);   q.v[3].push_back(out->psnr_pic); }
  if(metrics & QMIV_M_WSPSNR) { for(int c = 0; c < 3; c++) q.v[4 + c].push_back(out->wspsnr[c]); q.v[7].push_back(out->wspsnr_pic); }
  if(metrics & QMIV_M_IVPSNR) q.v[8].push_back(out->ivpsnr);
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
  if(!scp0 || !scp1) return fail(QMIV_BAD_ARG, "scp outputs are null");
  for(int c = 0; c < 3; c++) if(!scp0[c] || !scp1[c]) return fail(QMIV_BAD_ARG, "scp plane %d is null", c);
  if(!pic0) return fail(QMIV_BAD_ARG, "pic0 is null");
  if(scp_stride < pic0->width) return fail(QMIV_BAD_ARG, "scp_stride %d < width %d", scp_stride, pic0->width);
  cudaStream_t st = (cudaStream_t)stream;
  uint16_t* d0[3]; uint16_t* d1[3];
  const size_t area = (size_t)pic0->width * pic0->height;
  int32_t dstride = scp_stride;
  if(scp_is_device) { for(int c = 0; c < 3; c++) { d0[c] = scp0[c]; d1[c] = scp1[c]; } }
  else
  {
    if(pic0->width > h->max_w || pic0->height > h->max_h) return fail(QMIV_TOO_LARGE, "picture too large");
    for(int c = 0; c < 3; c++) { d0[c] = h->d_scp[0] + c * area; d1[c] = h->d_scp[1] + c * area; }
    dstride = pic0->width;
  }
  qmiv_frame_result r;
  qmiv_status s = frame_common(h, pic0, pic1, QMIV_M_IVSSIM, gcd, d0, d1, dstride, &r, st);
  if(s != QMIV_OK) return s;
  if(!scp_is_device)
  {
    for(int c = 0; c < 3; c++)
    {
      CUDA_TRY(cudaMemcpy2DAsync(scp0[c], (size_t)scp_stride * 2, d0[c], (size_t)dstride * 2, (size_t)pic0->width * 2, pic0->height, cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaMemcpy2DAsync(scp1[c], (size_t)scp_stride * 2, d1[c], (size_t)dstride * 2, (size_t)pic0->width * 2, pic0->height, cudaMemcpyDeviceToHost, st));
    }
    CUDA_TRY(cudaStreamSynchronize(st));
  }
  return QMIV_OK;
}

qmiv_status qmiv_calc_batch(qmiv_handle* h, const qmiv_job* jobs, int32_t n, qmiv_frame_result* results, qmiv_stream stream)
{
  if(!h) return fail(QMIV_BAD_ARG, "handle is null");
  if(!jobs || n < 1) return fail(QMIV_BAD_ARG, "no jobs");
  if(n > h->max_jobs) return fail(QMIV_TOO_LARGE, "%d jobs > max_jobs %d", n, h->max_jobs);
  if(!results) return fail(QMIV_BAD_ARG, "results is null");
  cudaStream_t st = (cudaStream_t)stream;
  for(int i = 0; i < n; i++)
  {
    const qmiv_job& jb = jobs[i];
    qmiv_status s = check_pair(h, &jb.pic0, &jb.pic1);
    if(s != QMIV_OK) return fail(s, "job %d: %s", i, g_last_error.c_str());
    if(!jb.pic0.is_device) return fail(QMIV_BAD_ARG, "job %d: batch pictures must be device pointers", i);
    if(jb.metrics & ~QMIV_M_ALL) return fail(QMIV_BAD_ARG, "job %d: metrics 0x%x", i, jb.metrics);
    if(jb.metrics & (QMIV_M_SSIM | QMIV_M_MSSSIM | QMIV_M_IVSSIM)) return fail(QMIV_UNSUPPORTED, "job %d: SSIM metrics in batches", i);
    DevJob& j = h->h_jobs[i];
    fill_job(h, j, &jb.pic0, &jb.pic1, jb.metrics | QMIV_M_PSNR, i);
    j.result = results + i;
    j.use_ws = jb.use_ws;
    if(j.use_ws) { s = ws_weights(h, j.H, &j.ws, &j.ws_corr); if(s != QMIV_OK) return s; }
    for(int c = 0; c < 3; c++) { j.scp0[c] = jb.scp0[c]; j.scp1[c] = jb.scp1[c]; }
    j.scp_stride = jb.scp_stride;
  }
  return run_psnr_family(h, n, st);
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
  for(int k = 0; k < 16; k++) nf = std::max(nf, q.v[k].size());
  out->num_frames = (int32_t)nf;
  for(int c = 0; c < 3; c++) { out->psnr[c] = avg(q.v[c]); out->wspsnr[c] = avg(q.v[4 + c]); out->ssim[c] = avg(q.v[9 + c]); out->msssim[c] = avg(q.v[13 + c]); }
  out->psnr_pic = avg(q.v[3]); out->wspsnr_pic = avg(q.v[7]); out->ivpsnr = avg(q.v[8]);
  out->ssim_pic = avg(q.v[12]);
  if(!q.v[3].empty()) out->metrics |= QMIV_M_PSNR;
  if(!q.v[7].empty()) out->metrics |= QMIV_M_WSPSNR;
  if(!q.v[8].empty()) out->metrics |= QMIV_M_IVPSNR;
  return QMIV_OK;
}

qmiv_status qmiv_reset_sequence(qmiv_handle* h)
{
  if(!h) return fail(QMIV_BAD_ARG, "handle is null");
  for(auto& v : h->seq.v) v.clear();
  return QMIV_OK;
}

// SSIM family: provided by the SSIM translation unit once built; until then these report
// UNSUPPORTED so callers fail loudly instead of silently skipping work.
qmiv_status qmiv_ssim(qmiv_handle* h, const qmiv_pic*, const qmiv_pic*, int32_t, double*, qmiv_stream)
{ return h ? fail(QMIV_UNSUPPORTED, "SSIM not built") : fail(QMIV_BAD_ARG, "handle is null"); }
qmiv_status qmiv_msssim(qmiv_handle* h, const qmiv_pic*, const qmiv_pic*, double*, qmiv_stream)
{ return h ? fail(QMIV_UNSUPPORTED, "MS-SSIM not built") : fail(QMIV_BAD_ARG, "handle is null"); }
qmiv_status qmiv_ivssim(qmiv_handle* h, const qmiv_pic*, const qmiv_pic*, const int32_t*, double*, double*, double*, qmiv_stream)
{ return h ? fail(QMIV_UNSUPPORTED, "IV-SSIM not built") : fail(QMIV_BAD_ARG, "handle is null"); }

}  // extern "C"
