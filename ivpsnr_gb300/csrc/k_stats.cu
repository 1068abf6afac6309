// Picture statistics kernel: per-row sums of differences and squared differences of the
// two input pictures, read once from their native layout (8/16-bit, 4:2:0 or 4:4:4).
// Its last block per job turns the rows into
//   * the global colour difference GCD_R2T (libs/pmbb-ivqm/src/xGlobClrDiff.cpp:15-48 with
//     the application's argument order, xGlobClrDiff.h:41),
//   * PSNR (xPSNR.cpp:17-36,93-111,139-146) with the application's exact-component
//     replacement (apps/QMIV/src/xAppQMIV.cpp:837-844),
//   * WS-PSNR (xWSPSNR.cpp:17-48,101-125).
// HBM-bound: each sample of both pictures is read once (1.5 samples per luma pixel for
// 4:2:0). For 4:2:0 the chroma sums of the 4:4:4 picture the reference works on are exact
// multiples of the native chroma sums (each chroma sample is replicated 2x2,
// xPixelOpsSTD.cpp:30-49), so the upsampled planes are never formed.
#include <cstddef>
#include <mutex>

#include "qmiv_device.cuh"

namespace qmiv {

namespace {

constexpr int kStatsThreads = 256;
constexpr int kRowPairsPerBlock = kStatsThreads / 32; // one warp per pair of luma rows

// Differences of the samples packed in two 32-bit words (2 x 16-bit or 4 x 8-bit): their sum
// into sd, the sum of their squares into q. Lanes are taken out with shifts and masks, so the
// loaded vectors stay in registers.
template <typename T>
__device__ __forceinline__ void word_stats(uint32_t a, uint32_t b, int& sd, unsigned int& q)
{
  if(sizeof(T) == 2)
  {
    const int d0 = (int)(a & 0xFFFFu) - (int)(b & 0xFFFFu), d1 = (int)(a >> 16) - (int)(b >> 16);
    sd += d0 + d1;
    q += (unsigned)(d0 * d0) + (unsigned)(d1 * d1);
  }
  else
  { // sum of |d|^2 as a byte dot product of the absolute differences with themselves
    const unsigned ad = __vabsdiffu4(a, b);
    q = __dp4a(ad, ad, q);
    sd += (int)__dp4a(a, 0x01010101u, 0u) - (int)__dp4a(b, 0x01010101u, 0u);
  }
}

// sum(a-b) and sum((a-b)^2) over n samples of two rows, one warp, 16-byte loads when aligned
template <typename T>
__device__ __forceinline__ void row_stats(const T* __restrict__ a, const T* __restrict__ b, int n, bool vec, int lane,
                                          int& sd, unsigned long long& ssd)
{
  int i0 = 0;
  if(vec)
  {
    constexpr int V = 16 / sizeof(T);
    const int nv = n / V;
    const uint4* av = reinterpret_cast<const uint4*>(a);
    const uint4* bv = reinterpret_cast<const uint4*>(b);
    #pragma unroll 4
    for(int i = lane; i < nv; i += 32)
    {
      const uint4 x = __ldg(av + i), y = __ldg(bv + i);
      unsigned int q = 0;
      word_stats<T>(x.x, y.x, sd, q);
      word_stats<T>(x.y, y.y, sd, q);
      word_stats<T>(x.z, y.z, sd, q);
      word_stats<T>(x.w, y.w, sd, q);
      ssd += q;
    }
    i0 = nv * V;
  }
  for(int i = i0 + lane; i < n; i += 32)
  {
    const int d = (int)a[i] - (int)b[i];
    sd += d; ssd += (unsigned long long)(d * d);
  }
}

template <typename T>
__device__ __forceinline__ void stats_rowpair(const DevJob& J, int y, bool vec, int lane, int (&sd)[2][3],
                                              unsigned long long (&ssd)[2][3])
{ // every loop unrolled, so that the accumulators stay in registers
  const bool two = y + 1 < J.H;
  #pragma unroll
  for(int r = 0; r < 2; r++)
    if(r == 0 || two)
      row_stats<T>((const T*)J.p1[0] + (int64_t)(y + r) * J.stride1[0], (const T*)J.p0[0] + (int64_t)(y + r) * J.stride0[0],
                   J.W, vec, lane, sd[r][0], ssd[r][0]);
  if(J.cshift)
  { // one chroma row serves luma rows y and y+1
    const int cy = y >> 1, cw = J.W >> 1;
    #pragma unroll
    for(int c = 1; c < 3; c++)
      row_stats<T>((const T*)J.p1[c] + (int64_t)cy * J.stride1[c], (const T*)J.p0[c] + (int64_t)cy * J.stride0[c], cw, vec,
                   lane, sd[0][c], ssd[0][c]);
  }
  else
  {
    #pragma unroll
    for(int r = 0; r < 2; r++)
      #pragma unroll
      for(int c = 1; c < 3; c++)
        if(r == 0 || two)
          row_stats<T>((const T*)J.p1[c] + (int64_t)(y + r) * J.stride1[c], (const T*)J.p0[c] + (int64_t)(y + r) * J.stride0[c],
                       J.W, vec, lane, sd[r][c], ssd[r][c]);
  }
}

__device__ bool vec_ok(const DevJob& J)
{
  const int sb = J.sbytes;
  for(int c = 0; c < 3; c++)
  {
    if((((uintptr_t)J.p0[c]) | ((uintptr_t)J.p1[c])) & 15) return false;
    if(((J.stride0[c] * sb) | (J.stride1[c] * sb)) & 15) return false;
  }
  return true;
}

// Last block of a job: GCD, exact flags, PSNR, WS-PSNR.
__device__ void finalize_stats(const DevJob& J, const Params& p, double* scratch)
{
  __shared__ long long s_sd[3];
  __shared__ unsigned long long s_ssd[3];
  const int64_t area = (int64_t)J.W * J.H;
  for(int c = 0; c < 3; c++)
  {
    long long sd = 0; unsigned long long ssd = 0;
    for(int y = threadIdx.x; y < J.H; y += blockDim.x)
    {
      sd  += __ldcg(J.stat_rows + (int64_t)y * 6 + c);
      ssd += (unsigned long long)__ldcg(J.stat_rows + (int64_t)y * 6 + 3 + c);
    }
    sd = warp_sum(sd); ssd = warp_sum(ssd);
    __syncthreads();
    if((threadIdx.x & 31) == 0) { scratch[2 * (threadIdx.x >> 5)] = __longlong_as_double(sd); scratch[2 * (threadIdx.x >> 5) + 1] = __longlong_as_double((long long)ssd); }
    __syncthreads();
    if(threadIdx.x == 0)
    {
      long long a = 0; unsigned long long b = 0;
      for(int w = 0; w < (int)(blockDim.x >> 5); w++) { a += __double_as_longlong(scratch[2 * w]); b += (unsigned long long)__double_as_longlong(scratch[2 * w + 1]); }
      s_sd[c] = a; s_ssd[c] = b;
    }
    __syncthreads();
  }

  double ws[3] = { 0, 0, 0 };
  if(J.use_ws && (J.metrics & QMIV_M_WSPSNR))
  {
    for(int c = 0; c < 3; c++)
    {
      Kbns k = { 0.0, 0.0 };
      for(int y = threadIdx.x; y < J.H; y += blockDim.x)
        k = kbns_add(k, __dmul_rn((double)(unsigned long long)__ldcg(J.stat_rows + (int64_t)y * 6 + 3 + c), J.ws[y]));
      ws[c] = block_kbns(k, scratch);
    }
  }

  if(threadIdx.x == 0)
  {
    qmiv_frame_result* R = J.result;
    const int mx = (1 << J.bd) - 1;
    int32_t g[4] = { 0, 0, 0, 0 };
    for(int c = 0; c < 3; c++)
    { // rne(sum / area) clipped to +-rne_f32(unc*Max) (xGlobClrDiff.cpp:21,43-45)
      const int md = p.maxdiff_for_bd[J.bd][c];
      int v = __double2int_rn(__ddiv_rn((double)s_sd[c], (double)area));
      g[c] = v < -md ? -md : (v > md ? md : v);
    }
    if(!J.gcd_given) { for(int c = 0; c < 4; c++) J.sc->gcd[c] = g[c]; }
    J.sc->status = 0;
    R->status = 0;
    double ps[3], wp[3];
    const double fake = psnr_from_ssd(1.0, area, J.bd);
    for(int c = 0; c < 3; c++)
    {
      const bool exact = s_ssd[c] == 0;
      R->exact[c] = exact;
      ps[c] = psnr_from_ssd((double)s_ssd[c], area, J.bd);
      if(J.use_ws) { const double e = __dmul_rn(ws[c], J.ws_corr); wp[c] = psnr_from_ssd(e, area, J.bd); }
      else wp[c] = ps[c];
      if(exact && p.fake_exact) { ps[c] = fake; wp[c] = fake; }
    }
    if(J.use_ws && p.legacy_ws8 && J.bd == 10)
    { // xWSPSNR.cpp:34-46
      const double real = (double)mx, fk = (double)(255 << 2);
      const double mod = __dmul_rn(10.0, __dsub_rn(log10(__dmul_rn(real, real)), log10(__dmul_rn(fk, fk))));
      for(int c = 0; c < 3; c++) wp[c] = __dsub_rn(wp[c], mod);
    }
    R->exact[3] = 0;
    for(int c = 0; c < 4; c++) R->gcd_r2t[c] = J.gcd_given ? J.sc->gcd[c] : g[c];
    if(J.metrics & QMIV_M_PSNR)   { for(int c = 0; c < 3; c++) R->psnr[c] = ps[c];   R->psnr[3] = 0;   R->psnr_pic = weighted3(ps, p.w_avg); }
    if(J.metrics & QMIV_M_WSPSNR) { for(int c = 0; c < 3; c++) R->wspsnr[c] = wp[c]; R->wspsnr[3] = 0; R->wspsnr_pic = weighted3(wp, p.w_avg); }
    __threadfence();
    J.sc->stats_done = 0; // self-reset for the next use of this job slot
  }
}

}  // namespace

__global__ void __launch_bounds__(kStatsThreads) k_stats(const DevJob* __restrict__ jobs, int njobs, Params p)
{
  __shared__ double scratch[2 * (kStatsThreads / 32)];
  __shared__ bool is_last;
  const int j = find_job<0>(jobs, njobs, blockIdx.x);
  const DevJob& J = jobs[j];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int y = 2 * ((blockIdx.x - J.stat_base) * kRowPairsPerBlock + w);

  if(y < J.H)
  {
    int sd[2][3] = { { 0, 0, 0 }, { 0, 0, 0 } };
    unsigned long long ssd[2][3] = { { 0, 0, 0 }, { 0, 0, 0 } };
    const bool vec = vec_ok(J);
    if(J.sbytes == 1) stats_rowpair<uint8_t>(J, y, vec, lane, sd, ssd);
    else              stats_rowpair<uint16_t>(J, y, vec, lane, sd, ssd);
    long long v[2][6];
    #pragma unroll
    for(int r = 0; r < 2; r++)
      #pragma unroll
      for(int c = 0; c < 3; c++)
      {
        v[r][c] = (long long)__reduce_add_sync(0xffffffffu, (unsigned)sd[r][c]);
        v[r][c] = (long long)(int)v[r][c];
        v[r][3 + c] = (long long)warp_sum(ssd[r][c]);
      }
    if(lane < 12)
    { // lane = r*6 + q: rows y, y+1; q: sd[3], ssd[3]; a chroma row counts 2x per luma row (4:2:0)
      const int r = lane / 6, q = lane % 6, c = q % 3;
      const bool chroma420 = J.cshift && c > 0;
      long long val = 0;
      #pragma unroll
      for(int rr = 0; rr < 2; rr++)
        #pragma unroll
        for(int qq = 0; qq < 6; qq++)
          if(qq == q && rr == (chroma420 ? 0 : r)) val = v[rr][qq];
      if(y + r < J.H) J.stat_rows[(int64_t)(y + r) * 6 + q] = chroma420 ? 2 * val : val;
    }
    // zero this row pair's CPS accumulators for the CPS kernel that follows
    if((J.metrics & (QMIV_M_IVPSNR | QMIV_M_IVSSIM)) && lane >= 16 && lane < 28)
    {
      const int t = lane - 16, dir = t / 6, r = (t % 6) / 3, c = t % 3;
      if(y + r < J.H) J.cps_rows[((int64_t)dir * J.H + y + r) * 3 + c] = 0ull;
    }
  }

  __threadfence();
  __syncthreads();
  if(threadIdx.x == 0) is_last = atomicAdd(&J.sc->stats_done, 1u) == (unsigned)(J.stat_blocks - 1);
  __syncthreads();
  if(is_last)
  {
    __threadfence();
    finalize_stats(J, p, scratch);
  }
}

// Every job's result entry cleared and stamped with its metric set before the metric kernels
// write their fields, so that the fields of metrics not requested read as zero.
__global__ void __launch_bounds__(256) k_init_results(const DevJob* __restrict__ jobs, int n)
{
  constexpr int kWords = (int)(sizeof(qmiv_frame_result) / 4);
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n * kWords; i += gridDim.x * blockDim.x)
  {
    const int j = i / kWords, w = i - j * kWords;
    reinterpret_cast<uint32_t*>(jobs[j].result)[w] = w == 0 ? jobs[j].metrics : 0u;
  }
}

// A call's tables copied from page-locked host memory by the SMs, not the copy engine: a copy
// engine runs its copies in order, so a small table copy would otherwise wait behind large
// picture uploads queued earlier on another stream.
__global__ void __launch_bounds__(256) k_copy_table(const uint4* __restrict__ src, uint4* __restrict__ dst, int n16)
{
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += gridDim.x * blockDim.x) dst[i] = src[i];
}

cudaError_t launch_copy_table(const void* src, void* dst, size_t bytes, cudaStream_t st)
{
  const int n16 = (int)(bytes / 16);
  if(n16 == 0) return cudaSuccess;
  k_copy_table<<<std::min(152, (n16 + 255) / 256), 256, 0, st>>>(static_cast<const uint4*>(src), static_cast<uint4*>(dst), n16);
  return cudaGetLastError();
}

cudaError_t launch_init_results(const DevJob* d_jobs, int n, cudaStream_t st)
{
  static_assert(sizeof(qmiv_frame_result) % 4 == 0 && offsetof(qmiv_frame_result, metrics) == 0, "result layout");
  const int words = n * (int)(sizeof(qmiv_frame_result) / 4);
  k_init_results<<<std::min(64, (words + 255) / 256), 256, 0, st>>>(d_jobs, n);
  return cudaGetLastError();
}

cudaError_t launch_stats(const DevJob* d_jobs, const DevJob* h_jobs, int n, const Params& p, cudaStream_t st)
{
  int blocks = 0;
  for(int i = 0; i < n; i++) blocks = h_jobs[i].stat_base + h_jobs[i].stat_blocks;
  if(blocks == 0) return cudaSuccess;
  k_stats<<<blocks, kStatsThreads, 0, st>>>(d_jobs, n, p);
  return cudaGetLastError();
}

// ---- statistics without any allocation --------------------------------------------------
// The same per-row statistics and last-block finalisation for one picture pair, with the job
// passed by value (no device job table) and the per-row sums, the counters and the result in
// one static device array instead of a handle's scratch. It serves callers that cannot
// allocate device memory at the point of the call.

namespace {

constexpr size_t kStaticRowsBytes = (size_t)kStaticMaxRows * 6 * sizeof(int64_t);
constexpr size_t kStaticScalarsOff = kStaticRowsBytes;
constexpr size_t kStaticResultOff = kStaticScalarsOff + ((sizeof(JobScalars) + 255) & ~(size_t)255);
constexpr size_t kStaticBytes = kStaticResultOff + ((sizeof(qmiv_frame_result) + 255) & ~(size_t)255);

// ~385 KiB: [kStaticMaxRows][6] row sums, then JobScalars, then the frame result
static __device__ __align__(256) unsigned char g_stats_scratch[kStaticBytes];

__global__ void __launch_bounds__(kStatsThreads) k_stats_static(const DevJob J, Params p)
{
  __shared__ double scratch[2 * (kStatsThreads / 32)];
  __shared__ bool is_last;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int y = 2 * (blockIdx.x * kRowPairsPerBlock + w);

  if(y < J.H)
  {
    int sd[2][3] = { { 0, 0, 0 }, { 0, 0, 0 } };
    unsigned long long ssd[2][3] = { { 0, 0, 0 }, { 0, 0, 0 } };
    const bool vec = vec_ok(J);
    if(J.sbytes == 1) stats_rowpair<uint8_t>(J, y, vec, lane, sd, ssd);
    else              stats_rowpair<uint16_t>(J, y, vec, lane, sd, ssd);
    long long v[2][6];
    #pragma unroll
    for(int r = 0; r < 2; r++)
      #pragma unroll
      for(int c = 0; c < 3; c++)
      {
        v[r][c] = (long long)(int)__reduce_add_sync(0xffffffffu, (unsigned)sd[r][c]);
        v[r][3 + c] = (long long)warp_sum(ssd[r][c]);
      }
    if(lane < 12)
    {
      const int r = lane / 6, q = lane % 6, c = q % 3;
      const bool chroma420 = J.cshift && c > 0;
      long long val = 0;
      #pragma unroll
      for(int rr = 0; rr < 2; rr++)
        #pragma unroll
        for(int qq = 0; qq < 6; qq++)
          if(qq == q && rr == (chroma420 ? 0 : r)) val = v[rr][qq];
      if(y + r < J.H) J.stat_rows[(int64_t)(y + r) * 6 + q] = chroma420 ? 2 * val : val;
    }
  }

  __threadfence();
  __syncthreads();
  if(threadIdx.x == 0) is_last = atomicAdd(&J.sc->stats_done, 1u) == (unsigned)(J.stat_blocks - 1);
  __syncthreads();
  if(is_last)
  {
    __threadfence();
    finalize_stats(J, p, scratch);
  }
}

int g_static_ready[kStaticMaxDevices];
StaticStatsScratch g_static_ptrs[kStaticMaxDevices];
std::mutex g_static_mu;

}  // namespace

cudaError_t stats_static_scratch(StaticStatsScratch* out)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if(e != cudaSuccess) return e;
  if(dev < 0 || dev >= kStaticMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_static_mu);
  if(!g_static_ready[dev])
  { // once per device, with that device current: the address of this module's static array
    unsigned char* base = nullptr;
    e = cudaGetSymbolAddress((void**)&base, g_stats_scratch);
    if(e != cudaSuccess) return e;
    g_static_ptrs[dev].stat_rows = reinterpret_cast<int64_t*>(base);
    g_static_ptrs[dev].sc = reinterpret_cast<JobScalars*>(base + kStaticScalarsOff);
    g_static_ptrs[dev].result = reinterpret_cast<qmiv_frame_result*>(base + kStaticResultOff);
    g_static_ready[dev] = 1;
  }
  *out = g_static_ptrs[dev];
  return cudaSuccess;
}

cudaError_t launch_stats_static(const DevJob& j, const Params& p, cudaStream_t st)
{
  if(j.stat_blocks == 0) return cudaSuccess;
  k_stats_static<<<j.stat_blocks, kStatsThreads, 0, st>>>(j, p);
  return cudaGetLastError();
}

}  // namespace qmiv
