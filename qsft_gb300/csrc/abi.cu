// Library-level entry points: version, status strings, workspace layout,
// result collection and the batched Reed-Solomon decoder.
#include <stdio.h>

#include <atomic>
#include <mutex>

#include "common.cuh"
#include "rs.cuh"

namespace qsft {

// one block per job: compact the recorded balls (count > 0) into the output.
// 1024 threads, positions taken a warp at a time (one shared atomic per warp)
// and k rows copied 16 bytes at a time when the buffers and kstride allow
constexpr int COLLECT_THREADS = 1024;
__global__ void __launch_bounds__(COLLECT_THREADS) collect_kernel(qsft_plan plan, uint8_t* out_k, double* out_val,
                                                                  int32_t* out_cnt, int64_t* out_index,
                                                                  unsigned long long* out_total) {
  const int jid = blockIdx.x;
  const qsft_job* job = plan.jobs + jid;
  const int nb = min(plan.ctrl[jid].n_balls, job->ball_cap);
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  __shared__ int count;
  __shared__ int pos;
  __shared__ unsigned long long start;
  if (threadIdx.x == 0) {
    count = 0;
    pos = 0;
  }
  __syncthreads();
  for (int i0 = 0; i0 < nb; i0 += blockDim.x) {  // uniform over the warp
    const int i = i0 + threadIdx.x;
    const unsigned m = __ballot_sync(~0u, i < nb && plan.ball_cnt[job->off_ball + i] > 0);
    if (lane == 0 && m) atomicAdd(&count, __popc(m));
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    start = atomicAdd(out_total, (unsigned long long)count);
    out_index[2 * jid] = (int64_t)start;
    out_index[2 * jid + 1] = count;
  }
  __syncthreads();
  const int ks = plan.kstride;
  const bool vec = ((reinterpret_cast<uintptr_t>(out_k) | reinterpret_cast<uintptr_t>(plan.ball_k) | (uintptr_t)ks) & 15) == 0;
  for (int i0 = 0; i0 < nb; i0 += blockDim.x) {
    const int i = i0 + threadIdx.x;
    const int64_t src = job->off_ball + i;
    const int c = i < nb ? plan.ball_cnt[src] : 0;
    const unsigned m = __ballot_sync(~0u, c > 0);
    int base = 0;
    if (lane == 0 && m) base = atomicAdd(&pos, __popc(m));
    base = __shfl_sync(~0u, base, 0);
    if (c <= 0) continue;
    const int64_t row = (int64_t)start + base + __popc(m & below);
    if (vec) {
      const uint4* ks_src = reinterpret_cast<const uint4*>(plan.ball_k + src * ks);
      uint4* ks_dst = reinterpret_cast<uint4*>(out_k + row * ks);
      for (int w = 0; w < ks / 16; ++w) ks_dst[w] = ks_src[w];
    } else {
      const uint32_t* ks_src = reinterpret_cast<const uint32_t*>(plan.ball_k + src * ks);
      uint32_t* ks_dst = reinterpret_cast<uint32_t*>(out_k + row * ks);
      for (int w = 0; w < ks / 4; ++w) ks_dst[w] = ks_src[w];
    }
    out_val[2 * row] = plan.ball_sum[2 * src] / c;
    out_val[2 * row + 1] = plan.ball_sum[2 * src + 1] / c;
    out_cnt[row] = c;
  }
}

__global__ void rs_decode_kernel(int q, int s, int t, int n, const int32_t* gf_tables, const uint8_t* syms,
                                 int64_t nrows, int16_t* k_out) {
  const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= nrows) return;
  const GFt g = make_gf(gf_tables, q, s);
  uint8_t sy[256];
  uint8_t k[QSFT_MAX_N], khi[QSFT_MAX_N];
  const int ns = 2 * t * s;
  for (int i = 0; i < ns; ++i) sy[i] = syms[row * ns + i];
  rs_decode(g, q, s, t, n, sy, k, khi);
  for (int i = 0; i < n; ++i) k_out[row * n + i] = (int16_t)(k[i] + q * khi[i]);
}

static int64_t next_pow2(int64_t v) {
  int64_t p = 1;
  while (p < v) p <<= 1;
  return p;
}

static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

bool ensure_smem(const void* func, int bytes) {
  struct Entry {
    const void* f;
    int dev;
    int bytes;
  };
  static Entry table[256];
  static int used = 0;
  static std::mutex mu;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  std::lock_guard<std::mutex> lock(mu);
  for (int i = 0; i < used; ++i)
    if (table[i].f == func && table[i].dev == dev) {
      if (table[i].bytes >= bytes) return true;
      if (cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess) return false;
      table[i].bytes = bytes;
      return true;
    }
  if (cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess) return false;
  if (used < 256) table[used++] = Entry{func, dev, bytes};
  return true;
}

}  // namespace qsft

using namespace qsft;

extern "C" int qsft_abi_version(void) { return 1; }

extern "C" int64_t qsft_launch_count(void) { return (int64_t)g_launches.load(std::memory_order_relaxed); }

extern "C" int qsft_built_arch(void) {
#ifdef QSFT_ARCH
  return QSFT_ARCH;
#else
  return 0;
#endif
}

extern "C" const char* qsft_status_string(int status) {
  switch (status) {
    case QSFT_OK: return "ok";
    case QSFT_ERR_ARG: return "invalid argument";
    case QSFT_ERR_CUDA: return "CUDA error";
    case QSFT_ERR_TOO_LARGE: return "shape exceeds a compiled limit";
    case QSFT_ERR_OVERFLOW: return "device table overflow";
    case QSFT_ERR_TIMEOUT: return "a bounded device wait gave up";
    default: return "unknown status";
  }
}

extern "C" int qsft_workspace_layout(qsft_job* jobs, int njobs, int64_t* total_bins, int64_t* total_slots,
                                     int64_t* total_balls, int32_t* kstride) {
  if (!jobs || njobs <= 0 || !total_bins || !total_slots || !total_balls || !kstride) return QSFT_ERR_ARG;
  int64_t bins = 0, slots = 0, balls = 0;
  int maxw = 1;  // k row bytes: n digits, and n high parts after them for a coded source
  for (int i = 0; i < njobs; ++i) {
    qsft_job& j = jobs[i];
    if (j.q < 2 || j.q > QSFT_MAX_Q || j.n < 1 || j.n > QSFT_MAX_N || j.b < 1 || j.C < 1 || j.R < 1 || j.P < 2 ||
        j.B < 1)
      return QSFT_ERR_ARG;
    if (j.P - 1 > 256) return QSFT_ERR_TOO_LARGE;
    if (j.chan != QSFT_CHAN_IDENTITY && j.chan != QSFT_CHAN_NSO) return QSFT_ERR_ARG;
    if (j.src != QSFT_SRC_IDENTITY && j.src != QSFT_SRC_CODED) return QSFT_ERR_ARG;
    if (j.src == QSFT_SRC_IDENTITY && j.P - 1 < j.n) return QSFT_ERR_ARG;
    if (j.src == QSFT_SRC_CODED) {
      if (j.rs_t < 1 || j.rs_t > QSFT_MAX_RS_T || j.rs_s < 1 || 2 * j.rs_t * j.rs_s != j.P - 1) return QSFT_ERR_ARG;
      int64_t order = 1;
      for (int s = 0; s < j.rs_s; ++s) order *= j.q;
      if (order > QSFT_MAX_GF || j.n > order - 1) return QSFT_ERR_TOO_LARGE;
    }
    {
      int64_t bq = 1;
      for (int s = 0; s < j.b; ++s) bq *= j.q;
      if (bq != j.B || j.B > (1 << 22)) return QSFT_ERR_ARG;
    }
    const int64_t cb = (int64_t)j.C * j.B;
    if (cb >= (1LL << 31)) return QSFT_ERR_TOO_LARGE;
    j.off_bin = bins;
    j.off_slot = slots;
    j.off_ball = balls;
    j.table_cap = (int32_t)next_pow2(cb * 2 < 64 ? 64 : cb * 2);
    j.ball_cap = (int32_t)(cb + 64);
    bins += cb;
    slots += j.table_cap;
    balls += j.ball_cap;
    const int w = j.src == QSFT_SRC_CODED ? 2 * j.n : j.n;
    if (w > maxw) maxw = w;
  }
  *total_bins = bins;
  *total_slots = slots;
  *total_balls = balls;
  *kstride = (int32_t)(((maxw + 15) / 16) * 16);
  return QSFT_OK;
}

extern "C" int qsft_collect(const qsft_plan* plan, uint8_t* out_k, double* out_val, int32_t* out_cnt,
                            int64_t* out_index, int64_t* out_total, qsft_stream_t stream) {
  if (!plan || plan->njobs <= 0 || !plan->ctrl || !plan->ball_cnt || !plan->ball_k || !plan->ball_sum || !out_k ||
      !out_val || !out_cnt || !out_index || !out_total)
    return QSFT_ERR_ARG;
  if (cudaMemsetAsync(out_total, 0, sizeof(int64_t), (cudaStream_t)stream) != cudaSuccess) return QSFT_ERR_CUDA;
  collect_kernel<<<plan->njobs, COLLECT_THREADS, 0, (cudaStream_t)stream>>>(*plan, out_k, out_val, out_cnt, out_index,
                                                                   reinterpret_cast<unsigned long long*>(out_total));
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
}

extern "C" int qsft_rs_decode(int q, int s, int t, int n, const int32_t* gf_tables, const uint8_t* syms,
                              int64_t nrows, int16_t* k_out, qsft_stream_t stream) {
  if (q < 2 || q > QSFT_MAX_Q || s < 1 || t < 1 || t > QSFT_MAX_RS_T || n < 1 || n > QSFT_MAX_N || nrows < 0)
    return QSFT_ERR_ARG;
  if (2 * t * s > 256) return QSFT_ERR_TOO_LARGE;
  int64_t order = 1;
  for (int i = 0; i < s; ++i) order *= q;
  if (order > QSFT_MAX_GF || n > order - 1) return QSFT_ERR_TOO_LARGE;
  if (nrows == 0) return QSFT_OK;
  if (!gf_tables || !syms || !k_out) return QSFT_ERR_ARG;
  const int64_t grid = (nrows + 127) / 128;
  rs_decode_kernel<<<(unsigned)grid, 128, 0, (cudaStream_t)stream>>>(q, s, t, n, gf_tables, syms, nrows, k_out);
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
}
