// Coset query generation + synthetic-signal evaluation (CUDA cores).
//
// f(x) = sum_s a_s * omega^(<x, k_s> mod q) for every query point x of every
// coset M_c l + d (mod q).  The integer dot products run on packed 8-bit
// digits with __dp4a (4 MACs per instruction); the root lookup and complex
// accumulation read a per-CTA table a_s * omega^r staged in shared memory.
#include "common.cuh"

namespace qsft {

constexpr int EVAL_THREADS = 256;
constexpr int EVAL_SPT = 4;                              // samples per thread
constexpr int EVAL_TILE = EVAL_THREADS * EVAL_SPT;       // samples per CTA
static_assert(EVAL_TILE == QSFT_EVAL_TILE, "eval tile size is part of the ABI");
constexpr int EVAL_ST = 128;                             // support entries per smem stage

template <typename T, int NW>
struct EvalSmem {
  static constexpr size_t kw_bytes = (size_t)EVAL_ST * NW * 4;
  static size_t bytes(int max_q) {
    return 32 * sizeof(double2) + kw_bytes + (size_t)EVAL_ST * max_q * sizeof(c2<T>);
  }
};

// Stage support entries [s0, s0+EVAL_ST) as packed digit words and the table
// a_s * omega^r (computed in double, rounded to T).  Entries past S are zero.
template <typename T, int NW>
__device__ __forceinline__ void stage_support(const int8_t* __restrict__ K, const c2<T>* __restrict__ A,
                                              int S, int n, int q, int s0, uint32_t* sK, c2<T>* sT,
                                              const double2* sW) {
  const int cnt = min(EVAL_ST, S - s0);
  for (int idx = threadIdx.x; idx < EVAL_ST * NW; idx += blockDim.x) {
    const int s = idx / NW, w = idx - (idx / NW) * NW;
    uint32_t word = 0;
    if (s < cnt) {
      const int8_t* kr = K + (int64_t)(s0 + s) * n;
#pragma unroll
      for (int bb = 0; bb < 4; ++bb) {
        const int i = 4 * w + bb;
        if (i < n) word |= (uint32_t)(uint8_t)__ldg(kr + i) << (8 * bb);
      }
    }
    sK[idx] = word;
  }
  for (int idx = threadIdx.x; idx < EVAL_ST * q; idx += blockDim.x) {
    const int s = idx / q, r = idx - (idx / q) * q;
    c2<T> v = cmake<c2<T>>(0.0, 0.0);
    if (s < cnt) {  // product in T: GB300's FP64 rate is a small fraction of FP32
      const c2<T> a = A[s0 + s];
      const c2<T> w = cmake<c2<T>>(sW[r].x, sW[r].y);
      v = cmul(a, w);
    }
    sT[idx] = v;
  }
}

// f[p] += sum_{s < cnt} table[s][<x_p, k_s> mod q]
template <typename T, int NW, bool POW2>
__device__ __forceinline__ void accumulate(const uint32_t (&x)[EVAL_SPT][NW], const uint32_t* __restrict__ sK,
                                           const c2<T>* __restrict__ sT, int cnt, int q, ModQ mq,
                                           T (&fr)[EVAL_SPT], T (&fi)[EVAL_SPT]) {
#pragma unroll 2
  for (int s = 0; s < cnt; ++s) {
    uint32_t kw[NW];
    const uint2* kp = reinterpret_cast<const uint2*>(sK + s * NW);
#pragma unroll
    for (int w = 0; w < NW / 2; ++w) {
      const uint2 v = kp[w];
      kw[2 * w] = v.x;
      kw[2 * w + 1] = v.y;
    }
    const c2<T>* row = sT + s * q;
#pragma unroll
    for (int p = 0; p < EVAL_SPT; ++p) {
      uint32_t acc = 0;
#pragma unroll
      for (int w = 0; w < NW; ++w) acc = __dp4a(x[p][w], kw[w], acc);
      const uint32_t r = POW2 ? (acc & mq.mask) : (acc - mq.q * __umulhi(acc, mq.mul));
      const c2<T> t = row[r];
      fr[p] += t.x;
      fi[p] += t.y;
    }
  }
}

template <typename T, int NW, bool POW2>
__global__ void __launch_bounds__(EVAL_THREADS) eval_cosets_kernel(qsft_plan plan) {
  extern __shared__ __align__(16) unsigned char smem[];
  double2* sW = reinterpret_cast<double2*>(smem);
  uint32_t* sK = reinterpret_cast<uint32_t*>(smem + 32 * sizeof(double2));
  c2<T>* sT = reinterpret_cast<c2<T>*>(smem + 32 * sizeof(double2) + EvalSmem<T, NW>::kw_bytes);

  const int64_t tile = blockIdx.x;
  const int j = find_job(plan.eval_prefix, plan.njobs, tile);
  const qsft_job* __restrict__ job = plan.jobs + j;
  const int q = job->q, n = job->n, b = job->b, B = job->B, S = job->S;
  const int RP = job->R * job->P;
  const int64_t total = (int64_t)job->C * RP * B;
  const int64_t base = (tile - plan.eval_prefix[j]) * EVAL_TILE;
  const int8_t* __restrict__ M = plan.i8 + job->off_M;
  const int8_t* __restrict__ D = plan.i8 + job->off_D;
  const int8_t* __restrict__ K = plan.i8 + job->off_K;
  const c2<T>* __restrict__ A = reinterpret_cast<const c2<T>*>(plan.A) + job->off_A;
  c2<T>* __restrict__ U = reinterpret_cast<c2<T>*>(plan.U) + job->off_U;
  const ModQ mq = make_modq(q);

  if (threadIdx.x < q) sW[threadIdx.x] = root_of_unity(threadIdx.x, q);

  // query digits x = (M_c l + d) mod q, packed 4 per word
  uint32_t x[EVAL_SPT][NW];
  int64_t gidx[EVAL_SPT];
#pragma unroll
  for (int p = 0; p < EVAL_SPT; ++p) {
    gidx[p] = base + p * EVAL_THREADS + threadIdx.x;
#pragma unroll
    for (int w = 0; w < NW; ++w) x[p][w] = 0;
    if (gidx[p] >= total) continue;
    const int64_t row = gidx[p] / B;
    int l = (int)(gidx[p] - row * B);
    const int c = (int)(row / RP);
    const int rp = (int)(row - (int64_t)c * RP);
    int ld[24];  // digits of l, MSB first (b <= 20 for q^b <= 2^20)
    for (int t = b - 1; t >= 0; --t) {
      ld[t] = l % q;
      l /= q;
    }
    const int8_t* Mc = M + (int64_t)c * n * b;
    const int8_t* d = D + ((int64_t)c * RP + rp) * n;
    uint32_t xw[NW];  // runtime-indexed staging (one-time per sample)
#pragma unroll 1
    for (int w = 0; w < NW; ++w) {
      uint32_t word = 0;
      for (int bb = 0; bb < 4; ++bb) {
        const int i = 4 * w + bb;
        if (i < n) {
          int acc = __ldg(d + i);
          for (int t = 0; t < b; ++t) acc += (int)__ldg(Mc + i * b + t) * ld[t];
          word |= (uint32_t)(acc % q) << (8 * bb);
        }
      }
      xw[w] = word;
    }
#pragma unroll
    for (int w = 0; w < NW; ++w) x[p][w] = xw[w];
  }

  T fr[EVAL_SPT], fi[EVAL_SPT];
#pragma unroll
  for (int p = 0; p < EVAL_SPT; ++p) fr[p] = fi[p] = (T)0;

  for (int s0 = 0; s0 < S; s0 += EVAL_ST) {
    __syncthreads();
    stage_support<T, NW>(K, A, S, n, q, s0, sK, sT, sW);
    __syncthreads();
    accumulate<T, NW, POW2>(x, sK, sT, min(EVAL_ST, S - s0), q, mq, fr, fi);
  }
#pragma unroll
  for (int p = 0; p < EVAL_SPT; ++p)
    if (gidx[p] < total) U[gidx[p]] = cmake<c2<T>>(fr[p], fi[p]);
}

template <typename T, int NW, bool POW2>
__global__ void __launch_bounds__(EVAL_THREADS) eval_points_kernel(int q, int n, int S, const int8_t* __restrict__ X,
                                                                   int64_t npoints, const int8_t* __restrict__ K,
                                                                   const c2<T>* __restrict__ A, c2<T>* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  double2* sW = reinterpret_cast<double2*>(smem);
  uint32_t* sK = reinterpret_cast<uint32_t*>(smem + 32 * sizeof(double2));
  c2<T>* sT = reinterpret_cast<c2<T>*>(smem + 32 * sizeof(double2) + EvalSmem<T, NW>::kw_bytes);
  const ModQ mq = make_modq(q);
  if (threadIdx.x < q) sW[threadIdx.x] = root_of_unity(threadIdx.x, q);
  const int64_t base = (int64_t)blockIdx.x * EVAL_TILE;
  uint32_t x[EVAL_SPT][NW];
  int64_t gidx[EVAL_SPT];
#pragma unroll
  for (int p = 0; p < EVAL_SPT; ++p) {
    gidx[p] = base + p * EVAL_THREADS + threadIdx.x;
    uint32_t xw[NW];
#pragma unroll 1
    for (int w = 0; w < NW; ++w) {
      uint32_t word = 0;
      if (gidx[p] < npoints) {
        for (int bb = 0; bb < 4; ++bb) {
          const int i = 4 * w + bb;
          if (i < n) word |= (uint32_t)(uint8_t)__ldg(X + gidx[p] * n + i) << (8 * bb);
        }
      }
      xw[w] = word;
    }
#pragma unroll
    for (int w = 0; w < NW; ++w) x[p][w] = xw[w];
  }
  T fr[EVAL_SPT], fi[EVAL_SPT];
#pragma unroll
  for (int p = 0; p < EVAL_SPT; ++p) fr[p] = fi[p] = (T)0;
  for (int s0 = 0; s0 < S; s0 += EVAL_ST) {
    __syncthreads();
    stage_support<T, NW>(K, A, S, n, q, s0, sK, sT, sW);
    __syncthreads();
    accumulate<T, NW, POW2>(x, sK, sT, min(EVAL_ST, S - s0), q, mq, fr, fi);
  }
#pragma unroll
  for (int p = 0; p < EVAL_SPT; ++p)
    if (gidx[p] < npoints) out[gidx[p]] = cmake<c2<T>>(fr[p], fi[p]);
}

// ---------------------------------------------------------------- dispatch
template <typename T, int NW, bool POW2>
static int launch_cosets(const qsft_plan* plan, cudaStream_t st) {
  const size_t sm = EvalSmem<T, NW>::bytes(plan->max_q);
  auto kern = eval_cosets_kernel<T, NW, POW2>;
  if (!ensure_smem((const void*)kern, (int)sm)) return QSFT_ERR_CUDA;
  if (plan->total_eval_tiles <= 0) return QSFT_OK;
  kern<<<(unsigned)plan->total_eval_tiles, EVAL_THREADS, sm, st>>>(*plan);
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
}

template <typename T, bool POW2>
static int cosets_nw(const qsft_plan* plan, cudaStream_t st) {
  const int n = plan->max_n;
  if (n <= 8) return launch_cosets<T, 2, POW2>(plan, st);
  if (n <= 16) return launch_cosets<T, 4, POW2>(plan, st);
  if (n <= 24) return launch_cosets<T, 6, POW2>(plan, st);
  if (n <= 32) return launch_cosets<T, 8, POW2>(plan, st);
  if (n <= 64) return launch_cosets<T, 16, POW2>(plan, st);
  return launch_cosets<T, 32, POW2>(plan, st);
}

template <typename T, int NW, bool POW2>
static int launch_points(int q, int n, int S, const int8_t* X, int64_t np, const int8_t* K, const void* A,
                         void* out, cudaStream_t st) {
  const size_t sm = EvalSmem<T, NW>::bytes(q);
  auto kern = eval_points_kernel<T, NW, POW2>;
  if (!ensure_smem((const void*)kern, (int)sm)) return QSFT_ERR_CUDA;
  const int64_t grid = (np + EVAL_TILE - 1) / EVAL_TILE;
  kern<<<(unsigned)grid, EVAL_THREADS, sm, st>>>(q, n, S, X, np, K, reinterpret_cast<const c2<T>*>(A),
                                                 reinterpret_cast<c2<T>*>(out));
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
}

template <typename T, bool POW2>
static int points_nw(int q, int n, int S, const int8_t* X, int64_t np, const int8_t* K, const void* A, void* out,
                     cudaStream_t st) {
  if (n <= 8) return launch_points<T, 2, POW2>(q, n, S, X, np, K, A, out, st);
  if (n <= 16) return launch_points<T, 4, POW2>(q, n, S, X, np, K, A, out, st);
  if (n <= 24) return launch_points<T, 6, POW2>(q, n, S, X, np, K, A, out, st);
  if (n <= 32) return launch_points<T, 8, POW2>(q, n, S, X, np, K, A, out, st);
  if (n <= 64) return launch_points<T, 16, POW2>(q, n, S, X, np, K, A, out, st);
  return launch_points<T, 32, POW2>(q, n, S, X, np, K, A, out, st);
}

}  // namespace qsft

using namespace qsft;

extern "C" int qsft_eval_cosets(const qsft_plan* plan, qsft_stream_t stream) {
  if (!plan || plan->njobs <= 0 || !plan->jobs || !plan->eval_prefix || !plan->i8 || !plan->A || !plan->U)
    return QSFT_ERR_ARG;
  if (plan->max_q < 2 || plan->max_q > QSFT_MAX_Q || plan->max_n < 1 || plan->max_n > QSFT_MAX_N)
    return QSFT_ERR_TOO_LARGE;
  if (plan->total_eval_tiles > 0x7fffffffLL) return QSFT_ERR_TOO_LARGE;
  cudaStream_t st = (cudaStream_t)stream;
  const bool p2 = plan->all_q_pow2 != 0;
  if (plan->prec == QSFT_F32) return p2 ? cosets_nw<float, true>(plan, st) : cosets_nw<float, false>(plan, st);
  if (plan->prec == QSFT_F64) return p2 ? cosets_nw<double, true>(plan, st) : cosets_nw<double, false>(plan, st);
  return QSFT_ERR_ARG;
}

extern "C" int qsft_eval_points(int prec, int q, int n, int S, const int8_t* X, int64_t npoints, const int8_t* K,
                                const void* A, void* out, qsft_stream_t stream) {
  if (q < 2 || q > QSFT_MAX_Q || n < 1 || n > QSFT_MAX_N || S < 0 || npoints < 0) return QSFT_ERR_ARG;
  if (npoints == 0) return QSFT_OK;
  if (!X || !out || (S > 0 && (!K || !A))) return QSFT_ERR_ARG;
  if ((npoints + EVAL_TILE - 1) / EVAL_TILE > 0x7fffffffLL) return QSFT_ERR_TOO_LARGE;
  cudaStream_t st = (cudaStream_t)stream;
  const bool p2 = (q & (q - 1)) == 0;
  if (prec == QSFT_F32)
    return p2 ? points_nw<float, true>(q, n, S, X, npoints, K, A, out, st)
              : points_nw<float, false>(q, n, S, X, npoints, K, A, out, st);
  if (prec == QSFT_F64)
    return p2 ? points_nw<double, true>(q, n, S, X, npoints, K, A, out, st)
              : points_nw<double, false>(q, n, S, X, npoints, K, A, out, st);
  return QSFT_ERR_ARG;
}
