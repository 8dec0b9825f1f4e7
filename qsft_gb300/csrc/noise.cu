// Bin-domain complex AWGN (the noise of SyntheticSubsampledSignal.get_MDU,
// synt_exp/synt_src/synthetic_signal.py:126-129), drawn on the device; the
// stream is defined in noise.cuh.
#include "noise.cuh"

namespace qsft {

// thread per (row, e < half) pair of every job; rows [r0, r0 + nrows) of the
// batch's row list when `rows` is given (row_off + row_meta), else all rows of
// every job
template <typename T>
__global__ void noise_kernel(qsft_plan plan) {
  const int j = blockIdx.y;
  const qsft_job* job = plan.jobs + j;
  const double nu = job->noise_nu;
  if (!(nu > 0.0)) return;
  const int64_t B = job->B, half = (B + 1) / 2;
  const int64_t rows = (int64_t)job->C * job->R * job->P;
  c2<T>* U = reinterpret_cast<c2<T>*>(plan.U) + job->off_U;
  const uint2 key = noise_key(job->noise_seed);
  const T tnu = (T)nu;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < rows * half;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = p / half, e = p - row * half;
    c2<T> g0, g1;
    noise_pair<T>(key, row, half, e, g0, g1);
    c2<T>* x = U + row * B;
    c2<T> v = x[e];
    v.x += tnu * g0.x;
    v.y += tnu * g0.y;
    x[e] = v;
    if (e + half < B) {
      c2<T> w = x[e + half];
      w.x += tnu * g1.x;
      w.y += tnu * g1.y;
      x[e + half] = w;
    }
  }
}

template <typename T>
__global__ void add_kernel(c2<T>* __restrict__ U, const c2<T>* __restrict__ X, int64_t count) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    c2<T> a = U[i];
    const c2<T> b = X[i];
    a.x += b.x;
    a.y += b.y;
    U[i] = a;
  }
}

}  // namespace qsft

using namespace qsft;

extern "C" int qsft_add_noise_philox(const qsft_plan* plan, qsft_stream_t stream) {
  if (!plan || plan->njobs <= 0 || !plan->jobs || !plan->U) return QSFT_ERR_ARG;
  if (plan->njobs > 65535) return QSFT_ERR_TOO_LARGE;
  dim3 grid(152 * 4, plan->njobs);
  cudaStream_t st = (cudaStream_t)stream;
  if (plan->prec == QSFT_F32) noise_kernel<float><<<grid, 256, 0, st>>>(*plan);
  else if (plan->prec == QSFT_F64) noise_kernel<double><<<grid, 256, 0, st>>>(*plan);
  else return QSFT_ERR_ARG;
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
}

extern "C" int qsft_add_bins(int prec, void* U, const void* X, int64_t count, qsft_stream_t stream) {
  if (count < 0 || (count > 0 && (!U || !X))) return QSFT_ERR_ARG;
  if (count == 0) return QSFT_OK;
  const int64_t want = (count + 255) / 256;
  const unsigned grid = (unsigned)(want < 152 * 16 ? want : 152 * 16);
  cudaStream_t st = (cudaStream_t)stream;
  if (prec == QSFT_F32)
    add_kernel<float><<<grid, 256, 0, st>>>((float2*)U, (const float2*)X, count);
  else if (prec == QSFT_F64)
    add_kernel<double><<<grid, 256, 0, st>>>((double2*)U, (const double2*)X, count);
  else
    return QSFT_ERR_ARG;
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
}
