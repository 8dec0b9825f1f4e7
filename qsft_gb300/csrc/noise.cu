// Bin-domain complex AWGN (the noise of SyntheticSubsampledSignal.get_MDU,
// synt_exp/synt_src/synthetic_signal.py:126-129), drawn on the device.
//
// Random bits: Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC 2011), counter = element index, key = the
// job's noise_seed: a job draws the same noise whatever batch it is part of.  Normals: Box-Muller on the two pairs of words.
#include "common.cuh"

namespace qsft {

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += W0;
    k.y += W1;
  }
  return c;
}

// two independent N(0,1) from two uniform words (Box-Muller), in T precision
__device__ __forceinline__ double2 box_muller(uint32_t a, uint32_t b, double) {
  const double u1 = ((double)a + 1.0) * 2.3283064365386963e-10;  // (0, 1]
  const double u2 = (double)b * 2.3283064365386963e-10;          // [0, 1)
  const double r = sqrt(-2.0 * log(u1));
  double s, c;
  sincospi(2.0 * u2, &s, &c);
  return make_double2(r * c, r * s);
}
__device__ __forceinline__ float2 box_muller(uint32_t a, uint32_t b, float) {
  const float u1 = ((float)(a >> 8) + 1.0f) * 5.9604645e-08f;  // (0, 1], 24-bit grid
  const float u2 = (float)(b >> 8) * 5.9604645e-08f;           // [0, 1)
  const float r = sqrtf(-2.0f * logf(u1));
  float s, c;
  sincospif(2.0f * u2, &s, &c);
  return make_float2(r * c, r * s);
}

template <typename T>
__global__ void noise_kernel(qsft_plan plan) {
  const int j = blockIdx.y;
  const qsft_job* job = plan.jobs + j;
  const double nu = job->noise_nu;
  if (!(nu > 0.0)) return;
  const int64_t count = (int64_t)job->C * job->R * job->P * job->B;
  c2<T>* U = reinterpret_cast<c2<T>*>(plan.U) + job->off_U;
  const uint2 key = make_uint2((uint32_t)job->noise_seed, (uint32_t)(job->noise_seed >> 32));
  // each thread draws 4 words -> 2 complex entries
  for (int64_t pair = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; 2 * pair < count;
       pair += (int64_t)gridDim.x * blockDim.x) {
    const uint4 r = philox4x32_10(make_uint4((uint32_t)pair, (uint32_t)(pair >> 32), 0x9e37u, 0x51f7u), key);
    const c2<T> g0 = box_muller(r.x, r.y, T(0));
    const c2<T> g1 = box_muller(r.z, r.w, T(0));
    const T tnu = (T)nu;
    const int64_t e = 2 * pair;
    c2<T> v = U[e];
    v.x += tnu * g0.x;
    v.y += tnu * g0.y;
    U[e] = v;
    if (e + 1 < count) {
      c2<T> w = U[e + 1];
      w.x += tnu * g1.x;
      w.y += tnu * g1.y;
      U[e + 1] = w;
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
