// Shared device helpers for the q-SFT kernels (sm_103a).
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/qsft_gb300.h"

namespace qsft {

template <typename T> struct cplx;
template <> struct cplx<float> { using type = float2; };
template <> struct cplx<double> { using type = double2; };
template <typename T> using c2 = typename cplx<T>::type;

template <typename V> __device__ __forceinline__ V cmake(double re, double im);
template <> __device__ __forceinline__ float2 cmake<float2>(double re, double im) {
  return make_float2((float)re, (float)im);
}
template <> __device__ __forceinline__ double2 cmake<double2>(double re, double im) {
  return make_double2(re, im);
}
template <typename V> __device__ __forceinline__ V cadd(V a, V b) { V r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename V> __device__ __forceinline__ V csub(V a, V b) { V r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename V> __device__ __forceinline__ V cmul(V a, V b) {
  V r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
// a * conj(b)
template <typename V> __device__ __forceinline__ V cmulc(V a, V b) {
  V r; r.x = a.x * b.x + a.y * b.y; r.y = a.y * b.x - a.x * b.y; return r;
}
__device__ __forceinline__ double2 to_d2(float2 v) { return make_double2(v.x, v.y); }
__device__ __forceinline__ double2 to_d2(double2 v) { return v; }

// exp(2 pi i m / q) in double, via the CUDA math library's sincospi.
__device__ __forceinline__ double2 root_of_unity(int m, int q) {
  double s, c;
  sincospi(2.0 * (double)m / (double)q, &s, &c);
  return make_double2(c, s);
}

// Index of the job owning work item `idx`: largest j with prefix[j] <= idx.
__device__ __forceinline__ int find_job(const int64_t* __restrict__ prefix, int njobs, int64_t idx) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(prefix + mid) <= idx) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// a mod q for 0 <= a < 2^17, q in [2, 32]: quotient by the round-up
// multiplier ceil(2^32 / q) (exact in that range; checked exhaustively on the host).
struct ModQ {
  uint32_t q, mul, mask;
  bool pow2;
};
__host__ __device__ inline ModQ make_modq(uint32_t q) {
  ModQ m;
  m.q = q;
  m.mul = (uint32_t)((0x100000000ull + q - 1) / q);
  m.pow2 = (q & (q - 1)) == 0;
  m.mask = q - 1;
  return m;
}
__device__ __forceinline__ uint32_t modq(uint32_t a, const ModQ& m) {
  if (m.pow2) return a & m.mask;
  return a - m.q * __umulhi(a, m.mul);
}

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

}  // namespace qsft

namespace qsft {
// kernels launched by this library since load (qsft_launch_count)
void count_launch();
// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) only when a kernel needs more
// than it was last given on this device: keeps launches free of non-stream API
// calls after the first, so they can be captured into CUDA graphs
bool ensure_smem(const void* func, int bytes);
}  // namespace qsft

#define QSFT_CUDA_CHECK_LAUNCH()                         \
  do {                                                   \
    cudaError_t e__ = cudaGetLastError();                \
    if (e__ != cudaSuccess) return QSFT_ERR_CUDA;        \
    qsft::count_launch();                                \
  } while (0)
