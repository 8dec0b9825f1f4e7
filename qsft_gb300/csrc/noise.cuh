// Device bin noise shared by the noise kernels and the fused GWHT + noise pass.
//
// Random bits: Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC 2011) keyed by the job's noise_seed.  One
// draw gives two complex normals (Box-Muller on each pair of words): for row
// r (0 .. C*R*P - 1) of the job and e < half = ceil(q^b / 2), counter
// r*half + e covers entries e and e + half of the row.  The noise of a job is
// thus a function of its own seed and indices only, whatever batch it is in,
// and a transform pass that holds entries e and e + half in one thread can add
// it without another pass over the bins.
#pragma once
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
  sincospi(2.0 * u2 - 1.0, &s, &c);  // the FP32 draw's angle 2 pi u2 - pi: one noise realisation
  return make_double2(r * c, r * s);
}
// FP32: the hardware approximations of log and sin/cos (__logf, __sincosf; the
// angle in [-pi, pi), where sin.approx/cos.approx are accurate to ~2^-20.5):
// noise needs the distribution, not correctly rounded samples, and the fused
// GWHT pass is bound by these instructions
__device__ __forceinline__ float2 box_muller(uint32_t a, uint32_t b, float) {
  // the FP64 draw's uniforms rounded to FP32 (small u1 exact: the tail matches too)
  const float u1 = ((float)a + 1.0f) * 2.3283064e-10f;  // (0, 1]
  const float u2 = (float)b * 2.3283064e-10f;           // [0, 1]
  const float r = sqrtf(fmaxf(-2.0f * __logf(u1), 0.0f));  // __logf's absolute error near 1: no NaN
  float s, c;
  __sincosf(6.2831853f * u2 - 3.1415927f, &s, &c);
  return make_float2(r * c, r * s);
}

__device__ __forceinline__ uint2 noise_key(uint64_t seed) { return make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)); }

// the pair (entry e, entry e + half) of row `row`: standard normals, complex
template <typename T>
__device__ __forceinline__ void noise_pair(uint2 key, int64_t row, int64_t half, int64_t e, c2<T>& g0, c2<T>& g1) {
  const uint64_t ctr = (uint64_t)row * (uint64_t)half + (uint64_t)e;
  const uint4 r = philox4x32_10(make_uint4((uint32_t)ctr, (uint32_t)(ctr >> 32), 0x9e37u, 0x51f7u), key);
  g0 = box_muller(r.x, r.y, T(0));
  g1 = box_muller(r.z, r.w, T(0));
}

// entry e of row `row` alone, for passes whose threads do not hold the pair
// (e, e + half): the same value noise_pair gives it
template <typename T>
__device__ __forceinline__ c2<T> noise_one(uint2 key, int64_t row, int64_t half, int64_t e) {
  const bool upper = e >= half;
  const uint64_t ctr = (uint64_t)row * (uint64_t)half + (uint64_t)(upper ? e - half : e);
  const uint4 r = philox4x32_10(make_uint4((uint32_t)ctr, (uint32_t)(ctr >> 32), 0x9e37u, 0x51f7u), key);
  return upper ? box_muller(r.z, r.w, T(0)) : box_muller(r.x, r.y, T(0));
}

}  // namespace qsft
