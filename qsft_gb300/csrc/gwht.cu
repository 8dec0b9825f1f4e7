// q-ary GWHT: fftn over the [q]^b tensor of every row, divided by q^b
// (the reference's gwht, qsft/utils.py:31-36), in place.
//
// A pass transforms the axes [a0, a1) of the row.  With outer = q^a0,
// mid = q^(a1-a0) and inner = q^(b-a1), element (o, m, t) sits at
// (o*mid + m)*inner + t.  A CTA stages a tile of NO outers x mid x TI inner
// columns in shared memory (coalesced rows of TI or NO*mid*TI contiguous
// elements), runs the radix-q DFT along each axis of the tile, and writes the
// tile back.  When the whole row fits (q^b complex values within the shared
// memory budget) one pass does everything and HBM sees one read and one write.
#include "common.cuh"

namespace qsft {

// y_k = sum_m x_m exp(-2 pi i m k / q)
template <typename V, int Q>
__device__ __forceinline__ void dft_small(V (&x)[Q], const V* __restrict__ tw) {
  if constexpr (Q == 2) {
    const V a = x[0], b = x[1];
    x[0] = cadd(a, b);
    x[1] = csub(a, b);
  } else if constexpr (Q == 4) {
    const V s02 = cadd(x[0], x[2]), d02 = csub(x[0], x[2]);
    const V s13 = cadd(x[1], x[3]), d13 = csub(x[1], x[3]);
    V mi;  // -i * d13
    mi.x = d13.y;
    mi.y = -d13.x;
    x[0] = cadd(s02, s13);
    x[2] = csub(s02, s13);
    x[1] = cadd(d02, mi);
    x[3] = csub(d02, mi);
  } else {
    V y[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      V acc = x[0];
#pragma unroll
      for (int m = 1; m < Q; ++m) acc = cadd(acc, cmul(x[m], tw[(m * k) % Q]));
      y[k] = acc;
    }
#pragma unroll
    for (int k = 0; k < Q; ++k) x[k] = y[k];
  }
}

template <typename T, int Q>
__device__ __forceinline__ void axis_pass_fixed(c2<T>* tile, int nel, int sm, const c2<T>* tw) {
  const int groups = nel / Q;
  for (int g = threadIdx.x; g < groups; g += blockDim.x) {
    const int hi = g / sm;
    const int base = hi * sm * Q + (g - hi * sm);
    c2<T> x[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) x[k] = tile[base + k * sm];
    dft_small<c2<T>, Q>(x, tw);
#pragma unroll
    for (int k = 0; k < Q; ++k) tile[base + k * sm] = x[k];
  }
}

// runtime q (any q <= QSFT_MAX_Q): O(q^2) direct DFT per group
template <typename T>
__device__ __forceinline__ void axis_pass_generic(c2<T>* tile, int nel, int sm, int q, const c2<T>* tw) {
  const int groups = nel / q;
  for (int g = threadIdx.x; g < groups; g += blockDim.x) {
    const int hi = g / sm;
    const int base = hi * sm * q + (g - hi * sm);
    c2<T> x[QSFT_MAX_Q];
    for (int k = 0; k < q; ++k) x[k] = tile[base + k * sm];
    for (int k = 0; k < q; ++k) {
      c2<T> acc = x[0];
      int idx = 0;
      for (int m = 1; m < q; ++m) {
        idx += k;
        if (idx >= q) idx -= q;
        acc = cadd(acc, cmul(x[m], tw[idx]));
      }
      tile[base + k * sm] = acc;
    }
  }
}

template <typename T, int Q>
__global__ void __launch_bounds__(512) gwht_pass_kernel(c2<T>* __restrict__ data, const int64_t* __restrict__ row_off,
                                                        int q, int naxes, int mid, int inner, int TI, int NO,
                                                        int tiles_per_row, T divisor) {
  extern __shared__ __align__(16) unsigned char smem[];
  c2<T>* tw = reinterpret_cast<c2<T>*>(smem);
  c2<T>* tile = tw + QSFT_MAX_Q;
  const int64_t blk = blockIdx.x;
  const int64_t row = blk / tiles_per_row;
  const int tr = (int)(blk - row * tiles_per_row);
  c2<T>* __restrict__ x = data + __ldg(row_off + row);
  const int ti_chunks = inner / TI;
  const int o0 = (tr / ti_chunks) * NO;
  const int t0 = (tr - (tr / ti_chunks) * ti_chunks) * TI;
  const int nel = NO * mid * TI;

  if (threadIdx.x < q) {
    const double2 w = root_of_unity(threadIdx.x, q);
    tw[threadIdx.x] = cmake<c2<T>>(w.x, -w.y);
  }
  if (TI == inner) {  // NO*mid*inner contiguous elements
    const c2<T>* src = x + (int64_t)o0 * mid * inner;
    for (int e = threadIdx.x; e < nel; e += blockDim.x) tile[e] = src[e];
  } else {
    for (int e = threadIdx.x; e < nel; e += blockDim.x) {
      const int t = e % TI;
      const int om = e / TI;  // oo*mid + m
      tile[e] = x[((int64_t)o0 * mid + om) * inner + t0 + t];
    }
  }
  __syncthreads();
  int stride_m = mid;
  for (int s = 0; s < naxes; ++s) {
    stride_m /= q;
    const int sm = stride_m * TI;
    if constexpr (Q > 0) axis_pass_fixed<T, Q>(tile, nel, sm, tw);
    else axis_pass_generic<T>(tile, nel, sm, q, tw);
    __syncthreads();
  }
  const bool scale = divisor != (T)1;
  if (TI == inner) {
    c2<T>* dst = x + (int64_t)o0 * mid * inner;
    for (int e = threadIdx.x; e < nel; e += blockDim.x) {
      c2<T> v = tile[e];
      if (scale) { v.x = v.x / divisor; v.y = v.y / divisor; }
      dst[e] = v;
    }
  } else {
    for (int e = threadIdx.x; e < nel; e += blockDim.x) {
      const int t = e % TI;
      const int om = e / TI;
      c2<T> v = tile[e];
      if (scale) { v.x = v.x / divisor; v.y = v.y / divisor; }
      x[((int64_t)o0 * mid + om) * inner + t0 + t] = v;
    }
  }
}

struct Pass {
  int a0, a1, TI, NO;
};

static int64_t ipow(int64_t q, int e) {
  int64_t r = 1;
  while (e-- > 0) r *= q;
  return r;
}

// Greedy pass plan: each pass takes as many leading axes as fit the budget.
static int plan_passes(int q, int b, size_t es, size_t budget, Pass* out, int maxp) {
  int np = 0, a0 = 0;
  while (a0 < b) {
    int best = -1, bestTI = 1, bestNO = 1;
    for (int a1 = b; a1 > a0; --a1) {
      const int64_t mid = ipow(q, a1 - a0), inner = ipow(q, b - a1), outer = ipow(q, a0);
      int64_t TI = 1;
      while (TI * q <= 64 && inner % (TI * q) == 0) TI *= q;
      if (inner < TI) TI = inner;
      if (inner <= 64) TI = inner;
      if ((size_t)(mid * TI) * es > budget) continue;
      int64_t NO = 1;
      if (TI == inner) {
        while (NO * q <= outer && outer % (NO * q) == 0 && (size_t)(NO * q * mid * TI) * es <= budget &&
               NO * mid * TI < 2048)
          NO *= q;
      }
      best = a1;
      bestTI = (int)TI;
      bestNO = (int)NO;
      break;
    }
    if (best < 0 || np >= maxp) return -1;
    out[np++] = Pass{a0, best, bestTI, bestNO};
    a0 = best;
  }
  return np;
}

template <typename T, int Q>
static int launch_pass(c2<T>* data, const int64_t* row_off, int64_t nrows, int q, int b, const Pass& p,
                       T divisor, cudaStream_t st) {
  const int mid = (int)ipow(q, p.a1 - p.a0), inner = (int)ipow(q, b - p.a1), outer = (int)ipow(q, p.a0);
  const int tiles_per_row = (outer / p.NO) * (inner / p.TI);
  const int nel = p.NO * mid * p.TI;
  const size_t sm = (size_t)(nel + QSFT_MAX_Q) * sizeof(c2<T>);
  auto kern = gwht_pass_kernel<T, Q>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
    return QSFT_ERR_CUDA;
  const int threads = nel >= 4096 ? 512 : (nel >= 1024 ? 256 : 128);
  const int64_t grid = nrows * tiles_per_row;
  if (grid > 0x7fffffffLL) return QSFT_ERR_TOO_LARGE;
  kern<<<(unsigned)grid, threads, sm, st>>>(data, row_off, q, p.a1 - p.a0, mid, inner, p.TI, p.NO,
                                            tiles_per_row, divisor);
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
}

template <typename T>
static int run_gwht(int q, int b, void* data, const int64_t* row_off, int64_t nrows, cudaStream_t st) {
  const size_t es = sizeof(c2<T>);
  const size_t budget = 200 * 1024 - QSFT_MAX_Q * es;
  Pass passes[24];
  const int np = plan_passes(q, b, es, budget, passes, 24);
  if (np <= 0) return QSFT_ERR_TOO_LARGE;
  c2<T>* d = reinterpret_cast<c2<T>*>(data);
  const T div = (T)ipow(q, b);
  for (int i = 0; i < np; ++i) {
    const T dv = (i == np - 1) ? div : (T)1;
    int rc;
    switch (q) {
      case 2: rc = launch_pass<T, 2>(d, row_off, nrows, q, b, passes[i], dv, st); break;
      case 3: rc = launch_pass<T, 3>(d, row_off, nrows, q, b, passes[i], dv, st); break;
      case 4: rc = launch_pass<T, 4>(d, row_off, nrows, q, b, passes[i], dv, st); break;
      case 5: rc = launch_pass<T, 5>(d, row_off, nrows, q, b, passes[i], dv, st); break;
      default: rc = launch_pass<T, 0>(d, row_off, nrows, q, b, passes[i], dv, st); break;
    }
    if (rc != QSFT_OK) return rc;
  }
  return QSFT_OK;
}

}  // namespace qsft

using namespace qsft;

extern "C" int qsft_gwht(int prec, int q, int b, void* data, const int64_t* row_off, int64_t nrows,
                         qsft_stream_t stream) {
  if (q < 2 || q > QSFT_MAX_Q || b < 1 || nrows < 0) return QSFT_ERR_ARG;
  if (ipow(q, b) > (1LL << 22)) return QSFT_ERR_TOO_LARGE;
  if (nrows == 0) return QSFT_OK;
  if (!data || !row_off) return QSFT_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (prec == QSFT_F32) return run_gwht<float>(q, b, data, row_off, nrows, st);
  if (prec == QSFT_F64) return run_gwht<double>(q, b, data, row_off, nrows, st);
  return QSFT_ERR_ARG;
}
