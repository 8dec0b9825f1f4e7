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
// Rows above 48 KB whose q^k-way split fits 64 KB per part (k with q^k <= 8)
// use a thread-block cluster per row instead (one HBM read and write, parts
// exchanged through distributed shared memory).
#include <cooperative_groups.h>

#include <atomic>

#include "common.cuh"
#include "noise.cuh"

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
  } else if constexpr (Q == 20) {
    // 20 = 4 x 5: n = 5 n1 + n2, k = k1 + 4 k2;
    // X[k1 + 4 k2] = sum_n2 W20^(n2 k1) W5^(n2 k2) sum_n1 x[5 n1 + n2] W4^(n1 k1)
    V t5[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) t5[j] = tw[4 * j];  // W5^j = W20^(4j)
    V y[4][5];
#pragma unroll
    for (int n2 = 0; n2 < 5; ++n2) {
      V a[4] = {x[n2], x[5 + n2], x[10 + n2], x[15 + n2]};
      dft_small<V, 4>(a, tw);
#pragma unroll
      for (int k1 = 0; k1 < 4; ++k1) y[k1][n2] = (n2 * k1 == 0) ? a[k1] : cmul(a[k1], tw[n2 * k1]);
    }
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
      dft_small<V, 5>(y[k1], t5);
#pragma unroll
      for (int k2 = 0; k2 < 5; ++k2) x[k1 + 4 * k2] = y[k1][k2];
    }
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

// g / d for 0 <= g < 2^24 through a float reciprocal, corrected to exact
__device__ __forceinline__ int div_small(int g, int d, float rd) {
  int h = (int)((float)g * rd);
  if (h * d > g) --h;
  else if ((h + 1) * d <= g) ++h;
  return h;
}

template <typename T, int Q>
__device__ __forceinline__ void axis_pass_fixed(c2<T>* tile, int nel, int sm, const c2<T>* tw) {
  const int groups = nel / Q;
  const float rsm = 1.0f / (float)sm;
  for (int g = threadIdx.x; g < groups; g += blockDim.x) {
    const int hi = div_small(g, sm, rsm);
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
  const float rsm = 1.0f / (float)sm;
  for (int g = threadIdx.x; g < groups; g += blockDim.x) {
    const int hi = div_small(g, sm, rsm);
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

// device bin noise of one row (noise.cuh); nu = 0: none
struct RowNoise {
  uint2 key;
  int64_t row;  // row index within its job
  double nu;
};

template <typename T, int Q>
__global__ void __launch_bounds__(512) gwht_pass_kernel(c2<T>* __restrict__ data, const int64_t* __restrict__ row_off,
                                                        int q, int naxes, int mid, int inner, int TI, int NO,
                                                        int tiles_per_row, T inv, int64_t B,
                                                        const qsft_job* __restrict__ jobs,
                                                        const int32_t* __restrict__ row_meta) {
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
  // element e of the tile is (om, t) = (e / TI, e % TI): stepped per thread without division
  const int t_first = threadIdx.x % TI, om_first = threadIdx.x / TI;
  const int dt = blockDim.x % TI, dom = blockDim.x / TI;

  if (threadIdx.x < q) {
    const double2 w = root_of_unity(threadIdx.x, q);
    tw[threadIdx.x] = cmake<c2<T>>(w.x, -w.y);
  }
  if (TI == inner) {  // NO*mid*inner contiguous elements
    const c2<T>* src = x + (int64_t)o0 * mid * inner;
    for (int e = threadIdx.x; e < nel; e += blockDim.x) tile[e] = src[e];
  } else {
    int t = t_first, om = om_first;  // om = oo*mid + m
    for (int e = threadIdx.x; e < nel; e += blockDim.x) {
      tile[e] = x[((int64_t)o0 * mid + om) * inner + t0 + t];
      t += dt;
      om += dom;
      if (t >= TI) {
        t -= TI;
        ++om;
      }
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
  // last pass: scale by 1/q^b and, with jobs, add the row's device bin noise
  const bool scale = inv != (T)1;
  RowNoise nz = {make_uint2(0, 0), 0, 0.0};
  if (jobs) {
    const qsft_job* jb = jobs + __ldg(row_meta + 2 * row);
    nz.key = noise_key(jb->noise_seed);
    nz.row = __ldg(row_meta + 2 * row + 1);
    nz.nu = jb->noise_nu;
  }
  const T tnu = (T)nz.nu;
  const int64_t half = (B + 1) / 2;
  auto finish = [&](c2<T> v, int64_t idx) {
    if (scale) {
      v.x *= inv;
      v.y *= inv;
    }
    if (nz.nu > 0.0) {
      const c2<T> g = noise_one<T>(nz.key, nz.row, half, idx);
      v.x += tnu * g.x;
      v.y += tnu * g.y;
    }
    return v;
  };
  if (TI == inner) {
    const int64_t e0 = (int64_t)o0 * mid * inner;
    c2<T>* dst = x + e0;
    for (int e = threadIdx.x; e < nel; e += blockDim.x) dst[e] = finish(tile[e], e0 + e);
  } else {
    int t = t_first, om = om_first;
    for (int e = threadIdx.x; e < nel; e += blockDim.x) {
      const int64_t idx = ((int64_t)o0 * mid + om) * inner + t0 + t;
      x[idx] = finish(tile[e], idx);
      t += dt;
      om += dom;
      if (t >= TI) {
        t -= TI;
        ++om;
      }
    }
  }
}

// ---------------------------------------------------------------- row path
// q in {2, 4}, whole row in shared memory (FP32 rows up to 16384 values, FP64
// up to 8192).  A persistent CTA of B/16 threads transforms whole rows: every
// pass gives each thread 16 elements -- 16/G groups of G = q^m elements along
// m consecutive digits -- and applies the q-point DFT along each digit in
// registers.  The first pass reads global memory and the last one writes it;
// passes in between go through shared memory, padded by one value every 16 so
// that every access pattern needs only the minimum of bank wavefronts.  While a row
// is transformed, the CTA's next row is prefetched into L2 (two rows ahead
// measured slower: the prefetched lines of 2 x 152 rows start to leave L2
// before they are read).
__device__ __forceinline__ int pad16(int e) { return e + (e >> 4); }

template <typename V, int Q, int G>
__device__ __forceinline__ void groups_dft(V (&x)[16]) {
#pragma unroll
  for (int st = G / Q; st >= 1; st /= Q) {  // stride of each digit of the group
#pragma unroll
    for (int k = 0; k < 16 / G; ++k) {
#pragma unroll
      for (int m = 0; m < G; ++m) {
        if ((m / st) % Q) continue;  // m = first element of a DFT along this digit
        V v[Q];
#pragma unroll
        for (int r = 0; r < Q; ++r) v[r] = x[k * G + m + r * st];
        dft_small<V, Q>(v, nullptr);
#pragma unroll
        for (int r = 0; r < Q; ++r) x[k * G + m + r * st] = v[r];
      }
    }
  }
}

// one pass over digits [d0, d0 + m) with G = q^m; slo = stride of the lowest of them
template <typename T, int Q, int G>
__device__ __forceinline__ void row_pass(c2<T> (&x)[16], int t, int B, int slo, int mode, const c2<T>* src,
                                         c2<T>* tile, c2<T>* dst, T scale, const RowNoise& nz) {
  const int nthr = B >> 4;
  int base[16 / G];
#pragma unroll
  for (int k = 0; k < 16 / G; ++k) {
    const int gi = t + k * nthr;
    base[k] = (gi % slo) + (gi / slo) * (slo * G);
  }
  // load: mode 0 from global (first pass), else from the padded tile
#pragma unroll
  for (int k = 0; k < 16 / G; ++k)
#pragma unroll
    for (int m = 0; m < G; ++m) {
      const int e = base[k] + m * slo;
      x[k * G + m] = mode == 0 ? src[e] : tile[pad16(e)];
    }
  groups_dft<c2<T>, Q, G>(x);
  // store: mode 2 to global (last pass: scaled, plus the row's noise), else to
  // the tile.  The last pass is over the top digits (its groups start below
  // B/G), so entries m and m + G/2 of a group are e and e + B/2: one noise
  // draw serves both.
  if (mode == 2) {
    const T tnu = (T)nz.nu;
#pragma unroll
    for (int k = 0; k < 16 / G; ++k)
#pragma unroll
      for (int m = 0; m < G / 2; ++m) {
        const int e0 = base[k] + m * slo, e1 = e0 + (G / 2) * slo;
        c2<T> v0 = x[k * G + m], v1 = x[k * G + m + G / 2];
        v0.x *= scale;
        v0.y *= scale;
        v1.x *= scale;
        v1.y *= scale;
        if (nz.nu > 0.0) {
          c2<T> g0, g1;
          noise_pair<T>(nz.key, nz.row, B / 2, e0, g0, g1);
          v0.x += tnu * g0.x;
          v0.y += tnu * g0.y;
          v1.x += tnu * g1.x;
          v1.y += tnu * g1.y;
        }
        dst[e0] = v0;
        dst[e1] = v1;
      }
  } else {
#pragma unroll
    for (int k = 0; k < 16 / G; ++k)
#pragma unroll
      for (int m = 0; m < G; ++m) tile[pad16(base[k] + m * slo)] = x[k * G + m];
  }
}

template <typename T, int Q>
__device__ __forceinline__ void row_pass_any(int nd, c2<T> (&v)[16], int t, int B, int slo, int mode, c2<T>* x,
                                             c2<T>* tile, T scale, const RowNoise& nz) {
  if constexpr (Q == 4) {
    if (nd == 2) row_pass<T, 4, 16>(v, t, B, slo, mode, x, tile, x, scale, nz);
    else row_pass<T, 4, 4>(v, t, B, slo, mode, x, tile, x, scale, nz);
  } else {
    if (nd == 4) row_pass<T, 2, 16>(v, t, B, slo, mode, x, tile, x, scale, nz);
    else if (nd == 3) row_pass<T, 2, 8>(v, t, B, slo, mode, x, tile, x, scale, nz);
    else if (nd == 2) row_pass<T, 2, 4>(v, t, B, slo, mode, x, tile, x, scale, nz);
    else row_pass<T, 2, 2>(v, t, B, slo, mode, x, tile, x, scale, nz);
  }
}

// rows of B = q^b >= 256 values: at least two passes (first from, last to global);
// the top and the lowest DPP digits are disjoint full groups
// jobs / row_meta (job, row within the job, per row) non-null: add each row's
// device bin noise in the last pass
template <typename T, int Q>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 1024 : 512)
    gwht_row_kernel(c2<T>* __restrict__ data, const int64_t* __restrict__ row_off, int64_t nrows, int b,
                    const qsft_job* __restrict__ jobs, const int32_t* __restrict__ row_meta) {
  extern __shared__ __align__(16) unsigned char smem[];
  c2<T>* tile = reinterpret_cast<c2<T>*>(smem);
  constexpr int LQ = Q == 4 ? 2 : 1;  // bits per digit
  constexpr int DPP = 4 / LQ;         // digits per full pass (16 elements)
  const int B = 1 << (LQ * b);
  const int t = threadIdx.x;
  const T scale = (T)1 / (T)B;        // exact: B is a power of two
  const int npass = (b + DPP - 1) / DPP;
  for (int64_t row = blockIdx.x; row < nrows; row += gridDim.x) {
    c2<T>* x = data + __ldg(row_off + row);
    if (t == 0 && row + (int64_t)gridDim.x < nrows) {  // this CTA's next row, into L2
      const c2<T>* nx = data + __ldg(row_off + row + (int64_t)gridDim.x);
      const uint32_t bytes = (uint32_t)B * (uint32_t)sizeof(c2<T>);
      if (((reinterpret_cast<uintptr_t>(nx) | bytes) & 15) == 0)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(nx), "r"(bytes) : "memory");
    }
    RowNoise nz = {make_uint2(0, 0), 0, 0.0};
    if (jobs) {
      const qsft_job* jb = jobs + __ldg(row_meta + 2 * row);
      nz.key = noise_key(jb->noise_seed);
      nz.row = __ldg(row_meta + 2 * row + 1);
      nz.nu = jb->noise_nu;
    }
    c2<T> v[16];
    // pass order (the digit axes are independent): the groups between the
    // top and the lowest DPP digits from high to low (the first reads global
    // memory; its values are at least 16 apart, so lanes cover whole lines),
    // then the lowest DPP digits, and the top DPP digits last: consecutive
    // lanes store consecutive values, and each thread holds entries e and
    // e + B/2 for the noise draws
    const int nmid = npass - 2;
    for (int p = 0; p < npass; ++p) {
      int d0, d1;
      if (p < nmid) {
        d1 = b - DPP - (nmid - 1 - p) * DPP;
        d0 = d1 - DPP > DPP ? d1 - DPP : DPP;
      } else if (p == nmid) {
        d0 = b - DPP;
        d1 = b;
      } else {
        d0 = 0;
        d1 = DPP;
      }
      const int mode = p == 0 ? 0 : (p == npass - 1 ? 2 : 1);
      row_pass_any<T, Q>(d1 - d0, v, t, B, 1 << (LQ * (b - d1)), mode, x, tile, scale, nz);
      __syncthreads();
    }
  }
}

template <typename T, int Q>
static int launch_row(c2<T>* data, const int64_t* row_off, int64_t nrows, int b, cudaStream_t st,
                      const qsft_job* jobs = nullptr, const int32_t* row_meta = nullptr) {
  const int LQ = Q == 4 ? 2 : 1;
  const int B = 1 << (LQ * b);
  const int threads = B / 16;
  const int sm = (B + B / 16) * (int)sizeof(c2<T>);
  auto kern = gwht_row_kernel<T, Q>;
  if (!ensure_smem((const void*)kern, sm)) return QSFT_ERR_CUDA;
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return QSFT_ERR_CUDA;
  }
  // resident CTAs per SM: shared memory and threads
  int per = (227 * 1024) / (sm + 1024);
  if (per > 2048 / threads) per = 2048 / threads;
  if (per < 1) per = 1;
  int64_t grid = (int64_t)sms * per;
  if (grid > nrows) grid = nrows;
  kern<<<(unsigned)grid, threads, sm, st>>>(data, row_off, nrows, b, jobs, row_meta);
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
}

// ---------------------------------------------------------------- row-cluster path
// q in {2, 4}, rows of B = RC_SL * CS values (CS = 2, 4 or 8): a thread-block
// cluster of CS CTAs per row, CTA r holding the slice [r*RC_SL, (r+1)*RC_SL)
// in shared memory (RC_SL/16 threads, 16 values each).  Three passes over the
// slice's 12 low bits (the first reads global memory, coalesced: lanes on
// consecutive values; the tile is padded by one value per 16 as in the row
// kernel), then one pass over the top log2(CS) bits across the cluster: each
// thread takes its CTA's share of the slice offsets, reads the CS values of an
// offset from the CS slices (distributed shared memory), transforms them, and
// stores them -- scaled and with the row's device noise -- straight to global
// memory.  Entries o + RC_SL*k and o + RC_SL*(k + CS/2) are e and e + B/2, so a
// thread draws one noise pair for both, the same values as the row kernel and
// the separate noise pass.  A CTA needs a quarter of the row kernel's shared
// memory, so several rows are in flight on an SM: one row's loads overlap
// another's butterflies.
constexpr int RC_SL = 4096;
constexpr int RC_THREADS = RC_SL / 16;

template <typename T, int Q, int CS>
__global__ void __launch_bounds__(RC_THREADS, sizeof(T) == 4 ? 4 : 2) gwht_rowc_kernel(c2<T>* __restrict__ data,
                                                               const int64_t* __restrict__ row_off,
                                                               const qsft_job* __restrict__ jobs,
                                                               const int32_t* __restrict__ row_meta) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char smem[];
  c2<T>* tile = reinterpret_cast<c2<T>*>(smem);
  const int rank = (int)cluster.block_rank();
  const int64_t row = blockIdx.x / CS;
  c2<T>* __restrict__ x = data + __ldg(row_off + row);
  const c2<T>* __restrict__ xs = x + (int64_t)rank * RC_SL;
  const int t = threadIdx.x;
  constexpr int B = RC_SL * CS;
  const RowNoise nz = [&] {
    RowNoise r = {make_uint2(0, 0), 0, 0.0};
    if (jobs) {
      const qsft_job* jb = jobs + __ldg(row_meta + 2 * row);
      r.key = noise_key(jb->noise_seed);
      r.row = __ldg(row_meta + 2 * row + 1);
      r.nu = jb->noise_nu;
    }
    return r;
  }();
  c2<T> v[16];
  // bits [8, 12): e = t + 256 m, from global memory
#pragma unroll
  for (int m = 0; m < 16; ++m) v[m] = xs[t + 256 * m];
  groups_dft<c2<T>, Q, 16>(v);
#pragma unroll
  for (int m = 0; m < 16; ++m) tile[pad16(t + 256 * m)] = v[m];
  __syncthreads();
  // bits [4, 8): e = (t % 16) + 256 (t / 16) + 16 m
  {
    const int base = (t & 15) + ((t >> 4) << 8);
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = tile[pad16(base + 16 * m)];
    groups_dft<c2<T>, Q, 16>(v);
#pragma unroll
    for (int m = 0; m < 16; ++m) tile[pad16(base + 16 * m)] = v[m];
  }
  __syncthreads();
  // bits [0, 4): e = 16 t + m
#pragma unroll
  for (int m = 0; m < 16; ++m) v[m] = tile[pad16(16 * t + m)];
  groups_dft<c2<T>, Q, 16>(v);
#pragma unroll
  for (int m = 0; m < 16; ++m) tile[pad16(16 * t + m)] = v[m];
  cluster.sync();  // every slice transformed along its low bits
  // the top log2(CS) bits across the cluster; this CTA's offsets [rank*OPC, (rank+1)*OPC)
  constexpr int OPC = RC_SL / CS;
  const c2<T>* part[CS];
#pragma unroll
  for (int k = 0; k < CS; ++k) part[k] = cluster.map_shared_rank(tile, k);
  const T scale = (T)1 / (T)B;
  const T tnu = (T)nz.nu;
#pragma unroll 1
  for (int o = rank * OPC + t; o < (rank + 1) * OPC; o += RC_THREADS) {
    c2<T> w[CS];
#pragma unroll
    for (int k = 0; k < CS; ++k) w[k] = part[k][pad16(o)];
    if constexpr (CS == Q) {
      dft_small<c2<T>, Q>(w, nullptr);
    } else {  // q = 2: the 2-point DFT along each of the log2(CS) binary digits
#pragma unroll
      for (int st = CS / 2; st >= 1; st /= 2)
#pragma unroll
        for (int k = 0; k < CS; ++k)
          if (!(k & st)) {
            const c2<T> a = w[k], c = w[k + st];
            w[k] = cadd(a, c);
            w[k + st] = csub(a, c);
          }
    }
#pragma unroll
    for (int k = 0; k < CS / 2; ++k) {
      const int64_t e0 = o + (int64_t)RC_SL * k, e1 = e0 + B / 2;
      c2<T> a = w[k], c = w[k + CS / 2];
      a.x *= scale;
      a.y *= scale;
      c.x *= scale;
      c.y *= scale;
      if (nz.nu > 0.0) {
        c2<T> g0, g1;
        noise_pair<T>(nz.key, nz.row, B / 2, e0, g0, g1);
        a.x += tnu * g0.x;
        a.y += tnu * g0.y;
        c.x += tnu * g1.x;
        c.y += tnu * g1.y;
      }
      x[e0] = a;
      x[e1] = c;
    }
  }
  cluster.sync();  // the other CTAs have read this CTA's slice
}

template <typename T, int Q, int CS>
static int launch_rowc(c2<T>* data, const int64_t* row_off, int64_t nrows, cudaStream_t st, const qsft_job* jobs,
                       const int32_t* row_meta) {
  const size_t sm = (size_t)(RC_SL + RC_SL / 16) * sizeof(c2<T>);
  auto kern = gwht_rowc_kernel<T, Q, CS>;
  if (!ensure_smem((const void*)kern, (int)sm)) return QSFT_ERR_CUDA;
  if (nrows * CS > 0x7fffffffLL) return QSFT_ERR_TOO_LARGE;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(nrows * CS));
  cfg.blockDim = dim3(RC_THREADS);
  cfg.dynamicSmemBytes = sm;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, kern, data, row_off, jobs, row_meta) != cudaSuccess) return QSFT_ERR_CUDA;
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
}

// the row-cluster kernel for B = 2^bits values, q in {2, 4}: bits 13..15 (CS = 2, 4, 8)
template <typename T>
static int launch_rowc_bits(int q, int bits, c2<T>* d, const int64_t* row_off, int64_t nrows, cudaStream_t st,
                            const qsft_job* jobs, const int32_t* row_meta) {
  if (q == 4 && bits == 14) return launch_rowc<T, 4, 4>(d, row_off, nrows, st, jobs, row_meta);
  if (q == 2 && bits == 13) return launch_rowc<T, 2, 2>(d, row_off, nrows, st, jobs, row_meta);
  if (q == 2 && bits == 14) return launch_rowc<T, 2, 4>(d, row_off, nrows, st, jobs, row_meta);
  if (q == 2 && bits == 15) return launch_rowc<T, 2, 8>(d, row_off, nrows, st, jobs, row_meta);
  return QSFT_ERR_ARG;
}

// ---------------------------------------------------------------- cluster path
// A row of B = q^b values is split over a cluster of CS = q^k CTAs (CTA j holds
// elements [j*Bp, (j+1)*Bp), Bp = B/CS).  Axes 0..k-1 span the CTAs: their
// butterflies read and write the other CTAs' shared memory (DSMEM), each CTA
// taking an equal share of the groups; axes k..b-1 are local to each part.
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// A part is moved by the TMA engine (one bulk copy and a bounded mbarrier wait)
// only when the call has a status word to report a timed-out wait to
// (status_word non-null) and the part is 16-byte aligned; otherwise by plain
// loads.  After a timed-out wait no CTA of the cluster touches the row: each
// CTA reads every peer's flag through DSMEM after the first cluster barrier,
// so the whole cluster skips the exchange and the stores alike, and the first
// CTA records QSFT_ERR_TIMEOUT in the status word.
template <typename T, int Q>
__global__ void __launch_bounds__(512) gwht_cluster_kernel(c2<T>* __restrict__ data,
                                                           const int64_t* __restrict__ row_off, int q, int b, int k,
                                                           int CS, T inv, const qsft_job* __restrict__ jobs,
                                                           const int32_t* __restrict__ row_meta,
                                                           int* __restrict__ status_word) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem);
  int* status = reinterpret_cast<int*>(smem + 8);
  c2<T>* tw = reinterpret_cast<c2<T>*>(smem + 16);
  c2<T>* part = tw + QSFT_MAX_Q;
  const int rank = (int)cluster.block_rank();
  const int64_t row = blockIdx.x / CS;
  int Bp = 1;
  for (int i = k; i < b; ++i) Bp *= q;
  c2<T>* __restrict__ x = data + __ldg(row_off + row) + (int64_t)rank * Bp;
  const uint32_t bytes = (uint32_t)Bp * (uint32_t)sizeof(c2<T>);
  // the TMA engine moves the part when source, destination and size are 16-byte aligned
  const bool bulk = status_word != nullptr && ((reinterpret_cast<uintptr_t>(x) | bytes) & 15) == 0;
  if (threadIdx.x == 0) {
    *status = 1;
    if (bulk) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(mbar)) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(mbar)), "r"(bytes)
                   : "memory");
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
              smem_addr(part)),
          "l"(x), "r"(bytes), "r"(smem_addr(mbar))
          : "memory");
    }
  }
  if (threadIdx.x < q) {
    const double2 w = root_of_unity(threadIdx.x, q);
    tw[threadIdx.x] = cmake<c2<T>>(w.x, -w.y);
  }
  if (bulk) {
    __syncthreads();  // barrier initialised before anyone waits on it
    bool done = false;
    // bounded wait; on a timeout wait once more (bounded) so that the copy is not
    // left writing into shared memory this CTA is about to give up
    for (int attempt = 0; attempt < 2 && !done; ++attempt) {
      for (long long i = 0; i < (1ll << 22) && !done; ++i) {
        uint32_t okp;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\tselp.u32 %0, 1, 0, "
            "p;\n}\n"
            : "=r"(okp)
            : "r"(smem_addr(mbar))
            : "memory");
        done = okp != 0;
      }
      if (!done && threadIdx.x == 0) *status = 0;  // the row is left untouched
    }
  } else {
    for (int e = threadIdx.x; e < Bp; e += blockDim.x) part[e] = x[e];
  }
  cluster.sync();
  // every part landed? (the same answer in every CTA of the cluster)
  bool all_ok = true;
  for (int r = 0; r < CS; ++r) all_ok &= *cluster.map_shared_rank(status, r) != 0;
  if (!all_ok) {
    if (rank == 0 && threadIdx.x == 0 && status_word) atomicExch(status_word, (int)QSFT_ERR_TIMEOUT);
    cluster.sync();  // peers have read this CTA's flag before it exits
    return;
  }
  // ---- axes spanning the cluster
  const int ngroups = (CS / q) * Bp;  // per axis
  const int per = ngroups / CS;
  int cstride = CS;                   // stride of digit a in CTA-index units
  for (int a = 0; a < k; ++a) {
    cstride /= q;
    for (int gi = threadIdx.x; gi < per; gi += blockDim.x) {
      const int G = rank * per + gi;
      const int g = G % Bp;            // local index
      const int ch = G / Bp;            // CTA index with digit a removed
      const int lo = ch % cstride, hi = ch / cstride;
      const int cta0 = hi * cstride * q + lo;
      c2<T> v[Q > 0 ? Q : QSFT_MAX_Q];
      for (int m = 0; m < q; ++m)
        v[m] = *cluster.map_shared_rank(part + g, cta0 + m * cstride);
      if constexpr (Q > 0) {
        dft_small<c2<T>, Q>(v, tw);
      } else {
        c2<T> y[QSFT_MAX_Q];
        for (int kk = 0; kk < q; ++kk) {
          c2<T> acc = v[0];
          int idx = 0;
          for (int m = 1; m < q; ++m) {
            idx += kk;
            if (idx >= q) idx -= q;
            acc = cadd(acc, cmul(v[m], tw[idx]));
          }
          y[kk] = acc;
        }
        for (int kk = 0; kk < q; ++kk) v[kk] = y[kk];
      }
      for (int m = 0; m < q; ++m) *cluster.map_shared_rank(part + g, cta0 + m * cstride) = v[m];
    }
    cluster.sync();
  }
  // ---- local axes
  int stride = Bp;
  for (int a = k; a < b; ++a) {
    stride /= q;
    if constexpr (Q > 0) axis_pass_fixed<T, Q>(part, Bp, stride, tw);
    else axis_pass_generic<T>(part, Bp, stride, q, tw);
    __syncthreads();
  }
  // scale by 1/q^b and, with jobs, add the row's device bin noise (entry rank*Bp + e)
  RowNoise nz = {make_uint2(0, 0), 0, 0.0};
  if (jobs) {
    const qsft_job* jb = jobs + __ldg(row_meta + 2 * row);
    nz.key = noise_key(jb->noise_seed);
    nz.row = __ldg(row_meta + 2 * row + 1);
    nz.nu = jb->noise_nu;
  }
  const T tnu = (T)nz.nu;
  const int64_t half = ((int64_t)Bp * CS + 1) / 2;
  auto finish = [&](c2<T> v, int e) {
    v.x *= inv;
    v.y *= inv;
    if (nz.nu > 0.0) {
      const c2<T> g = noise_one<T>(nz.key, nz.row, half, (int64_t)rank * Bp + e);
      v.x += tnu * g.x;
      v.y += tnu * g.y;
    }
    return v;
  };
  if (bulk) {
    for (int e = threadIdx.x; e < Bp; e += blockDim.x) part[e] = finish(part[e], e);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0 && *status) {
      asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(x), "r"(smem_addr(part)),
                   "r"(bytes)
                   : "memory");
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");  // smem must outlive the copy's reads
    }
  } else {
    for (int e = threadIdx.x; e < Bp; e += blockDim.x) x[e] = finish(part[e], e);
  }
}

// cluster size for a row of q^b values of es bytes, or 0 when the row fits one
// CTA (<= 48 KB) or no q^k <= 8 brings a part under 64 KB
static int cluster_split(int q, int b, size_t es, int* kout) {
  int64_t B = 1;
  for (int i = 0; i < b; ++i) B *= q;
  if ((size_t)B * es <= 48 * 1024) return 0;
  int cs = 1;
  for (int k = 1; k < b; ++k) {
    cs *= q;
    if (cs > 8) return 0;
    if ((size_t)(B / cs) * es <= 64 * 1024) {
      *kout = k;
      return cs;
    }
  }
  return 0;
}

template <typename T, int Q>
static int launch_cluster(c2<T>* data, const int64_t* row_off, int64_t nrows, int q, int b, int k, int CS,
                          T divisor, cudaStream_t st, const qsft_job* jobs, const int32_t* row_meta,
                          int* status_word) {
  int64_t Bp = 1;
  for (int i = k; i < b; ++i) Bp *= q;
  const size_t sm = 16 + (size_t)(Bp + QSFT_MAX_Q) * sizeof(c2<T>);
  auto kern = gwht_cluster_kernel<T, Q>;
  if (!ensure_smem((const void*)kern, (int)sm)) return QSFT_ERR_CUDA;
  if (nrows * CS > 0x7fffffffLL) return QSFT_ERR_TOO_LARGE;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(nrows * CS));
  cfg.blockDim = dim3(Bp >= 4096 ? 512 : 256);
  cfg.dynamicSmemBytes = sm;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, kern, data, row_off, q, b, k, CS, (T)1 / divisor, jobs, row_meta, status_word) !=
      cudaSuccess)
    return QSFT_ERR_CUDA;
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
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
                       T divisor, cudaStream_t st, const qsft_job* jobs, const int32_t* row_meta) {
  const int mid = (int)ipow(q, p.a1 - p.a0), inner = (int)ipow(q, b - p.a1), outer = (int)ipow(q, p.a0);
  const int tiles_per_row = (outer / p.NO) * (inner / p.TI);
  const int nel = p.NO * mid * p.TI;
  const size_t sm = (size_t)(nel + QSFT_MAX_Q) * sizeof(c2<T>);
  auto kern = gwht_pass_kernel<T, Q>;
  if (!ensure_smem((const void*)kern, (int)sm)) return QSFT_ERR_CUDA;
  const int threads = nel >= 4096 ? 512 : (nel >= 1024 ? 256 : 128);
  const int64_t grid = nrows * tiles_per_row;
  if (grid > 0x7fffffffLL) return QSFT_ERR_TOO_LARGE;
  kern<<<(unsigned)grid, threads, sm, st>>>(data, row_off, q, p.a1 - p.a0, mid, inner, p.TI, p.NO,
                                            tiles_per_row, (T)1 / divisor, ipow(q, b), jobs, row_meta);
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
}

// ---------------------------------------------------------------- schedules
// The kernels that can transform rows of a (q, b) shape, chosen per shape:
// the built-in rule (QSFT_GWHT_AUTO), or the schedule the caller selected
// with qsft_gwht_select -- normally the winner of a timing of every valid
// schedule on the device (the autotuner of qsft_gb300/autotune.py).
static std::atomic<int> g_sched[2][QSFT_MAX_Q + 1][23];  // [FP32, FP64][q][b]

static int rowc_ok(int q, int b) {
  const int bits = (q == 4 ? 2 : 1) * b;
  return (q == 4 && bits == 14) || (q == 2 && bits >= 13 && bits <= 15);
}
static int row_ok(int q, int b, size_t es) {
  if (q != 2 && q != 4) return 0;
  const int bits = (q == 4 ? 2 : 1) * b;
  return bits >= 8 && bits <= (es == 8 ? 14 : 13);
}
static int passes_ok(int q, int b, size_t es, size_t budget) {
  Pass passes[24];
  return plan_passes(q, b, es, budget - QSFT_MAX_Q * es, passes, 24) > 0;
}
static int sched_valid(int sched, int q, int b, size_t es) {
  int k = 0;
  switch (sched) {
    case QSFT_GWHT_ROW: return row_ok(q, b, es);
    case QSFT_GWHT_ROWC: return rowc_ok(q, b);
    case QSFT_GWHT_CLUSTER: return cluster_split(q, b, es, &k) > 0;
    case QSFT_GWHT_PASSES: return passes_ok(q, b, es, 200 * 1024);
    case QSFT_GWHT_PASSES_SMALL:  // a plan of its own only for rows above 48 KB
      return (size_t)ipow(q, b) * es > 48 * 1024 && passes_ok(q, b, es, 48 * 1024);
    default: return 0;
  }
}
// the built-in rule: the row-cluster kernel, else the row kernel, else a
// cluster per row, else tile passes through global memory
static int sched_default(int q, int b, size_t es) {
  const int order[] = {QSFT_GWHT_ROWC, QSFT_GWHT_ROW, QSFT_GWHT_CLUSTER, QSFT_GWHT_PASSES};
  for (int s : order)
    if (sched_valid(s, q, b, es)) return s;
  return 0;
}

template <typename T>
static int run_gwht(int q, int b, void* data, const int64_t* row_off, int64_t nrows, cudaStream_t st,
                    const qsft_job* jobs = nullptr, const int32_t* row_meta = nullptr, int* status_word = nullptr) {
  const size_t es = sizeof(c2<T>);
  int sched = g_sched[es == 8 ? 0 : 1][q][b].load(std::memory_order_relaxed);
  if (sched == QSFT_GWHT_AUTO || !sched_valid(sched, q, b, es)) sched = sched_default(q, b, es);
  if (!sched) return QSFT_ERR_TOO_LARGE;
  c2<T>* d = reinterpret_cast<c2<T>*>(data);
  const T div = (T)ipow(q, b);
  const int bits = (q == 4 ? 2 : 1) * b;
  if (sched == QSFT_GWHT_ROWC) return launch_rowc_bits<T>(q, bits, d, row_off, nrows, st, jobs, row_meta);
  if (sched == QSFT_GWHT_ROW)
    return q == 4 ? launch_row<T, 4>(d, row_off, nrows, b, st, jobs, row_meta)
                  : launch_row<T, 2>(d, row_off, nrows, b, st, jobs, row_meta);
  // other schedules: the noise (jobs non-null) goes into the last pass, one draw per entry
  if (sched == QSFT_GWHT_CLUSTER) {
    int k = 0;
    const int CS = cluster_split(q, b, es, &k);
    switch (q) {
      case 2: return launch_cluster<T, 2>(d, row_off, nrows, q, b, k, CS, div, st, jobs, row_meta, status_word);
      case 3: return launch_cluster<T, 3>(d, row_off, nrows, q, b, k, CS, div, st, jobs, row_meta, status_word);
      case 4: return launch_cluster<T, 4>(d, row_off, nrows, q, b, k, CS, div, st, jobs, row_meta, status_word);
      case 5: return launch_cluster<T, 5>(d, row_off, nrows, q, b, k, CS, div, st, jobs, row_meta, status_word);
      default: return launch_cluster<T, 0>(d, row_off, nrows, q, b, k, CS, div, st, jobs, row_meta, status_word);
    }
  }
  const size_t budget = (sched == QSFT_GWHT_PASSES_SMALL ? 48 : 200) * 1024 - QSFT_MAX_Q * es;
  Pass passes[24];
  const int np = plan_passes(q, b, es, budget, passes, 24);
  if (np <= 0) return QSFT_ERR_TOO_LARGE;
  for (int i = 0; i < np; ++i) {
    const bool last = i == np - 1;
    const T dv = last ? div : (T)1;
    const qsft_job* jl = last ? jobs : nullptr;
    const int32_t* ml = last ? row_meta : nullptr;
    int rc;
    switch (q) {
      case 2: rc = launch_pass<T, 2>(d, row_off, nrows, q, b, passes[i], dv, st, jl, ml); break;
      case 3: rc = launch_pass<T, 3>(d, row_off, nrows, q, b, passes[i], dv, st, jl, ml); break;
      case 4: rc = launch_pass<T, 4>(d, row_off, nrows, q, b, passes[i], dv, st, jl, ml); break;
      case 5: rc = launch_pass<T, 5>(d, row_off, nrows, q, b, passes[i], dv, st, jl, ml); break;
      case 20:  // 4 x 5 in registers; FP64 keeps the generic DFT (register pressure)
        rc = sizeof(T) == 4 ? launch_pass<T, 20>(d, row_off, nrows, q, b, passes[i], dv, st, jl, ml)
                            : launch_pass<T, 0>(d, row_off, nrows, q, b, passes[i], dv, st, jl, ml);
        break;
      default: rc = launch_pass<T, 0>(d, row_off, nrows, q, b, passes[i], dv, st, jl, ml); break;
    }
    if (rc != QSFT_OK) return rc;
  }
  return QSFT_OK;
}

}  // namespace qsft

using namespace qsft;

extern "C" int qsft_gwht_noise(const qsft_plan* plan, int q, int b, const int64_t* row_off, const int32_t* row_meta,
                               int64_t nrows, qsft_stream_t stream) {
  if (!plan || !plan->jobs || !plan->U || q < 2 || q > QSFT_MAX_Q || b < 1 || nrows < 0) return QSFT_ERR_ARG;
  if (ipow(q, b) > (1LL << 22)) return QSFT_ERR_TOO_LARGE;
  if (nrows == 0) return QSFT_OK;
  if (!row_off || !row_meta) return QSFT_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (plan->prec == QSFT_F32)
    return run_gwht<float>(q, b, plan->U, row_off, nrows, st, plan->jobs, row_meta, plan->status);
  if (plan->prec == QSFT_F64)
    return run_gwht<double>(q, b, plan->U, row_off, nrows, st, plan->jobs, row_meta, plan->status);
  return QSFT_ERR_ARG;
}

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

static int prec_es(int prec) { return prec == QSFT_F32 ? 8 : (prec == QSFT_F64 ? 16 : 0); }

extern "C" int qsft_gwht_schedules(int prec, int q, int b, int32_t* ids, int max_ids) {
  const int es = prec_es(prec);
  if (!es || q < 2 || q > QSFT_MAX_Q || b < 1 || b > 22 || ipow(q, b) > (1LL << 22) || max_ids < 0) return QSFT_ERR_ARG;
  int n = 0;
  for (int s = QSFT_GWHT_ROW; s <= QSFT_GWHT_PASSES_SMALL; ++s)
    if (sched_valid(s, q, b, (size_t)es)) {
      if (ids && n < max_ids) ids[n] = s;
      ++n;
    }
  return n;
}

extern "C" int qsft_gwht_select(int prec, int q, int b, int schedule) {
  const int es = prec_es(prec);
  if (!es || q < 2 || q > QSFT_MAX_Q || b < 1 || b > 22 || ipow(q, b) > (1LL << 22)) return QSFT_ERR_ARG;
  if (schedule != QSFT_GWHT_AUTO && !sched_valid(schedule, q, b, (size_t)es)) return QSFT_ERR_ARG;
  g_sched[es == 8 ? 0 : 1][q][b].store(schedule, std::memory_order_relaxed);
  return QSFT_OK;
}

extern "C" int qsft_gwht_selected(int prec, int q, int b) {
  const int es = prec_es(prec);
  if (!es || q < 2 || q > QSFT_MAX_Q || b < 1 || b > 22 || ipow(q, b) > (1LL << 22)) return QSFT_ERR_ARG;
  int s = g_sched[es == 8 ? 0 : 1][q][b].load(std::memory_order_relaxed);
  if (s == QSFT_GWHT_AUTO || !sched_valid(s, q, b, (size_t)es)) s = sched_default(q, b, (size_t)es);
  return s;
}
