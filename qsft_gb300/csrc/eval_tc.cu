// Coset evaluation with the integer dot products on the 5th-generation tensor
// cores (sm_103a tcgen05).
//
// For a tile of 128 query points x (rows) and a chunk of support vectors k_s
// (columns), the dot products <x, k_s> form a 128 x N integer matrix X K^T.
// Digits are < 32, so they are exact in FP16 and every sum (< 2^17) is exact
// in the FP32 accumulator: one tcgen05.mma kind::f16 per 16 digits computes
// them into tensor memory (TMEM).  The epilogue reads TMEM with tcgen05.ld and
// turns each dot into a_s * omega^(dot mod q) with one table lookup
// (mod q from the FP32 value's mantissa bits), summing over s in registers.
//
// CTA = 8 warps.  Operands live in shared memory in the no-swizzle K-major
// core-matrix layout (8 rows x 16 bytes per core matrix; LBO = 128 B between
// the core matrices of consecutive K chunks, SBO = K*2 B between groups of 8
// rows).  TMEM holds two 128-column FP32 accumulators so that the MMA of
// support sub-tile j+1 overlaps the epilogue of sub-tile j.  Every mbarrier
// wait is bounded; a timeout sets plan.status and the CTA still frees TMEM.
#include "common.cuh"
#include "tcgen05.cuh"

namespace qsft {
namespace tc {

constexpr int THREADS = 256;
constexpr int TILE_M = 128;
constexpr int SUB_N = 128;
constexpr int TMEM_COLS = 256;
constexpr int HDR = 2048;                  // barriers, TMEM slot, roots, partial sums
constexpr int MIN_SMEM = 80 * 1024;        // > 228/3 KB: at most 2 CTAs (512 TMEM columns) per SM
__device__ __forceinline__ uint32_t pack_h2(uint32_t lo, uint32_t hi) {
  const __half2 h = __halves2half2(__uint2half_rn(lo), __uint2half_rn(hi));
  return *reinterpret_cast<const uint32_t*>(&h);
}

inline size_t smem_bytes(int npad, int smax, int entry_bytes, int64_t table_bytes) {
  size_t b = HDR + (size_t)TILE_M * npad * 2 + (size_t)smax * npad * 2 + (size_t)smax * entry_bytes +
             (size_t)table_bytes;
  return b < (size_t)MIN_SMEM ? (size_t)MIN_SMEM : b;
}

__device__ __forceinline__ uint64_t lds64(uint32_t addr) {
  uint64_t v;
  asm volatile("ld.shared.b64 %0, [%1];" : "=l"(v) : "r"(addr));
  return v;
}
template <int IMM>
__device__ __forceinline__ uint64_t lds64_imm(uint32_t addr) {
  uint64_t v;
  asm volatile("ld.shared.b64 %0, [%1+%2];" : "=l"(v) : "r"(addr), "n"(IMM));
  return v;
}
__device__ __forceinline__ uint64_t add_f32x2(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ void red_add_v2(float* addr, float x, float y) {
  asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(addr), "f"(x), "f"(y) : "memory");
}

// acc[0..3] += sum over 16 TMEM columns (support entries s_rel .. s_rel+15)
// of a_s omega^(dot mod q).
//
// q in {2, 4} (QT): the table holds one row per PAIR of support entries,
// T[p][ma][mb] = a_2p omega^ma + a_2p+1 omega^mb (q*q entries of 8 bytes), so
// one lookup serves two columns.  v + 2^23 puts the integer v in the FP32
// mantissa, so fma(v, S, 2^23) holds S*v in its low bits; masking gives the
// byte offset S*(v mod q) for S = 8*QT (column 2p) and S = 8 (column 2p+1).
// The pair-row base is aligned to the table row size times 8, so OR adds the
// offsets and the row offset of pair p rides in the load's immediate.
template <int QT, int C>
__device__ __forceinline__ void add_pair(const uint32_t (&r)[16], uint32_t rowbase, uint64_t (&acc)[4]) {
  constexpr uint32_t mask_a = (uint32_t)(QT - 1) * QT * 8, mask_b = (uint32_t)(QT - 1) * 8;
  const uint32_t ba = __float_as_uint(fmaf(__uint_as_float(r[C]), (float)(QT * 8), 8388608.0f));
  const uint32_t bb = __float_as_uint(fmaf(__uint_as_float(r[C + 1]), 8.0f, 8388608.0f));
  const uint32_t off = (ba & mask_a) | ((bb & mask_b) | rowbase);
  acc[(C >> 1) & 3] = add_f32x2(acc[(C >> 1) & 3], lds64_imm<(C >> 1) * QT * QT * 8>(off));
}
template <int QT, int C>
__device__ __forceinline__ void add_pairs(const uint32_t (&r)[16], uint32_t rowbase, uint64_t (&acc)[4]) {
  if constexpr (C < 16) {
    add_pair<QT, C>(r, rowbase, acc);
    add_pairs<QT, C + 2>(r, rowbase, acc);
  }
}
template <int QT>
__device__ __forceinline__ void reduce16(const uint32_t (&r)[16], uint32_t sT_addr, const float2* __restrict__ sT,
                                         int s_rel, int q, ModQ mq, uint64_t (&acc)[4]) {
  if constexpr (QT == 2 || QT == 4) {
    add_pairs<QT, 0>(r, sT_addr + (uint32_t)(s_rel >> 1) * QT * QT * 8, acc);
  } else {
    const float2* rowp = sT + (size_t)s_rel * q;
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      const uint32_t v = __float_as_uint(__uint_as_float(r[c]) + 8388608.0f) & 0x7FFFFFu;
      const uint32_t m = v - mq.q * __umulhi(v, mq.mul);
      const float2 t = rowp[c * q + m];
      acc[c & 3] = add_f32x2(acc[c & 3], *reinterpret_cast<const uint64_t*>(&t));
    }
  }
}

// four packed bytes (each < 1024) -> two half2 words holding the same integers:
// 0x6400 | v is the FP16 encoding of 1024 + v, so subtracting 1024 leaves v.
__device__ __forceinline__ void bytes_to_h2(uint32_t w, uint32_t& lo, uint32_t& hi) {
  const uint32_t a = __byte_perm(w, 0x64006400u, 0x7150);  // [b0, 0x64, b1, 0x64]
  const uint32_t b = __byte_perm(w, 0x64006400u, 0x7352);  // [b2, 0x64, b3, 0x64]
  const __half2 k1024 = __halves2half2(__ushort_as_half(0x6400), __ushort_as_half(0x6400));
  const __half2 ha = __hsub2(*reinterpret_cast<const __half2*>(&a), k1024);
  const __half2 hb = __hsub2(*reinterpret_cast<const __half2*>(&b), k1024);
  lo = *reinterpret_cast<const uint32_t*>(&ha);
  hi = *reinterpret_cast<const uint32_t*>(&hb);
}

// Roles: every warp builds its share of the query-digit tile sA, then reduces
// one lane quarter (32 sample rows) x one column half (64 support entries) of
// each accumulator; lane 0 of warp 0 also issues the MMAs.  Handshakes, all
// mbarriers with bounded waits:
//   aready     8 warp arrivals: sA of the current tile is written
//   full[b]    tcgen05.commit: accumulator b holds a finished sub-tile
//   empty[b]   8 warp arrivals: accumulator b has been read out
template <int NPAD, int QT>
__global__ void __launch_bounds__(THREADS, 2) eval_tc_kernel(qsft_plan plan) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);            // [2]
  uint64_t* empty = full + 2;                                     // [2]
  uint64_t* aready = full + 4;                                    // [1]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 48);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + 52);
  float2* sW = reinterpret_cast<float2*>(smem + 128);            // 32 roots
  unsigned char* sA = smem + HDR;                                 // 128 x NPAD fp16
  unsigned char* sB = sA + TILE_M * NPAD * 2;                     // smax x NPAD fp16
  const int smax = plan.tc_smax;
  float2* sT = reinterpret_cast<float2*>(sB + (size_t)smax * NPAD * 2);  // smax x q
  // digit tables: sX[(c*b + t)*q + v] = NPAD bytes (M[c][i][t] * v) mod q, i < n;
  //               sD[c*RP + rp]       = NPAD bytes d_{c,rp}[i]
  unsigned char* sX = reinterpret_cast<unsigned char*>(sT) + (size_t)smax * plan.tc_entry_bytes;

  constexpr uint32_t SBO = NPAD * 16;  // bytes between 8-row groups
  constexpr uint32_t IDESC = make_idesc(TILE_M, SUB_N);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // ---- work item
  const int64_t w = blockIdx.x;
  const int j = find_job(plan.tc_prefix, plan.njobs, w);
  const qsft_job* __restrict__ job = plan.jobs + j;
  const int q = QT ? QT : job->q;
  const int n = job->n, b = job->b, B = job->B, S = job->S, RP = job->R * job->P;
  const int64_t total = (int64_t)job->C * RP * B;
  const int64_t tiles = (total + TILE_M - 1) / TILE_M;
  const int64_t groups = (tiles + QSFT_TC_TILES - 1) / QSFT_TC_TILES;
  const int64_t local = w - plan.tc_prefix[j];
  const int chunk = (int)(local / groups);
  const int64_t grp = local - (int64_t)chunk * groups;
  const int s0 = chunk * smax;
  const int scnt = min(smax, S - s0);
  const int nsub = (scnt + SUB_N - 1) / SUB_N;
  const int8_t* __restrict__ M = plan.i8 + job->off_M;
  const int8_t* __restrict__ D = plan.i8 + job->off_D;
  const int8_t* __restrict__ K = plan.i8 + job->off_K + (int64_t)s0 * n;
  const float2* __restrict__ A = reinterpret_cast<const float2*>(plan.A) + job->off_A + s0;
  float2* __restrict__ U = reinterpret_cast<float2*>(plan.U) + job->off_U;
  const ModQ mq = make_modq(q);

  // ---- setup: TMEM, barriers, roots, support operand and table
  if (warp == 0) {
    tmem_alloc(tmem_slot, TMEM_COLS);
    tmem_relinquish();
  }
  if (tid == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    mbar_init(&empty[0], THREADS / 32);
    mbar_init(&empty[1], THREADS / 32);
    mbar_init(aready, THREADS / 32);
    *abort_flag = 0;
    fence_mbar_init();
  }
  if (tid < q) {
    const double2 wr = root_of_unity(tid, q);
    sW[tid] = make_float2((float)wr.x, (float)wr.y);
  }
  __syncthreads();
  const int rows_b = nsub * SUB_N;
  for (int idx = tid; idx < rows_b * (NPAD / 8); idx += THREADS) {
    const int r = idx / (NPAD / 8), kc = idx - (idx / (NPAD / 8)) * (NPAD / 8);
    uint32_t d[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int i = kc * 8 + e;
      d[e] = (r < scnt && i < n) ? (uint32_t)(uint8_t)__ldg(K + (int64_t)r * n + i) : 0u;
    }
    uint4 v = make_uint4(pack_h2(d[0], d[1]), pack_h2(d[2], d[3]), pack_h2(d[4], d[5]), pack_h2(d[6], d[7]));
    *reinterpret_cast<uint4*>(sB + (r >> 3) * SBO + kc * 128 + (r & 7) * 16) = v;
  }
  // FP32 products: GB300's FP64 rate is a small fraction of FP32
  if constexpr (QT == 2 || QT == 4) {
    for (int idx = tid; idx < (rows_b / 2) * QT * QT; idx += THREADS) {
      const int p = idx / (QT * QT), ma = (idx / QT) % QT, mb = idx % QT;
      float2 v = make_float2(0.f, 0.f);
      if (2 * p < scnt) {
        const float2 a = A[2 * p], w2 = sW[ma];
        v = make_float2(fmaf(a.x, w2.x, -a.y * w2.y), fmaf(a.x, w2.y, a.y * w2.x));
      }
      if (2 * p + 1 < scnt) {
        const float2 a = A[2 * p + 1], w2 = sW[mb];
        v.x += fmaf(a.x, w2.x, -a.y * w2.y);
        v.y += fmaf(a.x, w2.y, a.y * w2.x);
      }
      sT[idx] = v;
    }
  } else {
    for (int idx = tid; idx < rows_b * q; idx += THREADS) {
      const int s = idx / q, rr = idx - (idx / q) * q;
      float2 v = make_float2(0.f, 0.f);
      if (s < scnt) {
        const float2 a = A[s];
        const float2 wr = sW[rr];
        v = make_float2(fmaf(a.x, wr.x, -a.y * wr.y), fmaf(a.x, wr.y, a.y * wr.x));
      }
      sT[idx] = v;
    }
  }
  const int C = job->C;
  unsigned char* sD = sX + (size_t)C * b * q * NPAD;
  for (int idx = tid; idx < C * b * q * (NPAD / 4); idx += THREADS) {
    const int wi = idx % (NPAD / 4), e = idx / (NPAD / 4);  // e = (c*b + t)*q + v
    const int v = e % q, ct = e / q, t = ct % b, c = ct / b;
    uint32_t word = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int i = wi * 4 + k;
      if (i < n) word |= modq((uint32_t)__ldg(M + ((int64_t)c * n + i) * b + t) * (uint32_t)v, mq) << (8 * k);
    }
    reinterpret_cast<uint32_t*>(sX)[idx] = word;
  }
  for (int idx = tid; idx < C * RP * (NPAD / 4); idx += THREADS) {
    const int wi = idx % (NPAD / 4), row_d = idx / (NPAD / 4);
    uint32_t word = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int i = wi * 4 + k;
      if (i < n) word |= (uint32_t)(uint8_t)__ldg(D + (int64_t)row_d * n + i) << (8 * k);
    }
    reinterpret_cast<uint32_t*>(sD)[idx] = word;
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t sA_addr = smem_u32(sA), sB_addr = smem_u32(sB), sT_addr = smem_u32(sT);

  const bool issuer = (tid == 0);
  const int row = tid & (TILE_M - 1), half = tid >> 7;
  const int lq = warp & 3, h = warp >> 2;
  const int trow = lq * 32 + lane;  // the sample row this thread reduces
  uint32_t full_ph[2] = {0, 0}, empty_ph[2] = {1, 1}, ready_ph = 0;  // phases
  bool ok = true;

  for (int ti = 0; ti < QSFT_TC_TILES && ok; ++ti) {
    const int64_t tile = grp * QSFT_TC_TILES + ti;
    if (tile >= tiles) break;
    const int64_t base = tile * TILE_M;
    // ---- query digits of this tile -> sA (the previous tile's MMAs are complete:
    //      this warp waited for the last of them before its last read-out).
    //      x'_i = d_i + sum_t ((M[i][t] l_t) mod q) < 256 is x_i plus a multiple of
    //      q, so <x', k> = <x, k> (mod q); summed four digits per 32-bit word.
    {
      const int64_t gidx = base + row;
      constexpr int HW = NPAD / 8;  // 32-bit words (4 digits each) in this thread's half
      uint32_t xw[HW];
#pragma unroll
      for (int k = 0; k < HW; ++k) xw[k] = 0;
      if (gidx < total) {
        const int64_t rw = gidx / B;
        uint32_t l = (uint32_t)(gidx - rw * B);
        const int c = (int)(rw / RP);
        const int rp = (int)(rw - (int64_t)c * RP);
        const uint32_t* dr = reinterpret_cast<const uint32_t*>(sD + ((size_t)c * RP + rp) * NPAD) + half * HW;
#pragma unroll
        for (int k = 0; k < HW; ++k) xw[k] = dr[k];
        const unsigned char* xc = sX + (size_t)c * b * q * NPAD;
        for (int t = b - 1; t >= 0; --t) {  // l < 2^22: the round-up quotient is exact
          const uint32_t qt = mq.pow2 ? (l >> (31 - __clz(q))) : __umulhi(l, mq.mul);
          const uint32_t lt = l - qt * (uint32_t)q;
          l = qt;
          const uint32_t* tr = reinterpret_cast<const uint32_t*>(xc + ((size_t)t * q + lt) * NPAD) + half * HW;
#pragma unroll
          for (int k = 0; k < HW; ++k) xw[k] += tr[k];
        }
      }
#pragma unroll
      for (int kc = 0; kc < NPAD / 16; ++kc) {  // 8 digits = 2 words -> one 16-byte core-matrix row
        uint4 v;
        bytes_to_h2(xw[2 * kc], v.x, v.y);
        bytes_to_h2(xw[2 * kc + 1], v.z, v.w);
        *reinterpret_cast<uint4*>(sA + (row >> 3) * SBO + (half * (NPAD / 16) + kc) * 128 + (row & 7) * 16) = v;
      }
    }
    fence_async_smem();
    __syncwarp();
    if (lane == 0) mbar_arrive(aready);
    // ---- issue sub-tile 0 once every warp has written its rows of sA
    if (issuer) {
      bool g = mbar_wait(aready, ready_ph) && mbar_wait(&empty[0], empty_ph[0]);
      empty_ph[0] ^= 1;
      tc_fence_after();
      if (g) {
#pragma unroll
        for (int ks = 0; ks < NPAD / 16; ++ks)
          mma_f16(tmem, make_desc(sA_addr + ks * 256, 128, SBO), make_desc(sB_addr + ks * 256, 128, SBO), IDESC,
                  ks > 0);
        mma_commit(&full[0]);
      } else {
        *abort_flag = 1;
      }
    }
    ready_ph ^= 1;
    uint64_t acc[4] = {0, 0, 0, 0};  // (re, im) partial sums of this thread's row over its column half
    for (int sub = 0; sub < nsub; ++sub) {
      const int buf = sub & 1;
      if (issuer && sub + 1 < nsub && !*abort_flag) {  // next sub-tile into the other accumulator
        const bool g = mbar_wait(&empty[buf ^ 1], empty_ph[buf ^ 1]);
        empty_ph[buf ^ 1] ^= 1;
        tc_fence_after();
        if (g) {
          const uint32_t bb = sB_addr + (uint32_t)(sub + 1) * (SUB_N / 8) * SBO;
#pragma unroll
          for (int ks = 0; ks < NPAD / 16; ++ks)
            mma_f16(tmem + (buf ^ 1) * SUB_N, make_desc(sA_addr + ks * 256, 128, SBO),
                    make_desc(bb + ks * 256, 128, SBO), IDESC, ks > 0);
          mma_commit(&full[buf ^ 1]);
        } else {
          *abort_flag = 1;
        }
      }
      __syncwarp();
      const bool got = mbar_wait(&full[buf], full_ph[buf]);
      full_ph[buf] ^= 1;
      if (!got || *abort_flag) {
        *abort_flag = 1;
        ok = false;
        break;
      }
      tc_fence_after();
      {  // 64 columns in four 16-column loads, the next load in flight while one is reduced
        const uint32_t taddr = tmem + ((uint32_t)(lq * 32) << 16) + buf * SUB_N + h * 64;
        const int s_rel = sub * SUB_N + h * 64;
        uint32_t ra[16], rb[16];
        tmem_ld16(taddr, ra);
        tmem_ld_wait_regs(ra);
        tmem_ld16(taddr + 16, rb);
        reduce16<QT>(ra, sT_addr, sT, s_rel, q, mq, acc);
        tmem_ld_wait_regs(rb);
        tmem_ld16(taddr + 32, ra);
        reduce16<QT>(rb, sT_addr, sT, s_rel + 16, q, mq, acc);
        tmem_ld_wait_regs(ra);
        tmem_ld16(taddr + 48, rb);
        reduce16<QT>(ra, sT_addr, sT, s_rel + 32, q, mq, acc);
        tmem_ld_wait_regs(rb);
        reduce16<QT>(rb, sT_addr, sT, s_rel + 48, q, mq, acc);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[buf]);
    }
    if (!ok) break;
    // ---- add this half's partial sums to the samples (U was zeroed by the caller)
    const int64_t gidx = base + trow;
    if (gidx < total) {
      const uint64_t a2 = add_f32x2(add_f32x2(acc[0], acc[1]), add_f32x2(acc[2], acc[3]));
      const float2 f = *reinterpret_cast<const float2*>(&a2);
      red_add_v2(reinterpret_cast<float*>(U + gidx), f.x, f.y);
    }
  }
  if (!ok || *abort_flag) {  // a wait gave up: report, give in-flight MMAs one more bounded wait
    if (tid == 0) atomicExch(plan.status, (int)QSFT_ERR_TIMEOUT);
    mbar_wait(&full[0], full_ph[0]);
    mbar_wait(&full[1], full_ph[1]);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, TMEM_COLS);
}

template <int NPAD, int QT>
static int launch(const qsft_plan* p, cudaStream_t st) {
  const int pairs = (QT == 2 || QT == 4);
  if (p->tc_entry_bytes != (pairs ? QT * QT * 4 : p->max_q * 8)) return QSFT_ERR_ARG;
  const size_t sm = smem_bytes(NPAD, p->tc_smax, p->tc_entry_bytes, p->tc_table_bytes);
  if (sm > 227 * 1024) return QSFT_ERR_TOO_LARGE;
  auto kern = eval_tc_kernel<NPAD, QT>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
    return QSFT_ERR_CUDA;
  kern<<<(unsigned)p->total_tc_work, THREADS, sm, st>>>(*p);
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
}

template <int NPAD>
static int launch_q(const qsft_plan* p, cudaStream_t st) {
  if (p->max_q == 4 && p->min_q == 4) return launch<NPAD, 4>(p, st);
  if (p->max_q == 2 && p->min_q == 2) return launch<NPAD, 2>(p, st);
  return launch<NPAD, 0>(p, st);
}

}  // namespace tc
}  // namespace qsft

using namespace qsft;

extern "C" int qsft_eval_cosets_tc(const qsft_plan* plan, qsft_stream_t stream) {
  if (!plan || plan->njobs <= 0 || !plan->jobs || !plan->tc_prefix || !plan->i8 || !plan->A || !plan->U ||
      !plan->status)
    return QSFT_ERR_ARG;
  if (plan->prec != QSFT_F32) return QSFT_ERR_ARG;
  if (plan->max_q < 2 || plan->max_q > QSFT_MAX_Q || plan->min_q < 2 || plan->max_n > plan->tc_npad)
    return QSFT_ERR_ARG;
  if (plan->tc_smax < tc::SUB_N || plan->tc_smax % tc::SUB_N) return QSFT_ERR_ARG;
  if (plan->total_tc_work <= 0) return QSFT_OK;
  if (plan->total_tc_work > 0x7fffffffLL) return QSFT_ERR_TOO_LARGE;
  cudaStream_t st = (cudaStream_t)stream;
  switch (plan->tc_npad) {
    case 32: return tc::launch_q<32>(plan, st);
    case 64: return tc::launch_q<64>(plan, st);
    case 128: return tc::launch_q<128>(plan, st);
    default: return QSFT_ERR_ARG;
  }
}
