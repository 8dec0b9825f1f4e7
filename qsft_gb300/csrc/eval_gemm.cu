// Coset evaluation as a complex GEMM on the 5th-generation tensor cores.
//
// The samples of group c are U[rp][l] = f(M_c l + d_rp), l in Z_q^b, with
// f(x) = sum_s a_s omega^(<x, k_s>) (synthetic_signal.py:100-118 evaluated on
// the cosets of qsft/input_signal_subsampled.py:183-206).  Because
//   <M_c l + d, k_s> = <l, j_s> + <d, k_s>  (mod q),  j_s = M_c^T k_s mod q,
// every coset row is the same character matrix applied to different
// coefficients:
//   U[rp][l] = sum_s W[l][s] C[s][rp],   W[l][s] = omega^(<l, j_s>),
//                                         C[s][rp] = a_s omega^(<d_rp, k_s>).
// W has q^b rows and S columns, C has S rows and R*P columns: one GEMM per
// (job, group) with K = S replaces S table lookups per sample.
//
// Precision.  For q in {2, 4} the characters are 0, +-1, +-i: exact in FP16.
// Other q use W = W_hi + W_lo (FP16 halves of the FP64 root).  C is scaled by
// a power of two per job (largest |a_s| -> [2^13, 2^14)) and split into
// C_hi + C_lo FP16 halves, so each product carries ~22 significant bits; the
// tensor core multiplies exactly and accumulates in FP32.
//
// Real GEMM layout.  Complex products become real ones over K entries per
// support vector (KPS) and four N columns per delay row, (re, im) x (hi, lo)
// of the coefficient:
//   KPS = 2 (q in {2, 4}):  A[l][2s..2s+1] = [Wr, Wi]
//     B[2s..2s+1][4rp + 0, 1] = [Chr, -Chi], [Clr, -Cli]   (real part of W C)
//     B[2s..2s+1][4rp + 2, 3] = [Chi,  Chr], [Cli,  Clr]   (imaginary part)
//   KPS = 4:                A[l][4s..4s+3] = [Whr, Whi, Wlr, Wli]
//     B rows repeat the two KPS = 2 rows for the W_lo entries.
// The epilogue adds the hi and lo columns.  Putting the C halves on N rather
// than K keeps K at 2 (or 4) entries per support vector and makes each MMA
// wide: halves on K (per K step two MMAs of half the N, each reading the same
// A, into one accumulator) measured 27% slower for the whole evaluation, and
// accumulating the lo products into the hi accumulator lost FP32 accuracy
// for q = 20.  Delay rows go in equal chunks of at most 56
// (N <= 224, so two accumulator buffers of a 128-row tile still fit tensor
// memory).  An operand kernel writes B (and the group's table) into a
// workspace in the exact shared-memory image of each 64-entry K chunk
// (128-byte-swizzled K-major rows), so the GEMM kernel streams it with one
// bulk copy per chunk.  The GEMM kernel generates A in tensor memory from the
// row's digits (two dp4a per support vector for b <= 8) and issues
// tcgen05.mma kind::f16 (M = 128, N, K = 16) into tensor memory.
//
// Work unit: MT tiles of 128 rows of one (job, group, chunk of delay rows).
// The GEMM kernel is persistent (one CTA per SM; units taken from a global
// counter) with three roles: two sets of producer warps (one thread per row
// in each) write the two halves of every A chunk into a tensor-memory ring,
// the second set also reading each unit's accumulators back (tcgen05.ld) and
// storing U; one warp issues the MMAs; one warp streams the B chunks into a
// shared-memory ring with bulk copies (and hands out the units, decoded once
// into a shared-memory queue, each with its group's table of j_s digits and
// FP16 roots copied into one of two table buffers).  A chunk takes a producer
// about as long as its MMAs take the tensor pipe, so one set alone (the
// epilogue warps idle between drains) left the MMA threads waiting for A.
// mbarriers: afull (both producer sets wrote an A chunk) / bfull (bulk copy
// landed), one "chunk consumed" barrier per B slot that frees both rings (one
// commit per chunk), accf (a unit's MMAs completed) / acce (its accumulators
// were read), the unit queue's full / empty and the table buffers' full /
// empty.  Every wait is bounded; on a timeout the CTA sets plan.status, drains
// its copies and MMAs (bounded) and frees its tensor memory.
#include "common.cuh"
#include "tcgen05.cuh"

namespace qsft {
namespace gm {
using namespace qsft::tc;

constexpr int KC = 64;                     // K entries per stage: one 128-byte row (4 MMAs of K = 16)
constexpr int TM = 128;                    // rows per MMA tile
constexpr int HDR = 2048;                  // barriers, TMEM slot, flags, unit queue
constexpr int UNIT_OFF = 1024;             // unit queue: UQ decoded units of UNIT_BYTES
constexpr int UNIT_BYTES = 128;
constexpr int A_COLS = KC / 2;             // TMEM columns of one tile's A chunk (two FP16 per column)
constexpr int PREP_S = 32;                 // support vectors per operand block
constexpr int REGION_HDR = 256;            // per-job header (inverse scale; the first also the unit counter)
constexpr int SCHED_OFF = 8;               // byte offset of the GEMM kernel's work-unit counter in gm_ws
constexpr int TAB_HDR = 256;               // a group's table: FP16 (hi, lo) roots omega^m, m < 32, then j_s words
constexpr int MAX_SMEM = 227 * 1024;

constexpr int RPC_MAX = 56;                // delay rows per N chunk (N = 4 columns each, <= 224)

struct Geo {
  int RPC, nch;       // delay rows per chunk, chunks
  int NP;             // N extent: 4*RPC rounded up to 16
  int S_pad, nK;      // support vectors padded to whole stages, K chunks
  uint32_t CB;        // bytes of one B chunk image (NP x KC FP16)
  uint32_t tab_copy;  // bytes of a group's table the GEMM kernel copies (roots + j words)
  int64_t tab_bytes;  // the table's bytes in the workspace, 256-aligned
  int64_t region_c;   // bytes per group: table + nch x nK B chunks
};
__host__ __device__ inline Geo geo(int RP, int S, int kps, int nw) {
  Geo g;
  g.nch = (RP + RPC_MAX - 1) / RPC_MAX;  // chunks of equal size (the last one at most one row shorter)
  g.RPC = (RP + g.nch - 1) / g.nch;
  g.NP = (4 * g.RPC + 15) / 16 * 16;
  const int spc = KC / kps;
  g.S_pad = (S + spc - 1) / spc * spc;
  g.nK = g.S_pad * kps / KC;
  g.CB = (uint32_t)g.NP * KC * 2;
  g.tab_copy = (uint32_t)(TAB_HDR + g.S_pad * nw * 4);  // S_pad is a multiple of 16: a multiple of 16 bytes
  g.tab_bytes = ((int64_t)g.tab_copy + 255) / 256 * 256;
  g.region_c = g.tab_bytes + (int64_t)g.nch * g.nK * g.CB;
  return g;
}
// shared-memory bytes of one table buffer for the largest table (keeps the B ring 1024-byte aligned)
__host__ __device__ inline int tab_smem(const Geo& g) { return (int)((g.tab_copy + 1023) / 1024 * 1024); }
__host__ __device__ inline int64_t region_bytes(const Geo& g, int C) { return REGION_HDR + (int64_t)C * g.region_c; }

// Operand tiles use the 128-byte-swizzled K-major layout: a row of a tile is
// its 64 K entries (128 bytes), 8 rows form a 1024-byte atom, and the 16-byte
// chunk c of row r is stored at chunk c ^ (r % 8).  Offset of entry k of row r:
__host__ __device__ inline uint32_t sw128(int r, int k) {
  return (uint32_t)(r >> 3) * 1024 + (uint32_t)(r & 7) * 128 + (uint32_t)(((k >> 3) ^ (r & 7)) * 16) +
         (uint32_t)(k & 7) * 2;
}
// tcgen05 shared-memory descriptor of such a tile (atoms 1024-byte aligned):
// start >> 4, LBO 16 B (unused for swizzled K-major), SBO 1024 B between 8-row
// groups, version 1, layout type 2 = 128-byte swizzle
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// FP16 bits of x, and of the remainder x - hi
__device__ __forceinline__ void split_h(double x, __half& hi, __half& lo) {
  hi = __double2half(x);
  lo = __double2half(x - (double)__half2float(hi));
}
__device__ __forceinline__ uint32_t h2_bits(__half lo16, __half hi16) {
  const __half2 h = __halves2half2(lo16, hi16);
  return *reinterpret_cast<const uint32_t*>(&h);
}

// ---------------------------------------------------------------- operands
// Block = (job, group, 32 support vectors).  Writes the scaled C halves into
// the B chunks and the group's table: the packed j_s digits (digit t in byte
// t%4 of word t/4; for q = 2 the digit is doubled so that the GEMM kernel
// works mod 4) after the (hi, lo) FP16 half2 words of omega^m.
// FP32 throughout (GB300's FP64 rate is a small fraction of FP32): a_s is
// FP32 already, the roots come from plan.roots, and the power-of-two scaling
// is exact, so hi + lo carry C to FP32 accuracy.
constexpr int PREP_MAXN = QSFT_MAX_N;
constexpr int PREP_MAXRP = 128;
template <int KPS, int NW>
__global__ void __launch_bounds__(256) gemm_prep_kernel(qsft_plan plan) {
  // k_s and delay rows as int8 digits, rows padded with zeros to whole 32-bit
  // words (stride np4) so that <d, k> is a run of dp4a
  __shared__ __align__(16) int8_t sK[PREP_S * PREP_MAXN];
  __shared__ __align__(16) int8_t sD[PREP_MAXRP * PREP_MAXN];
  __shared__ float2 sW[QSFT_MAX_Q];
  __shared__ float red[8];
  const int nj = plan.njobs;
  const int64_t* __restrict__ idx = plan.gm_index;
  const int64_t w = blockIdx.x;
  const int j = find_job(idx + nj + 1, nj, w);
  const qsft_job* __restrict__ job = plan.jobs + j;
  const int q = job->q, n = job->n, b = job->b, S = job->S, RP = job->R * job->P;
  const Geo g = geo(RP, S, KPS, NW);
  const int sblocks = (g.S_pad + PREP_S - 1) / PREP_S;
  const int64_t local = w - idx[nj + 1 + j];
  const int c = (int)(local / sblocks);
  const int sb = (int)(local - (int64_t)c * sblocks);
  const int s_lo = sb * PREP_S, s_hi = min(s_lo + PREP_S, g.S_pad), s_live = max(0, min(s_hi, S) - s_lo);
  const float2* __restrict__ A = reinterpret_cast<const float2*>(plan.A) + job->off_A;
  const int8_t* __restrict__ M = plan.i8 + job->off_M + (int64_t)c * n * b;
  const int8_t* __restrict__ D = plan.i8 + job->off_D + (int64_t)c * RP * n;
  const int8_t* __restrict__ K = plan.i8 + job->off_K + (int64_t)s_lo * n;
  unsigned char* region = reinterpret_cast<unsigned char*>(plan.gm_ws) + idx[2 * (nj + 1) + j];
  unsigned char* rc = region + REGION_HDR + (int64_t)c * g.region_c;
  const int tid = threadIdx.x;

  const int np4 = (n + 3) & ~3, nw4 = np4 >> 2;
  for (int i = tid; i < s_live * np4; i += blockDim.x) {
    const int r = i / np4, k = i - r * np4;
    sK[i] = k < n ? K[r * n + k] : (int8_t)0;
  }
  for (int i = tid; i < RP * np4; i += blockDim.x) {
    const int r = i / np4, k = i - r * np4;
    sD[i] = k < n ? D[r * n + k] : (int8_t)0;
  }
  if (tid < q) {
    const double* r = plan.roots + ((int64_t)q * 32 + tid) * 2;
    sW[tid] = make_float2((float)r[0], (float)r[1]);
  }
  // scale: 2^(14 - e) with max|a_s| < 2^e
  float mx = 0.f;
  for (int s = tid; s < S; s += blockDim.x) {
    const float2 a = A[s];
    mx = fmaxf(mx, sqrtf(a.x * a.x + a.y * a.y));
  }
  for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(~0u, mx, o));
  if ((tid & 31) == 0) red[tid >> 5] = mx;
  __syncthreads();
  mx = red[0];
  for (int i = 1; i < (int)(blockDim.x >> 5); ++i) mx = fmaxf(mx, red[i]);
  int ex = 0;
  if (mx > 0.f && isfinite(mx)) frexpf(mx, &ex);
  if (c == 0 && sb == 0 && tid == 0) *reinterpret_cast<float*>(region) = ldexpf(1.0f, ex - 14);
  // the GEMM kernel's work-unit counter (header of the first region), reset before it runs
  if (blockIdx.x == 0 && tid == 0)
    *reinterpret_cast<unsigned long long*>(reinterpret_cast<unsigned char*>(plan.gm_ws) + SCHED_OFF) = 0ull;
  const float sc = ldexpf(1.0f, 14 - ex);

  // roots (KPS = 4: W = W_hi + W_lo), once per group
  if (KPS == 4 && sb == 0 && tid < q) {
    const float2 wq = sW[tid];
    const __half hr = __float2half_rn(wq.x), hi = __float2half_rn(wq.y);
    reinterpret_cast<uint2*>(rc)[tid] =
        make_uint2(h2_bits(hr, hi), h2_bits(__float2half_rn(wq.x - __half2float(hr)),
                                            __float2half_rn(wq.y - __half2float(hi))));
  }
  // j table
  uint32_t* jtab = reinterpret_cast<uint32_t*>(rc + TAB_HDR);
  for (int e = tid; e < (s_hi - s_lo) * NW; e += blockDim.x) {
    const int sl = e / NW, wi = e % NW;
    uint32_t word = 0;
    if (sl < s_live) {
      for (int k = 0; k < 4; ++k) {
        const int t = wi * 4 + k;
        if (t >= b) break;
        int acc = 0;
        for (int i = 0; i < n; ++i) acc += (int)M[i * b + t] * (int)sK[sl * np4 + i];
        uint32_t v = (uint32_t)(acc % q);
        if (KPS == 2 && q == 2) v *= 2;
        word |= v << (8 * k);
      }
    }
    jtab[(int64_t)(s_lo + sl) * NW + wi] = word;
  }

  // B entries: (support vector, delay row) items write the row's four columns
  auto dst = [&](int s, int h, int nn) {
    const int k0 = KPS * s;
    const int kc = k0 / KC, kin = k0 % KC;
    return rc + g.tab_bytes + ((int64_t)h * g.nK + kc) * g.CB + sw128(nn, kin);
  };
  auto put = [&](unsigned char* p, uint32_t v) {
    if (KPS == 2)
      *reinterpret_cast<uint32_t*>(p) = v;
    else
      *reinterpret_cast<uint2*>(p) = make_uint2(v, v);
  };
  // items (delay row, support vector), support vector fastest: a warp writes
  // 32 consecutive words of each B row (one 128-byte swizzled row), not one
  // word of 32 rows
  const int ns = s_hi - s_lo;
  for (int e = tid; e < ns * RP; e += blockDim.x) {
    const int rp = e / ns, sl = e - rp * ns, s = s_lo + sl;
    const int h = rp / g.RPC, nb = 4 * (rp - h * g.RPC);
    uint32_t rh = 0, rl = 0, ih = 0, il = 0;
    if (sl < s_live) {
      const int* dw = reinterpret_cast<const int*>(sD + rp * np4);
      const int* kw = reinterpret_cast<const int*>(sK + sl * np4);
      int acc = 0;
      for (int w = 0; w < nw4; ++w) acc = __dp4a(dw[w], kw[w], acc);
      const float2 wr = sW[acc % q];
      const float2 a = A[s];
      const float cr = (a.x * wr.x - a.y * wr.y) * sc;
      const float ci = (a.x * wr.y + a.y * wr.x) * sc;
      const __half hr = __float2half_rn(cr), hi = __float2half_rn(ci);
      const __half lr = __float2half_rn(cr - __half2float(hr)), li = __float2half_rn(ci - __half2float(hi));
      rh = h2_bits(hr, __hneg(hi));  // real-part columns: [Chr, -Chi], [Clr, -Cli]
      rl = h2_bits(lr, __hneg(li));
      ih = h2_bits(hi, hr);          // imaginary-part columns: [Chi, Chr], [Cli, Clr]
      il = h2_bits(li, lr);
    }
    put(dst(s, h, nb + 0), rh);
    put(dst(s, h, nb + 1), rl);
    put(dst(s, h, nb + 2), ih);
    put(dst(s, h, nb + 3), il);
  }
  // padding columns of every chunk (the last chunk may hold fewer delay rows)
  for (int h = 0; h < g.nch; ++h) {
    const int rows = min(g.RPC, RP - h * g.RPC), npad = g.NP - 4 * rows;
    for (int e = tid; e < ns * npad; e += blockDim.x)
      put(dst(s_lo + e % ns, h, 4 * rows + e / ns), 0u);
  }
}

// ---------------------------------------------------------------- GEMM
// Persistent: one CTA per SM takes work units (job, group, chunk of delay
// rows, block of MT*128 rows) from a global counter until none is left, so
// units of unequal cost balance by themselves.  Its load warp takes them and
// publishes them in a small shared-memory queue; every role reads the same
// sequence from it:
//   producer set 0 (MT*4 warps)  K entries 0..31 of each A chunk into a TMEM ring
//   producer set 1 (MT*4 warps)  K entries 32..63; then accumulators -> U, one
//                                32-row quarter of one tile each
//   MMA warps (one per tile)     tcgen05.mma into accumulator buffer (unit % nacc)
//   load warp                    units, tables and B chunks (bulk copies)
// The A and B rings run on across unit boundaries, so set 0 and the load warp
// stage the next unit's operands while set 1 drains the last one.
// B stages.  Four: the bulk copies are off the critical path (skipping them
// changed nothing), and the smaller shared-memory footprint (110 KB instead of
// 200 KB per CTA) measured 4% faster per step with four batches in flight
// (1% slower for one batch alone)
constexpr int MAX_NB = 4;
constexpr int MAX_NA = 4;   // A stages
constexpr int TMEM_COLS = 512;
constexpr int UQ = 8;       // queue of work units shared by the roles

// A stages that fit beside nacc accumulator buffers of MT tiles x npmax columns
__host__ __device__ inline int tmem_na(int mt, int nacc, int npmax) {
  const int acc = (nacc * mt * npmax + 31) / 32 * 32;
  const int na = (TMEM_COLS - acc) / (mt * A_COLS);
  return na > MAX_NA ? MAX_NA : na;
}

// A work unit as the load warp decodes it into the shared-memory queue (j < 0
// ends the queue).  seq counts the CTA's units; its table goes to buffer seq % 2.
struct Unit {
  int j, c, h, q, b, S_pad, nK, NP, RP, rp0, nrp, seq;
  int64_t B, row0;
  const unsigned char* region;  // the job's region (header: inverse scale)
  const unsigned char* gT;      // the group's table (roots, j words)
  const unsigned char* gB;      // the chunk's B images
  uint32_t CB, TB;              // bytes of a B chunk, of the table copy
  float2* U;                    // samples of (job, group, first delay row of the chunk)
};
static_assert(sizeof(Unit) <= UNIT_BYTES, "unit queue entry");

template <int KPS, int NW>
__device__ __forceinline__ Unit decode_unit(const qsft_plan& plan, int64_t w, int nrows) {
  Unit x;
  x.seq = 0;
  const int nj = plan.njobs;
  const int64_t* __restrict__ idx = plan.gm_index;
  x.j = find_job(idx, nj, w);
  const qsft_job* __restrict__ job = plan.jobs + x.j;
  x.q = job->q;
  x.b = job->b;
  x.B = job->B;
  x.RP = job->R * job->P;
  const Geo g = geo(x.RP, job->S, KPS, NW);
  const int64_t rblocks = (x.B + nrows - 1) / nrows;
  const int64_t local = w - __ldg(idx + x.j);
  const int ch = (int)(local / rblocks);
  x.c = ch / g.nch;
  x.h = ch - x.c * g.nch;
  x.row0 = (local - (int64_t)ch * rblocks) * nrows;
  x.rp0 = x.h * g.RPC;
  x.nrp = min(g.RPC, x.RP - x.rp0);
  x.nK = g.nK;
  x.NP = g.NP;
  x.S_pad = g.S_pad;
  x.CB = g.CB;
  x.TB = g.tab_copy;
  x.region = reinterpret_cast<const unsigned char*>(plan.gm_ws) + __ldg(idx + 2 * (nj + 1) + x.j);
  const unsigned char* gc = x.region + REGION_HDR + (int64_t)x.c * g.region_c;
  x.gT = gc;
  x.gB = gc + g.tab_bytes + (int64_t)x.h * g.nK * g.CB;
  x.U = reinterpret_cast<float2*>(plan.U) + job->off_U + ((int64_t)x.c * x.RP + x.rp0) * x.B;
  return x;
}


// a ring position (slot, phase parity), advanced without division
struct Ring {
  uint32_t slot, phase, n;
  __device__ __forceinline__ explicit Ring(uint32_t size) : slot(0), phase(0), n(size) {}
  __device__ __forceinline__ void next() {
    if (++slot == n) {
      slot = 0;
      phase ^= 1;
    }
  }
};

template <int KPS, int NW>
__global__ void __launch_bounds__(2 * 2 * TM + 96, 1) eval_gemm_kernel(qsft_plan plan, int nb) {
  extern __shared__ __align__(1024) unsigned char smem[];
  // chunk g (counted over the CTA's whole unit range) uses A slot g % NA and B slot g % nb
  uint64_t* bfull = reinterpret_cast<uint64_t*>(smem);  // [MAX_NB] B chunk landed
  uint64_t* cons = bfull + MAX_NB;                      // [MAX_NB] every MMA of chunk g (at g % nb) completed
  uint64_t* afull = cons + MAX_NB;                      // [MAX_NA] A chunk written (by both producer sets)
  uint64_t* accf = afull + MAX_NA;                      // [2] accumulator buffer written
  uint64_t* acce = accf + 2;                            // [2] accumulator buffer drained
  uint64_t* done = acce + 2;                            // every MMA issued has completed
  uint64_t* uq_full = done + 1;                         // [UQ] unit published
  uint64_t* uq_empty = uq_full + UQ;                    // [UQ] every consumer warp has read it
  uint64_t* tfull = uq_empty + UQ;                      // [2] table buffer landed
  uint64_t* tempty = tfull + 2;                         // [2] every producer warp is done with the table
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 960);  // after the barriers
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + 964);
  volatile uint32_t* n_con = reinterpret_cast<volatile uint32_t*>(smem + 968);
  Unit* units = reinterpret_cast<Unit*>(smem + UNIT_OFF);  // [UQ] decoded units
  unsigned char* tbuf = smem + HDR;                        // [2] table buffers of plan.gm_jt_bytes
  const int MT = plan.gm_mt, nacc = plan.gm_nacc, npmax = plan.gm_npmax;
  const uint32_t TBB = (uint32_t)plan.gm_jt_bytes;
  // A slots: what tensor memory holds beside the accumulators, and fewer than the
  // B slots, so that a wait on cons[] for chunk g - NA cannot alias a later phase
  const int NA = min(tmem_na(MT, nacc, npmax), nb - 1);
  const uint32_t B_SLOT = (uint32_t)npmax * KC * 2;
  unsigned char* bring = tbuf + 2 * TBB;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nprod = MT * TM;
  // warps 0 and 2 issue the MMAs of tiles 0 and 1 (one thread each: issuing
  // an MMA takes a thread ~50 cycles, so one thread for both tiles left the
  // tensor pipe waiting), warp 1 loads, warps 3.. are the two producer sets
  const int mma_warp = 0, load_warp = 1, mma_warp2 = 2, prod_warp0 = 3;
  const int n_mma = MT;  // MMA threads

  // ---- setup: accumulators at column buf*MT*npmax + t*npmax, then NA slots of MT A tiles
  const uint32_t acols = (uint32_t)(nacc * MT * npmax + 31) / 32 * 32;
  const uint32_t ncols = TMEM_COLS;
  if (warp == mma_warp) {
    tmem_alloc(tmem_slot, ncols);
    tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < MAX_NB; ++i) {
      mbar_init(&bfull[i], 1);
      mbar_init(&cons[i], n_mma);
    }
    for (int i = 0; i < MAX_NA; ++i) mbar_init(&afull[i], 2 * MT * 4);  // both producer sets
    for (int i = 0; i < 2; ++i) {
      mbar_init(&accf[i], n_mma);
      mbar_init(&acce[i], MT * 4);
      mbar_init(&tfull[i], 1);
      mbar_init(&tempty[i], 2 * MT * 4);
    }
    mbar_init(done, n_mma);
    for (int i = 0; i < UQ; ++i) {
      mbar_init(&uq_full[i], 1);
      mbar_init(&uq_empty[i], 2 * MT * 4 + n_mma);  // both producer sets, the MMA threads
    }
    // the swizzled layout needs 1024-byte aligned atoms; the TMEM plan must fit
    *abort_flag = ((smem_u32(bring) & 1023u) || (TBB & 1023u) || NA < 2 || nb > MAX_NB || (MT != 1 && MT != 2) ||
                   (nacc != 1 && nacc != 2)) ? 1 : 0;
    *n_con = 0;
    fence_mbar_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  uint32_t iss = 0, tl = 0;  // bulk copies of B chunks and of tables issued (load warp, lane 0)
  // the next unit of a consumer warp, read by every lane from the queue (whose
  // slot is freed at once); false when the queue has ended or a wait gave up
  auto take_unit = [&](Ring& r, Unit& x) -> bool {
    const int ok = __all_sync(~0u, mbar_wait(&uq_full[r.slot], r.phase) ? 1 : 0);
    if (ok) x = units[r.slot];
    __syncwarp();
    if (lane == 0) {
      if (!ok) *abort_flag = 1;
      mbar_arrive(&uq_empty[r.slot]);
    }
    r.next();
    return ok && x.j >= 0;
  };

  if (warp >= prod_warp0) {
    // ---- producers, in two sets of MT*4 warps over the same rows: set 0
    // writes K entries 0..31 of every chunk, set 1 entries 32..63, one row
    // per thread; set 1 also reads each unit's accumulators back (the
    // epilogue) once its MMAs have completed, and stores U
    const int pw = warp - prod_warp0, set = pw / (MT * 4), wi = pw - set * MT * 4;
    const int t = wi >> 2, lq = warp & 3;  // tile, lane quarter (warp % 4: the TMEM lanes this warp may access)
    const int rr = t * TM + lq * 32 + lane;  // row within the unit
    const uint32_t a_lane =
        tmem + ((uint32_t)(lq * 32) << 16) + acols + (uint32_t)t * A_COLS + (uint32_t)set * (A_COLS / 2);
    Ring fa((uint32_t)NA);   // A slot of chunk g
    Ring ce((uint32_t)nb);   // cons[] position of chunk g - NA
    Ring ac((uint32_t)nacc), uqr(UQ);
    uint32_t g = 0;
    Unit x;
    while (take_unit(uqr, x)) {
      if (*abort_flag) continue;  // keep taking units until the queue ends
      // the unit's table (every lane waits, so that the copied words are visible to it)
      const uint32_t tk = (uint32_t)x.seq & 1u;
      if (!__all_sync(~0u, mbar_wait(&tfull[tk], ((uint32_t)x.seq >> 1) & 1u) ? 1 : 0)) {
        if (lane == 0) *abort_flag = 1;
        continue;
      }
      const unsigned char* tab = tbuf + tk * TBB;
      const uint2* qtab = reinterpret_cast<const uint2*>(tab);  // KPS = 4: (hi, lo) half2 words of omega^m
      const uint32_t* jt = reinterpret_cast<const uint32_t*>(tab + TAB_HDR);
      const int64_t l = x.row0 + rr;
      uint32_t lw[NW];
#pragma unroll
      for (int k = 0; k < NW; ++k) lw[k] = 0;
      if (l < x.B) {
        uint32_t v = (uint32_t)l;
#pragma unroll
        for (int d = 4 * NW - 1; d >= 0; --d) {  // MSB-first digits: digit b-1 is l mod q
          if (d < x.b) {
            const uint32_t qt = v / (uint32_t)x.q;
            lw[d >> 2] |= (v - qt * (uint32_t)x.q) << (8 * (d & 3));
            v = qt;
          }
        }
      }
      const ModQ mq = make_modq(x.q);
      bool ok = true;
      // each half chunk is computed before its slot is free (the wait overlaps the work)
      for (int kc = 0; kc < x.nK; ++kc) {
        const int s0 = kc * (KC / KPS) + set * (KC / 2 / KPS);
        uint32_t av[16];  // the row's 32 FP16 entries of this half chunk, K order
        if constexpr (KPS == 2) {
          // four support vectors per 16-byte chunk; omega_4^m as half2 (re, im):
          // high bytes from the tables 0x00BC003C (re) and 0xBC003C00 (im), low bytes zero
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const uint32_t* jp = jt + (s0 + 4 * i) * NW;
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              uint32_t d = 0;
#pragma unroll
              for (int k = 0; k < NW; ++k) d = __dp4a(lw[k], jp[e * NW + k], d);
              av[4 * i + e] = __byte_perm(0x00BC003Cu, 0xBC003C00u, 0x4101u + (d & 3u) * 0x1010u);
            }
          }
        } else {
          // two support vectors per 16-byte chunk: (hi, lo) half2 words of omega^m
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const uint32_t* jp = jt + (s0 + 2 * i) * NW;
            uint32_t d0 = 0, d1 = 0;
#pragma unroll
            for (int k = 0; k < NW; ++k) {
              d0 = __dp4a(lw[k], jp[k], d0);
              d1 = __dp4a(lw[k], jp[NW + k], d1);
            }
            const uint2 h0 = qtab[modq(d0, mq)], h1 = qtab[modq(d1, mq)];
            av[4 * i] = h0.x;
            av[4 * i + 1] = h0.y;
            av[4 * i + 2] = h1.x;
            av[4 * i + 3] = h1.y;
          }
        }
        if (g >= (uint32_t)NA) {  // slot reuse: the MMAs of chunk g - NA have completed
          int go = 1;
          if (lane == 0) go = !*abort_flag && mbar_wait(&cons[ce.slot], ce.phase);
          go = __shfl_sync(~0u, go, 0);
          if (!go) {
            if (lane == 0) *abort_flag = 1;
            ok = false;
            break;
          }
          ce.next();
        }
        // store and signal at once: the MMA threads wait for this chunk, not for the next one's compute
        tmem_st16(a_lane + fa.slot * (uint32_t)(MT * A_COLS), av);
        tmem_st_wait();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&afull[fa.slot]);
        fa.next();
        ++g;
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[tk]);  // this warp is done with the table
      if (set == 0 || !ok) continue;

      // ---- epilogue (set 1): tile t, rows lq*32 + lane of it
      const bool live = l < x.B;
      float2* __restrict__ ur = x.U + l;
      const float inv = *reinterpret_cast<const float*>(x.region);
      int ready = 1;
      // one accumulator buffer: the MMA threads wait for this drain, so notice the
      // unit's end soon (128 ns cap); two: the drain overlaps MMAs, sleep longer
      if (lane == 0) ready = !*abort_flag && mbar_wait_sleep(&accf[ac.slot], ac.phase, nacc == 1 ? 128u : 2048u);
      ready = __shfl_sync(~0u, ready, 0);
      if (!ready) {
        if (lane == 0) *abort_flag = 1;
        continue;
      }
      tc_fence_after();
      const uint32_t tb = tmem + ((uint32_t)(lq * 32) << 16) + ac.slot * (uint32_t)(MT * npmax) + (uint32_t)(t * npmax);
      const int ng = x.NP / 16;
      const int nrp = x.nrp;
      const int64_t B = x.B;
      // 16 columns = 4 delay rows x (re hi, re lo, im hi, im lo)
      auto emit = [&](const uint32_t(&r)[16], int cg) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int rp = cg * 4 + k;
          if (live && rp < nrp)
            ur[(int64_t)rp * B] =
                make_float2((__uint_as_float(r[4 * k]) + __uint_as_float(r[4 * k + 1])) * inv,
                            (__uint_as_float(r[4 * k + 2]) + __uint_as_float(r[4 * k + 3])) * inv);
        }
      };
      // rounds of three 16-column loads and one wait (a wait covers every load in flight)
      for (int cg0 = 0; cg0 < ng; cg0 += 3) {
        uint32_t r0[16], r1[16], r2[16];
        tmem_ld16(tb + cg0 * 16, r0);
        if (cg0 + 1 < ng) tmem_ld16(tb + (cg0 + 1) * 16, r1);
        if (cg0 + 2 < ng) tmem_ld16(tb + (cg0 + 2) * 16, r2);
        tmem_ld_wait_regs(r0);
        tmem_ld_wait_regs(r1);
        tmem_ld_wait_regs(r2);
        emit(r0, cg0);
        if (cg0 + 1 < ng) emit(r1, cg0 + 1);
        if (cg0 + 2 < ng) emit(r2, cg0 + 2);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[ac.slot]);
      ac.next();
    }
  } else if (warp == mma_warp || (warp == mma_warp2 && MT == 2)) {
    // ---- MMA issue.  Descriptors differ between slots, tiles and K steps
    // only in the start-address field (smem address >> 4 < 2^14, no carry),
    // so they are built once and advanced by additions.  The loop is kept
    // short: a thread needs ~50 cycles to issue one MMA, so every cycle it
    // spends elsewhere can leave the tensor pipe without queued work.
    if (lane == 0) {
      const uint32_t tile = warp == mma_warp ? 0u : 1u;  // this thread's tile
      const uint64_t b_first = desc_sw128(smem_u32(bring));
      const uint32_t a_first = tmem + acols + tile * A_COLS;
      const uint32_t a_step = (uint32_t)(MT * A_COLS), b_step = B_SLOT >> 4;
      Ring fa((uint32_t)NA), fb((uint32_t)nb), ac((uint32_t)nacc), uqr(UQ);
      uint32_t a_addr = a_first;  // A slot of chunk g
      uint64_t b_desc = b_first;  // B slot of chunk g
      uint32_t g = 0;
      // the four K = 16 steps of one tile (K = 16 is 32 bytes along the swizzled row)
      auto tile_mmas = [&](uint32_t d, uint32_t a, uint64_t b, uint32_t idesc, uint32_t acc0) {
        mma_f16_ts(d, a, b, idesc, acc0);
        mma_f16_ts(d, a + 8, b + 2, idesc, 1u);
        mma_f16_ts(d, a + 16, b + 4, idesc, 1u);
        mma_f16_ts(d, a + 24, b + 6, idesc, 1u);
      };
      for (;;) {
        // lane 0 alone runs this loop: the queue without the warp-wide take
        int nK = 0, NP = 16, live = 0;
        if (mbar_wait(&uq_full[uqr.slot], uqr.phase)) {
          const Unit& s = units[uqr.slot];
          live = s.j >= 0;
          nK = s.nK;
          NP = s.NP;
        } else {
          *abort_flag = 1;
        }
        mbar_arrive(&uq_empty[uqr.slot]);
        uqr.next();
        if (!live || *abort_flag) break;
        if (!mbar_wait(&acce[ac.slot], ac.phase ^ 1)) {
          *abort_flag = 1;
          break;
        }
        tc_fence_after();
        const uint32_t idesc = tc::make_idesc(TM, NP);
        const uint32_t d = tmem + ac.slot * (uint32_t)(MT * npmax) + tile * (uint32_t)npmax;
        bool ok = true;
        for (int kc = 0; kc < nK; ++kc) {
          // both operands of chunk g: one non-blocking test each, issued together;
          // the bounded blocking waits only when either is not there yet
          const bool rb = mbar_test_wait(&bfull[fb.slot], fb.phase);
          const bool ra = mbar_test_wait(&afull[fa.slot], fa.phase);
          if (!(rb && ra) && (*abort_flag || !mbar_wait(&bfull[fb.slot], fb.phase) ||
                               !mbar_wait(&afull[fa.slot], fa.phase))) {
            ok = false;
            break;
          }
          tc_fence_after();
          tile_mmas(d, a_addr, b_desc, idesc, kc > 0 ? 1u : 0u);
          mma_commit(&cons[fb.slot]);  // with the other tile's: frees A slot and B slot of chunk g
          if (++fa.slot == fa.n) {
            fa.slot = 0;
            fa.phase ^= 1;
            a_addr = a_first;
          } else {
            a_addr += a_step;
          }
          if (++fb.slot == fb.n) {
            fb.slot = 0;
            fb.phase ^= 1;
            b_desc = b_first;
          } else {
            b_desc += b_step;
          }
          ++g;
        }
        if (!ok) {
          *abort_flag = 1;
          break;
        }
        mma_commit(&accf[ac.slot]);  // with the other tile's: every MMA of the unit has completed
        ac.next();
      }
      atomicMax(const_cast<uint32_t*>(n_con), g);  // chunks whose B copy an MMA thread saw land
      mma_commit(done);  // arrives once every MMA issued above has completed
      if (!mbar_wait(done, 0)) *abort_flag = 1;
    }
    __syncwarp();
  } else if (warp == load_warp) {
    // ---- scheduler and copies: takes units from the global counter (reset by
    // the operand kernel), decodes each into the queue, then copies its table
    // and streams its B chunks, one bulk copy per slot, up to nb in flight
    if (lane == 0) {
      unsigned long long* counter =
          reinterpret_cast<unsigned long long*>(reinterpret_cast<unsigned char*>(plan.gm_ws) + SCHED_OFF);
      const long long total = plan.total_gm_work;
      Ring fb((uint32_t)nb), uqw(UQ);
      bool ended = false;
      int seq = 0;
      // one unit per take: units of unequal cost balance by themselves and the
      // tail is a single unit (runs of consecutive units measured slower)
      auto publish = [&](bool stop) -> int {  // queue slot of the unit published, -1 at the end
        if (ended) return -1;
        if (!mbar_wait(&uq_empty[uqw.slot], uqw.phase ^ 1)) {
          *abort_flag = 1;
          ended = true;
          return -1;
        }
        long long u = -1;
        if (!stop) {
          u = (long long)atomicAdd(counter, 1ull);
          if (u >= total) u = -1;
        }
        Unit* s = units + uqw.slot;
        if (u >= 0) {
          *s = decode_unit<KPS, NW>(plan, u, nprod);
          s->seq = seq++;
        } else {
          s->j = -1;
          ended = true;
        }
        mbar_arrive(&uq_full[uqw.slot]);  // release: the unit is visible with the phase
        const int slot = (int)uqw.slot;
        uqw.next();
        return u >= 0 ? slot : -1;
      };
      uint32_t g = 0;
      int cur = publish(false);
      while (cur >= 0) {
        const Unit x = units[cur];  // its slot is rewritten only UQ publications later
        // the table into buffer seq % 2 once the producers are done with the
        // unit two before (they are in the previous unit by now)
        const uint32_t tk = (uint32_t)x.seq & 1u;
        if (*abort_flag || (x.seq >= 2 && !mbar_wait(&tempty[tk], (((uint32_t)x.seq >> 1) - 1u) & 1u))) {
          *abort_flag = 1;
          break;
        }
        mbar_arrive_expect_tx(&tfull[tk], x.TB);
        bulk_g2s(tbuf + tk * TBB, x.gT, x.TB, &tfull[tk]);
        tl = (uint32_t)x.seq + 1;
        const int nxt = publish(false);  // decoded while this unit's copies wait for slots
        for (int kc = 0; kc < x.nK; ++kc) {
          // slot reuse: the MMAs of chunk g - nb have completed (the first round passes)
          if (*abort_flag || !mbar_wait(&cons[fb.slot], fb.phase ^ 1)) {
            *abort_flag = 1;
            break;
          }
          mbar_arrive_expect_tx(&bfull[fb.slot], x.CB);
          bulk_g2s(bring + fb.slot * B_SLOT, x.gB + (int64_t)kc * x.CB, x.CB, &bfull[fb.slot]);
          fb.next();
          iss = ++g;
        }
        if (*abort_flag) break;
        cur = nxt;
      }
      publish(true);  // ends the queue for every consumer (after an abort too)
    }
    __syncwarp();
  }
  __syncthreads();  // every role loop has ended; n_con is final
  if (warp == load_warp && lane == 0) {
    for (uint32_t k = *n_con; k < iss; ++k)  // copies that no MMA consumed: let them land (bounded)
      mbar_wait(&bfull[k % (uint32_t)nb], (k / (uint32_t)nb) & 1);
    // the last table copy of each buffer (an earlier one was consumed before the buffer was reused)
    for (uint32_t k = tl > 2 ? tl - 2 : 0; k < tl; ++k) mbar_wait(&tfull[k & 1u], (k >> 1) & 1u);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (tid == 0 && *abort_flag) atomicExch(plan.status, (int)QSFT_ERR_TIMEOUT);
  if (warp == mma_warp) tmem_dealloc(tmem, ncols);
}

// B slots for the shared-memory budget (A lives in tensor memory; two table buffers)
inline bool pick_stages(int npmax, int jt_bytes, int& nb, int& smem) {
  const int fixed = HDR + 2 * jt_bytes, bb = npmax * KC * 2;
  for (nb = MAX_NB; nb >= 3; --nb)  // at least 3: the A ring keeps 2 slots below it
    if (fixed + nb * bb <= MAX_SMEM) {
      smem = fixed + nb * bb;
      return true;
    }
  return false;
}

template <int KPS, int NW>
static int launch(const qsft_plan* p, cudaStream_t st) {
  int nb, smem;
  if (!pick_stages(p->gm_npmax, p->gm_jt_bytes, nb, smem)) return QSFT_ERR_TOO_LARGE;
  if (p->total_gm_prep > 0) {
    gemm_prep_kernel<KPS, NW><<<(unsigned)p->total_gm_prep, 256, 0, st>>>(*p);
    QSFT_CUDA_CHECK_LAUNCH();
  }
  auto kern = eval_gemm_kernel<KPS, NW>;
  if (!ensure_smem((const void*)kern, smem)) return QSFT_ERR_CUDA;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return QSFT_ERR_CUDA;
  const int64_t grid = p->total_gm_work < sms ? p->total_gm_work : sms;  // persistent: one CTA per SM
  kern<<<(unsigned)grid, 2 * p->gm_mt * TM + 96, smem, st>>>(*p, nb);
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
}

template <int KPS>
static int launch_nw(const qsft_plan* p, cudaStream_t st) {
  switch (p->gm_nw) {
    case 1: return launch<KPS, 1>(p, st);
    case 2: return launch<KPS, 2>(p, st);
    case 4: return launch<KPS, 4>(p, st);
    default: return QSFT_ERR_ARG;
  }
}

}  // namespace gm
}  // namespace qsft

using namespace qsft;

extern "C" int qsft_gemm_layout(const qsft_job* jobs, int njobs, qsft_plan* plan, int64_t* index) {
  if (!jobs || njobs <= 0 || !plan || !index) return QSFT_ERR_ARG;
  int kps = 2, maxb = 0, jt = 0;
  int64_t maxB = 1;
  for (int i = 0; i < njobs; ++i) {
    const qsft_job& jb = jobs[i];
    if (jb.q < 2 || jb.n < 1 || jb.b < 1 || jb.C < 1 || jb.R < 1 || jb.P < 1 || jb.S < 1) return QSFT_ERR_ARG;
    if (jb.q > QSFT_MAX_Q || jb.b > 16 || jb.R * jb.P > gm::PREP_MAXRP || jb.S > 8192 || jb.n > QSFT_MAX_N)
      return QSFT_ERR_TOO_LARGE;
    if (jb.q != 2 && jb.q != 4) kps = 4;
    maxb = maxb > jb.b ? maxb : jb.b;
    maxB = maxB > jb.B ? maxB : jb.B;
  }
  const int nw = maxb <= 4 ? 1 : (maxb <= 8 ? 2 : 4);
  int npmax = 16;
  for (int i = 0; i < njobs; ++i) {
    const gm::Geo g = gm::geo(jobs[i].R * jobs[i].P, jobs[i].S, kps, nw);
    npmax = npmax > g.NP ? npmax : g.NP;
  }
  // tensor memory: nacc accumulator buffers of mt tiles + at least two A slots.
  // Preference: the larger mt (a B chunk feeds more rows, and the per-chunk
  // waits and commits cover twice the MMAs), then at least three A
  // slots, then two buffers (the epilogue overlaps the next unit's MMAs).
  // Presets cap mt and nacc.
  const int mt_cap = (plan->gm_mt == 1 || plan->gm_mt == 2) ? plan->gm_mt : 2;
  const int nacc_cap = plan->gm_nacc == 1 ? 1 : 2;
  int mt = 0, nacc = 0;
  for (int m = mt_cap; m >= 1 && !mt; --m)
    for (int min_na = 3; min_na >= 2 && !mt; --min_na)
      for (int na_ = nacc_cap; na_ >= 1 && !mt; --na_)
        if ((m == 1 || (int64_t)(m / 2) * gm::TM < maxB) && gm::tmem_na(m, na_, npmax) >= min_na) {
          mt = m;
          nacc = na_;
        }
  if (!mt) return QSFT_ERR_TOO_LARGE;
  int64_t work = 0, prep = 0, off = 0;
  index[0] = 0;
  index[njobs + 1] = 0;
  for (int i = 0; i < njobs; ++i) {
    const qsft_job& jb = jobs[i];
    const gm::Geo g = gm::geo(jb.R * jb.P, jb.S, kps, nw);
    const int64_t rows = (int64_t)mt * gm::TM;
    work += (int64_t)jb.C * g.nch * ((jb.B + rows - 1) / rows);
    prep += (int64_t)jb.C * ((g.S_pad + gm::PREP_S - 1) / gm::PREP_S);
    index[i + 1] = work;
    index[njobs + 2 + i] = prep;
    index[2 * (njobs + 1) + i] = off;
    off += gm::region_bytes(g, jb.C);
    const int jtb = gm::tab_smem(g);
    jt = jt > jtb ? jt : jtb;
  }
  int nb, smem;
  if (!gm::pick_stages(npmax, jt, nb, smem)) return QSFT_ERR_TOO_LARGE;
  if (work > 0x7fffffffLL || prep > 0x7fffffffLL) return QSFT_ERR_TOO_LARGE;
  plan->gm_mt = mt;
  plan->gm_nacc = nacc;
  plan->gm_kps = kps;
  plan->gm_nw = nw;
  plan->gm_npmax = npmax;
  plan->gm_jt_bytes = jt;
  plan->total_gm_work = work;
  plan->total_gm_prep = prep;
  plan->gm_ws_bytes = off;
  return QSFT_OK;
}

extern "C" int qsft_eval_cosets_gemm(const qsft_plan* plan, qsft_stream_t stream) {
  if (!plan || plan->njobs <= 0 || !plan->jobs || !plan->gm_index || !plan->gm_ws || !plan->i8 || !plan->A ||
      !plan->U || !plan->status)
    return QSFT_ERR_ARG;
  if (plan->prec != QSFT_F32) return QSFT_ERR_ARG;
  if ((plan->gm_mt != 1 && plan->gm_mt != 2) || (plan->gm_nacc != 1 && plan->gm_nacc != 2)) return QSFT_ERR_ARG;
  if (plan->gm_npmax < 16 || plan->gm_npmax > 4 * gm::RPC_MAX || plan->gm_npmax % 16 ||
      gm::tmem_na(plan->gm_mt, plan->gm_nacc, plan->gm_npmax) < 2)
    return QSFT_ERR_ARG;
  if (plan->total_gm_work <= 0) return QSFT_OK;
  cudaStream_t st = (cudaStream_t)stream;
  if (plan->gm_kps == 2) {
    if (plan->max_q > 4) return QSFT_ERR_ARG;
    return gm::launch_nw<2>(plan, st);
  }
  if (plan->gm_kps == 4) return gm::launch_nw<4>(plan, st);
  return QSFT_ERR_ARG;
}
