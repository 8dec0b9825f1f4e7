// Singleton detection and peeling: QSFT.transform's while-loop
// (qsft/qsft.py:151-255) for a batch of transforms.
//
// One iteration = three launches:
//   scan     a warp takes 32 bins at a time, a lane per bin (the first
//            iteration: every bin, consecutive bins of a group -- coalesced;
//            later ones: the bins the previous subtractions changed, the
//            others keeping their class, a function of their unchanged
//            values): the zeroton test ||col||^2 > cutoff*len
//            (qsft/qsft.py:164).  Bins above it are queued and their columns
//            copied, while still in L2, into a compact staging buffer.
//   decode   a group of 8 lanes per queued bin: channel decoding of k
//            (noiseless qsft/reconstruct.py:12-31 or NSO "nso1" :100-113),
//            optional Reed-Solomon source decoding (:34-51), projection
//            rho = <omega^(Dk), col>/len and residual energy, bin-match test
//            (qsft/qsft.py:174-190).  Each singleton is recorded at once: it
//            finds (or creates) the ball of its k in a persistent hash table,
//            adds rho to the ball's running sum (the `result` list and its
//            mean, :217, 247-255) and marks the ball detected in this
//            iteration keeping the largest (group, bin) -- the reference's
//            dict order, `ball_values` (:209-216).
//   peel     per (detected ball, group l) -- a thread, or 8 for short lists:
//            subtract rho * omega^(D_l k) from bin M_l^T k (mod q) of group l
//            (qsft/qsft.py:223-241) and queue the changed bin for the next
//            scan.  The block that finishes last closes the iteration for
//            every job: iteration count, cumulative peel count and the loop's
//            stopping rules (qsft/qsft.py:151, 204-205).
//
// FP32 data path: bins are stored as float2.  Energy, phase and residual
// decisions that fall within a small band of their thresholds are recomputed
// in FP64 (GB300's FP64 rate is a small fraction of its FP32 rate).
#include "common.cuh"
#include "rs.cuh"

namespace qsft {

constexpr int PEEL_THREADS = 256;
constexpr int MAX_SYMS = 256;  // channel symbols per bin (P - 1 <= 256)
constexpr int LIST_BLOCKS = 152 * 3;   // the peel kernel's grid: resident at once (3 blocks of 256 threads per SM)

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ uint32_t hash_row(const uint8_t* row, int words) {
  uint64_t h = 0xcbf29ce484222325ull;
  const uint32_t* w = reinterpret_cast<const uint32_t*>(row);
  for (int i = 0; i < words; ++i) {
    h ^= w[i];
    h *= 0x100000001b3ull;
  }
  h ^= h >> 29;
  h *= 0xbf58476d1ce4e5b9ull;
  h ^= h >> 32;
  return (uint32_t)h;
}
__device__ __forceinline__ double2 root(const double* roots, int q, int m) {
  return make_double2(__ldg(roots + (q * 32 + m) * 2), __ldg(roots + (q * 32 + m) * 2 + 1));
}
// index of the nearest value among 2 pi m / q, m = 0..q (first on ties), mod q
__device__ __forceinline__ int nearest_root(double ang, int q) {
  const double step = 6.283185307179586 / q;
  int best = 0;
  double bd = fabs(ang);
  for (int m = 1; m <= q; ++m) {
    const double dd = fabs(step * m - ang);
    if (dd < bd) {
      bd = dd;
      best = m;
    }
  }
  return best % q;
}
__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// ||col||^2 with the FP64 recomputation band of the FP32 path
template <typename T>
__device__ __forceinline__ double col_energy(const c2<T>* col, int RP, int B, double thr) {
  // the loads of 16 rows (8 in FP64) are issued before their sum (in row
  // order) is taken: a lane keeps that many independent loads in flight
  constexpr int BATCH = sizeof(T) == 4 ? 16 : 8;
  T e = 0;
  for (int r0 = 0; r0 < RP; r0 += BATCH) {
    c2<T> v[BATCH];
#pragma unroll
    for (int k = 0; k < BATCH; ++k)
      if (r0 + k < RP) v[k] = col[(int64_t)(r0 + k) * B];
#pragma unroll
    for (int k = 0; k < BATCH; ++k)
      if (r0 + k < RP) e += v[k].x * v[k].x + v[k].y * v[k].y;
  }
  double E = (double)e;
  if (sizeof(T) == 4 && fabs(E - thr) <= 1e-3 * thr) {
    E = 0.0;
    for (int r = 0; r < RP; ++r) {
      const double2 v = to_d2(col[(int64_t)r * B]);
      E += v.x * v.x + v.y * v.y;
    }
  }
  return E;
}
// warp-aggregated append of `want` lanes to a per-job list (lanes may be of different jobs)
__device__ __forceinline__ int warp_append(bool want, int jid, int* counter) {
  const unsigned peers = __match_any_sync(0xffffffffu, jid);
  const unsigned mask = __ballot_sync(0xffffffffu, want) & peers;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  int base = 0;
  if (lane == leader && mask) base = atomicAdd(counter, __popc(mask));
  base = __shfl_sync(0xffffffffu, base, leader);
  return base + __popc(mask & ((1u << lane) - 1));
}

// ---------------------------------------------------------------- decode

// phase <d, k> mod q of delay row d (n digits) against k (kstride-padded bytes)
__device__ __forceinline__ int row_phase(const int8_t* dr, const uint8_t* kl, int n, bool words_ok, int q) {
  int ph = 0;
  if (words_ok) {
    const uint32_t* dw = reinterpret_cast<const uint32_t*>(dr);
    const uint32_t* kw = reinterpret_cast<const uint32_t*>(kl);
    for (int w = 0; w < (n >> 2); ++w) ph = (int)__dp4a((unsigned)__ldg(dw + w), (unsigned)kw[w], (unsigned)ph);
  } else {
    for (int i = 0; i < n; ++i) ph += (int)dr[i] * (int)kl[i];
  }
  return ph % q;
}

// k rows (kstride bytes, 16-byte multiples) compared with 16-byte loads through L2
__device__ __forceinline__ bool krow_eq(const uint8_t* mine, const uint8_t* other, int ks) {
  const uint4* a = reinterpret_cast<const uint4*>(mine);
  const uint4* b = reinterpret_cast<const uint4*>(other);
  bool eq = true;
  for (int i = 0; i < ks / 16; ++i) {
    const uint4 x = a[i], y = __ldcg(b + i);
    eq &= (x.x == y.x) & (x.y == y.y) & (x.z == y.z) & (x.w == y.w);
  }
  return eq;
}

// A candidate bin is decoded by a group of G threads (G consecutive lanes; a
// warp holds 32 / G bins; G = 8 in the first iteration, 16 later, when there
// are fewer candidates to overlap): symbols, rows and digits are dealt
// over the group and its sums reduced with in-group shuffles, so the dependent
// chain of one bin stays short.  A warp works on bins of one job (chunks dealt
// round-robin), so control flow is uniform.  The column's RP values (stride B
// in U) are staged in shared memory with one round of loads when
// RP <= DEC_STAGE_RP; FP32 roots for every q come from a block-wide table.
constexpr int DEC_THREADS = 128;
constexpr int DEC_G = 8;        // lanes per candidate in the first iteration (and the persistent loop)
constexpr int DEC_G_LATER = 16; // in later iterations: fewer candidates, more lanes on each
constexpr int DEC_STAGE_RP = 64;
constexpr int DEC_KB = 2 * QSFT_MAX_N;   // k row: n digits mod q, then n high parts for a coded source
constexpr int PEEL_THREAD_MIN = 1024;  // peel items of a job at least this many: one thread per item

template <int G, typename V>
__device__ __forceinline__ V group_sum(V v, unsigned mask) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
  return v;
}
// the same over groups of g (a power of two <= 32) lanes, g chosen at run time
template <typename V>
__device__ __forceinline__ V group_sum_g(V v, unsigned mask, int g) {
  for (int o = g >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
  return v;
}

// ---------------------------------------------------------------- record
// One singleton (k in the 16-byte aligned row kr, coefficient rho) of bin
// `local`: find (or create) the ball of its k in the job's persistent table
// (tags first, k rows only on a tag hit), add rho to the ball's running sum,
// and mark the ball detected in this iteration with (iteration << 32 | local)
// by atomicMax -- the largest local bin wins, the reference's last-write order
// over (group, bin) (qsft/qsft.py:209-216).  Returns the ball id (-1 when a
// table is full: ctrl.err) and whether this is the ball's first detection in
// the iteration (the old value's iteration field tells).
__device__ __forceinline__ int record_one(const qsft_plan& plan, const qsft_job* __restrict__ job, qsft_ctrl* ctl,
                                          const uint8_t* kr, int local, double2 rho, long long iter, int ks,
                                          bool& first) {
  first = false;
  const int64_t mask = job->table_cap - 1;
  unsigned long long* tab = reinterpret_cast<unsigned long long*>(plan.ball_tab + job->off_slot);
  const uint32_t h = hash_row(kr, ks / 4);
  const unsigned long long tag = (unsigned long long)(h | 1u) << 32;
  int64_t slot = h & mask;
  int myid = -1, bid = -1;
  for (int64_t probe = 0; probe < job->table_cap; ++probe) {
    unsigned long long cur = __ldcg(tab + slot);
    if (cur == 0) {
      if (myid < 0) {  // publish our k row before the slot that points at it
        myid = atomicAdd(&ctl->n_balls, 1);
        if (myid >= job->ball_cap) break;
        const uint4* src = reinterpret_cast<const uint4*>(kr);
        uint4* dst = reinterpret_cast<uint4*>(plan.ball_k + (job->off_ball + myid) * ks);
        for (int w = 0; w < ks / 16; ++w) dst[w] = src[w];
        __threadfence();
      }
      const unsigned long long prev = atomicCAS(tab + slot, 0ull, tag | (unsigned long long)(myid + 1));
      if (prev == 0) {
        bid = myid;
        break;
      }
      cur = prev;
    }
    if ((cur & 0xffffffff00000000ull) == tag) {
      const int other = (int)(cur & 0xffffffffull) - 1;
      if (krow_eq(kr, plan.ball_k + (job->off_ball + other) * ks, ks)) {
        bid = other;
        break;
      }
    }
    slot = (slot + 1) & mask;
  }
  if (bid < 0) {
    atomicExch(&ctl->err, (int)QSFT_ERR_OVERFLOW);
    return -1;
  }
  // a ball id allocated for a k that another thread inserted first stays an
  // empty row (count 0): the collection skips it
  const int64_t gball = job->off_ball + bid;
  atomicAdd(plan.ball_sum + 2 * gball, rho.x);
  atomicAdd(plan.ball_sum + 2 * gball + 1, rho.y);
  atomicAdd(plan.ball_cnt + gball, 1);
  const unsigned long long old = atomicMax(reinterpret_cast<unsigned long long*>(plan.ball_best) + gball,
                                           (unsigned long long)((iter << 32) | (unsigned)local));
  first = (long long)(old >> 32) != iter;
  return bid;
}

// ---------------------------------------------------------------- scan
// The staged copy of candidate `pos`'s column of job `jid`: job j owns staging
// columns [bin_prefix[j] / 8, bin_prefix[j+1] / 8), of stage_rp entries each.
// nullptr (the decoder then reads the column from U): no staging buffer, a
// column longer than stage_rp, or more candidates than the job's share.
template <typename T>
__device__ __forceinline__ c2<T>* stage_col(const qsft_plan& plan, int jid, int pos, int RP) {
  if (!plan.stage || RP > plan.stage_rp) return nullptr;
  const int64_t s0 = __ldg(plan.bin_prefix + jid) / 8, s1 = __ldg(plan.bin_prefix + jid + 1) / 8;
  if (pos >= s1 - s0) return nullptr;
  return reinterpret_cast<c2<T>*>(plan.stage) + (s0 + pos) * plan.stage_rp;
}

// Every phase deals the chunks of all jobs round-robin to the warps, so a warp
// needs the item count of every job before its own.  The blocks load the
// counts of a window of jobs at once (-1 for a job that has left the loop): a
// warp that walked the jobs reading each control record in turn paid a
// dependent L2 round trip per job before it reached its work.
constexpr int JOB_WIN = 256;
template <class F>
__device__ __forceinline__ void job_counts(int j0, int nj, int* s_cnt, F count) {
  __syncthreads();  // the previous window's counts are read by every warp
  for (int i = threadIdx.x; i < nj; i += blockDim.x) s_cnt[i] = count(j0 + i);
  __syncthreads();
}

// A warp takes 32 bins at a time, a lane per bin: the first iteration every
// bin (consecutive bins of a group: coalesced rows), later ones the bins the
// previous iteration's subtractions changed.  Each bin's class is reset (the
// multiton count kept up to date); a bin above the energy cutoff is queued in
// the job's candidate list, and the warp copies its column into the staging
// buffer at once -- the values are still in L2 -- so that the decoder reads
// one contiguous column instead of RP scattered sectors from HBM.
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_BLOCKS = 152 * 4;   // resident at once (4 blocks of 256 threads per SM)

template <typename T>
__device__ __forceinline__ void scan_phase(const qsft_plan& plan, int first) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  // every job's item count at once (up to JOB_WIN jobs; a warp reading the
  // control records in turn paid an L2 round trip per job: the first scan
  // measured 91 -> 79 us for 16 jobs), else the walk
  __shared__ int s_cnt[JOB_WIN];
  const bool win = plan.njobs <= JOB_WIN;
  if (win)
    job_counts(0, plan.njobs, s_cnt, [&](int jid) -> int {
      const qsft_ctrl* c = plan.ctrl + jid;
      if (__ldcg(&c->done)) return -1;
      return first ? plan.jobs[jid].C * plan.jobs[jid].B : __ldcg(&c->n_dirty[__ldcg(&c->iter) & 1]);
    });
  // Jobs last to first: the pass before a scan (the transform, or the previous
  // iteration's peel) walks them first to last, so the bins of the last jobs
  // are the ones still in L2 when the scan starts (16 transforms: first scan
  // 79.7 -> 71.5 us, second 70 -> 67 us against first-to-last)
  int64_t chunk0 = 0;  // 32-bin chunks of all jobs are dealt round-robin to the warps
  for (int jj = 0; jj < plan.njobs; ++jj) {
    const int jid = plan.njobs - 1 - jj;
    qsft_ctrl* ctl = plan.ctrl + jid;
    int cnt;
    if (win) {
      cnt = s_cnt[jid];
      if (cnt < 0) continue;
    } else {
      if (ctl->done) continue;
      cnt = first ? plan.jobs[jid].C * plan.jobs[jid].B : ctl->n_dirty[ctl->iter & 1];
    }
    const qsft_job* __restrict__ job = plan.jobs + jid;
    const int B = job->B, RP = job->R * job->P;
    const int parity = ctl->iter & 1;   // the dirty list the peel of iteration `iter` wrote
    const int nch = (cnt + 31) >> 5;
    const int start = (int)(((int64_t)gw - chunk0) % nw + nw) % nw;
    chunk0 += nch;
    if (start >= nch) continue;
    const double thr = job->cutoff * RP;
    const int32_t* list = plan.dirty + (int64_t)parity * plan.total_bins + job->off_bin;
    const c2<T>* U = reinterpret_cast<const c2<T>*>(plan.U) + job->off_U;
    for (int ch = start; ch < nch; ch += nw) {   // uniform over the warp
      const int i = ch * 32 + lane;
      bool is_cand = false, was_multi = false;
      int local = 0;
      if (i < cnt) {
        local = first ? i : list[i];
        const int64_t gb = job->off_bin + local;
        was_multi = !first && plan.bin_status[gb] == 1;
        plan.bin_status[gb] = 0;
        const int c = local / B, jb = local - (local / B) * B;
        is_cand = col_energy<T>(U + (int64_t)c * RP * B + jb, RP, B, thr) > thr;
      }
      const unsigned nm = __ballot_sync(0xffffffffu, was_multi);   // multitons re-classified: one atomic per warp
      if (lane == 0 && nm) atomicSub(&ctl->n_multi, __popc(nm));
      const int pos = warp_append(is_cand, jid, &ctl->n_cand);
      if (is_cand) plan.cand[job->off_bin + pos] = local;
      for (unsigned m = __ballot_sync(0xffffffffu, is_cand); m; m &= m - 1) {
        const int src = __ffs(m) - 1;
        const int p = __shfl_sync(0xffffffffu, pos, src);
        const int lc = __shfl_sync(0xffffffffu, local, src);
        c2<T>* dst = stage_col<T>(plan, jid, p, RP);
        if (dst) {
          const c2<T>* col = U + (int64_t)(lc / B) * RP * B + (lc - (lc / B) * B);
          for (int r = lane; r < RP; r += 32) dst[r] = col[(int64_t)r * B];
        }
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS, sizeof(T) == 4 ? 4 : 3) scan_kernel(qsft_plan plan, int first) {
  if (__ldcg(plan.done_count) >= plan.njobs) return;  // every job has left the loop
  scan_phase<T>(plan, first);
}

// ---------------------------------------------------------------- decode
// Groups of DEC_G lanes take the candidates of the job's list; each singleton
// is recorded at once (record_one) and the ball's first detection of the
// iteration appended to the iteration's list.
constexpr int DEC_BLOCKS = 152 * 5;   // resident at once (5 blocks of 128 threads per SM)

// blocks of NT threads (NT / G bin slots), groups of G lanes per candidate
template <typename T, int NT, int G>
__device__ __forceinline__ void decode_phase(const qsft_plan& plan) {
  constexpr int NB = NT / G;
  __shared__ float2 s_w[33 * 32];                            // roots, FP32
  __shared__ c2<T> s_col[NB][DEC_STAGE_RP];
  __shared__ __align__(16) uint8_t s_k[NB][DEC_KB];
  __shared__ uint8_t s_sym[NB][MAX_SYMS];
  for (int i = threadIdx.x; i < 33 * 32; i += blockDim.x)
    s_w[i] = make_float2((float)plan.roots[2 * i], (float)plan.roots[2 * i + 1]);
  __syncthreads();
  const int lane = threadIdx.x & 31, gi = lane % G;
  const int slot = threadIdx.x / G;                      // the block's bin slot of this group
  const unsigned gmask = ((1u << G) - 1) << (lane - gi);
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  const int ks = plan.kstride;
  c2<T>* sc = s_col[slot];
  uint8_t* kl = s_k[slot];
  __shared__ int s_cnt[JOB_WIN];
  int64_t chunk0 = 0;
  for (int j0 = 0; j0 < plan.njobs; j0 += JOB_WIN) {
    const int nj = min(JOB_WIN, plan.njobs - j0);
    job_counts(j0, nj, s_cnt, [&](int jid) -> int {
      const qsft_ctrl* c = plan.ctrl + jid;
      return __ldcg(&c->done) ? -1 : __ldcg(&c->n_cand);
    });
    for (int w = 0; w < nj; ++w) {
      const int jid = j0 + w, cnt = s_cnt[w];
      if (cnt < 0) continue;
      qsft_ctrl* ctl = plan.ctrl + jid;
      const int nch = (cnt + (32 / G) - 1) / (32 / G);
      const int start = (int)(((int64_t)gw - chunk0) % nw + nw) % nw;
      chunk0 += nch;
      if (start >= nch) continue;
      const qsft_job* __restrict__ job = plan.jobs + jid;
      const int q = job->q, n = job->n, b = job->b, B = job->B, P = job->P, R = job->R;
      const int RP = R * P, nsym = P - 1;
      const double thr = job->cutoff * RP;
      const bool staged = RP <= DEC_STAGE_RP;
      const bool words_ok = (n & 3) == 0 && ((job->off_D & 3) == 0);
      const float2* wq = s_w + q * 32;
      uint8_t* syms = job->src == QSFT_SRC_CODED ? s_sym[slot] : kl;
      const long long iter = (long long)ctl->iter + 1;
      for (int ch = start; ch < nch; ch += nw) {   // uniform over the warp: every lane runs every sync
        const int u = ch * (32 / G) + lane / G;
        const bool active = u < cnt;
        const int local = active ? plan.cand[job->off_bin + u] : 0;
        const int c = local / B, jb = local - (local / B) * B;
        const int64_t gb = job->off_bin + local;
        const c2<T>* col = reinterpret_cast<const c2<T>*>(plan.U) + job->off_U + (int64_t)c * RP * B + jb;
        const c2<T>* stg = active ? stage_col<T>(plan, jid, u, RP) : nullptr;
        if (staged && active) {
          if (stg)
            for (int r = gi; r < RP; r += G) sc[r] = stg[r];
          else
            for (int r = gi; r < RP; r += G) sc[r] = col[(int64_t)r * B];
        }
        __syncwarp();
        auto V = [&](int r) -> c2<T> { return staged ? sc[r] : col[(int64_t)r * B]; };
        // ---- channel decoding, symbols dealt over the group
        if (active) {
          if (job->chan == QSFT_CHAN_IDENTITY) {
            const c2<T> v0 = V(0);
            const T a0 = atan2(v0.y, v0.x);
            for (int i = 1 + gi; i < RP && i <= nsym; i += G) {
              const c2<T> vi = V(i);
              const T ai = atan2(vi.y, vi.x);
              double a = (double)((T)q * (ai - a0) / (T)6.283185307179586);
              if (sizeof(T) == 4 && fabs(a - floor(a) - 0.5) < 1e-3)
                a = (double)q * (atan2((double)vi.y, (double)vi.x) - atan2((double)v0.y, (double)v0.x)) /
                    6.283185307179586;
              long long m = (long long)rint(a);  // round half to even, like np.round
              m %= q;
              if (m < 0) m += q;
              syms[i - 1] = (uint8_t)m;
            }
          } else {
            for (int i = 1 + gi; i <= nsym; i += G) {
              T zr = 0, zi = 0;
              for (int r = 0; r < R; ++r) {
                const c2<T> u0 = V(r * P), ui = V(r * P + i);
                zr += u0.x * ui.x + u0.y * ui.y;
                zi += u0.y * ui.x - u0.x * ui.y;
              }
              if (sizeof(T) == 4) {
                float ang = atan2f((float)zi, (float)zr);
                if (ang < 0.f) ang += 6.28318530717958647f;
                const float tq = ang * (float)q * 0.15915494309189535f;
                if (fabsf(tq - floorf(tq) - 0.5f) >= 1e-3f) {
                  // away from a tie the nearest of 2 pi m / q, m = 0..q, is floor(tq + 1/2)
                  syms[i - 1] = (uint8_t)(((int)floorf(tq + 0.5f)) % q);
                  continue;
                }
                double dzr = 0, dzi = 0;  // near a rounding boundary: recompute in FP64
                for (int r = 0; r < R; ++r) {
                  const double2 u0 = to_d2(V(r * P)), ui = to_d2(V(r * P + i));
                  dzr += u0.x * ui.x + u0.y * ui.y;
                  dzi += u0.y * ui.x - u0.x * ui.y;
                }
                double ang64 = atan2(dzi, dzr);
                if (ang64 < 0) ang64 += 6.283185307179586;
                syms[i - 1] = (uint8_t)nearest_root(ang64, q);
              } else {
                double ang = (double)atan2(zi, zr);
                if (ang < 0) ang += 6.283185307179586;
                syms[i - 1] = (uint8_t)nearest_root(ang, q);
              }
            }
          }
        }
        __syncwarp();
        // ---- source decoding
        const bool coded = job->src == QSFT_SRC_CODED;
        if (coded && active && gi == 0) {
          const GFt g = make_gf(plan.gf_tables + job->rs_gf_off, q, job->rs_s);
          rs_decode(g, q, job->rs_s, job->rs_t, n, syms, kl, kl + n);
        }
        __syncwarp();
        for (int i = (coded ? 2 * n : n) + gi; i < ks; i += G) kl[i] = 0;
        __syncwarp();
        // ---- projection rho = <omega^(Dk), col> / RP and residual energy, rows
        //      dealt over the group: FP32 for FP32 plans (FP64 within 1% of the
        //      threshold), FP64 for FP64 plans
        const int8_t* Dc = plan.i8 + job->off_D + (int64_t)c * RP * n;
        auto project64 = [&](double2& rho_out, double& res_out) {
          double ar = 0, ai = 0;
          for (int r = gi; r < RP; r += G) {
            const double2 w = root(plan.roots, q, row_phase(Dc + (int64_t)r * n, kl, n, words_ok, q));
            const double2 v = to_d2(V(r));
            ar += w.x * v.x + w.y * v.y;
            ai += w.x * v.y - w.y * v.x;
          }
          ar = group_sum<G>(ar, gmask);
          ai = group_sum<G>(ai, gmask);
          const double2 rh = make_double2(ar / RP, ai / RP);
          double rs = 0;
          for (int r = gi; r < RP; r += G) {
            const double2 w = root(plan.roots, q, row_phase(Dc + (int64_t)r * n, kl, n, words_ok, q));
            const double2 v = to_d2(V(r));
            const double dx = v.x - (rh.x * w.x - rh.y * w.y);
            const double dy = v.y - (rh.x * w.y + rh.y * w.x);
            rs += dx * dx + dy * dy;
          }
          rho_out = rh;
          res_out = group_sum<G>(rs, gmask);
        };
        double2 rho = make_double2(0.0, 0.0);
        double res = 0.0;
        if (sizeof(T) == 4) {
          int ph[(DEC_STAGE_RP + G - 1) / G];
          float ar = 0.f, ai = 0.f;
  #pragma unroll
          for (int k = 0; k < (DEC_STAGE_RP + G - 1) / G; ++k) {
            const int r = gi + k * G;
            ph[k] = 0;
            if (r < RP) {
              ph[k] = row_phase(Dc + (int64_t)r * n, kl, n, words_ok, q);
              const float2 w = wq[ph[k]];
              const c2<T> v = V(r);
              ar += w.x * (float)v.x + w.y * (float)v.y;
              ai += w.x * (float)v.y - w.y * (float)v.x;
            }
          }
          for (int r = gi + DEC_STAGE_RP; r < RP; r += G) {  // rows past the register-held phases
            const float2 w = wq[row_phase(Dc + (int64_t)r * n, kl, n, words_ok, q)];
            const c2<T> v = V(r);
            ar += w.x * (float)v.x + w.y * (float)v.y;
            ai += w.x * (float)v.y - w.y * (float)v.x;
          }
          ar = group_sum<G>(ar, gmask) / (float)RP;
          ai = group_sum<G>(ai, gmask) / (float)RP;
          float rs = 0.f;
  #pragma unroll
          for (int k = 0; k < (DEC_STAGE_RP + G - 1) / G; ++k) {
            const int r = gi + k * G;
            if (r < RP) {
              const float2 w = wq[ph[k]];
              const c2<T> v = V(r);
              const float dx = (float)v.x - (ar * w.x - ai * w.y);
              const float dy = (float)v.y - (ar * w.y + ai * w.x);
              rs += dx * dx + dy * dy;
            }
          }
          for (int r = gi + DEC_STAGE_RP; r < RP; r += G) {
            const float2 w = wq[row_phase(Dc + (int64_t)r * n, kl, n, words_ok, q)];
            const c2<T> v = V(r);
            const float dx = (float)v.x - (ar * w.x - ai * w.y);
            const float dy = (float)v.y - (ar * w.y + ai * w.x);
            rs += dx * dx + dy * dy;
          }
          rs = group_sum<G>(rs, gmask);
          rho = make_double2(ar, ai);
          res = rs;
          if (fabsf(rs - (float)thr) <= 1e-2f * (float)thr) project64(rho, res);  // group-uniform
        } else {
          project64(rho, res);
        }
        // ---- bin match: digit t of M_c^T k equals digit t of j (MSB first), digits over the group
        bool ok = true;
        {
          const int8_t* Mc = plan.i8 + job->off_M + (int64_t)c * n * b;
          for (int t = gi; t < b; t += G) {
            int jr = jb;
            for (int tt = b - 1; tt > t; --tt) jr /= q;
            int dg = 0;
            for (int i = 0; i < n; ++i) dg += (int)Mc[i * b + t] * (int)kl[i];
            ok &= (dg % q) == (jr % q);
          }
        }
        const bool match = (__ballot_sync(0xffffffffu, !ok) & gmask) == 0;
        const bool single = match && !(res > thr);
        bool firstb = false;
        int bid = -1;
        if (active && gi == 0) {
          plan.bin_status[gb] = single ? 2 : 1;
          if (single) {
            plan.rho[2 * gb] = rho.x;   // the peel reads the coefficient of the ball's last bin
            plan.rho[2 * gb + 1] = rho.y;
            bid = record_one(plan, job, ctl, kl, local, rho, iter, ks, firstb);
          }
        }
        {  // the class counts, one atomic per warp and counter
          const unsigned ns = __ballot_sync(0xffffffffu, active && gi == 0 && single);
          const unsigned nm = __ballot_sync(0xffffffffu, active && gi == 0 && !single);
          if (lane == 0) {
            if (ns) atomicAdd(&ctl->n_single, __popc(ns));
            if (nm) atomicAdd(&ctl->n_multi, __popc(nm));
          }
        }
        const int pos = warp_append(firstb, jid, &ctl->n_unique);   // the iteration's list of balls
        if (firstb) plan.uniq[job->off_ball + pos] = bid;
        __syncwarp();  // the slot's buffers are reused by the next bin
      }
    }
  }
}

template <typename T, int G>
// FP32: 5 blocks per SM (up to 102 registers)
__global__ void __launch_bounds__(DEC_THREADS, sizeof(T) == 4 ? 5 : 4) decode_kernel(qsft_plan plan) {
  if (__ldcg(plan.done_count) >= plan.njobs) return;  // every job has left the loop
  decode_phase<T, DEC_THREADS, G>(plan);
}

// ---------------------------------------------------------------- peel
// Per job, by one block after every subtraction of the iteration: iteration
// count, cumulative peel count and the loop's stopping rules (qsft/qsft.py:151,
// 204-205); the counters of the next iteration start at zero.  *s_iter
// receives the largest iteration count (the WHILE node's bound).
__device__ __forceinline__ void end_iteration(const qsft_plan& plan, int* s_iter) {
  for (int jid = threadIdx.x; jid < plan.njobs; jid += blockDim.x) {
    volatile qsft_ctrl* ctl = plan.ctrl + jid;
    const qsft_job* job = plan.jobs + jid;
    if (ctl->done) continue;
    const int it = ctl->iter + 1;
    ctl->iter = it;
    atomicMax(s_iter, it);
    ctl->num_peeling = ctl->num_peeling + ctl->n_unique;
    if (ctl->n_multi == 0 || ctl->n_single == 0 || it >= job->max_iter || ctl->num_peeling >= job->peeling_max ||
        ctl->err != 0) {
      ctl->done = 1;
      atomicAdd(plan.done_count, 1);
    }
    ctl->n_single = 0;
    ctl->n_unique = 0;
    ctl->n_cand = 0;
    ctl->n_dirty[(it - 1) & 1] = 0;  // consumed by this iteration's scan
  }
}

// one bin-entry subtraction: U -= (dx, dy)
__device__ __forceinline__ void sub_entry(float2* p, float dx, float dy) {
  asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(-dx), "f"(-dy) : "memory");
}
__device__ __forceinline__ void sub_entry(double2* p, double dx, double dy) {
  atomicAdd(&p->x, -dx);
  atomicAdd(&p->y, -dy);
}

// Per (ball detected in the iteration, group l): each of the RP rows of bin
// M_l^T k gets U -= rho * omega^(<d_r, k>) (one vector reduction) and the
// changed bin is queued for the next scan once per iteration (stamped).  A
// job's long list (the first iteration) takes one thread per item; a short
// one takes DEC_G threads per item, digits and rows dealt over the group, to
// cut the latency of each item when there are few to overlap.  FP32 plans
// rotate rho in FP32 (the entries it is subtracted from are FP32).
template <typename T>
__device__ __forceinline__ void peel_phase(const qsft_plan& plan) {
  __shared__ float2 s_w[33 * 32];                     // FP32 roots, loaded on first use
  bool have_w = false;
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  const int ks = plan.kstride;
  __shared__ int s_cnt[JOB_WIN];
  int64_t chunk0 = 0;
  for (int j0 = 0; j0 < plan.njobs; j0 += JOB_WIN) {
    const int nj = min(JOB_WIN, plan.njobs - j0);
    job_counts(j0, nj, s_cnt, [&](int jid) -> int {
      const qsft_ctrl* c = plan.ctrl + jid;
      return __ldcg(&c->done) ? -1 : __ldcg(&c->n_unique) * __ldg(&plan.jobs[jid].C);
    });
    for (int w = 0; w < nj; ++w) {
      const int jid = j0 + w, cnt = s_cnt[w];
      if (cnt < 0) continue;
      qsft_ctrl* ctl = plan.ctrl + jid;
      const qsft_job* __restrict__ job = plan.jobs + jid;
      const int C = job->C;
      const int G = cnt >= PEEL_THREAD_MIN ? 1 : DEC_G, cpw = 32 / G, gi = lane % G;
      if (G > 1 && !have_w && cnt > 0) {  // uniform over the block: every thread sees the same counts
        for (int i = threadIdx.x; i < 33 * 32; i += blockDim.x)
          s_w[i] = make_float2((float)plan.roots[2 * i], (float)plan.roots[2 * i + 1]);
        __syncthreads();
        have_w = true;
      }
      const unsigned gmask = ((1u << G) - 1) << (lane - gi);
      const int nch = (cnt + cpw - 1) / cpw;
      const int start = (int)(((int64_t)gw - chunk0) % nw + nw) % nw;
      chunk0 += nch;
      if (start >= nch) continue;
      const int q = job->q, n = job->n, b = job->b, B = job->B;
      const int RP = job->R * job->P;
      const int iter = ctl->iter + 1;
      const int parity = iter & 1;
      const bool words_ok = (n & 3) == 0 && ((job->off_D & 3) == 0);
      const float2* wq = s_w + q * 32;
      int32_t* list = plan.dirty + (int64_t)parity * plan.total_bins + job->off_bin;
      for (int ch = start; ch < nch; ch += nw) {   // uniform over the warp
        const int it = ch * cpw + lane / G;
        bool fresh = false;
        int lb = 0;
        if (G == 1) {
          if (it < cnt) {
            const int u = it / C, l = it - (it / C) * C;
            const int bid = __ldcg(plan.uniq + job->off_ball + u);
            const int64_t gball = job->off_ball + bid;
            const unsigned long long best = __ldcg(reinterpret_cast<const unsigned long long*>(plan.ball_best) + gball);
            const int64_t gbest = job->off_bin + (int64_t)(best & 0xffffffffull);
            const double2 rho = make_double2(__ldcg(plan.rho + 2 * gbest), __ldcg(plan.rho + 2 * gbest + 1));
            const uint8_t* kl = plan.ball_k + gball * ks;  // written by the record kernel
            const int8_t* Ml = plan.i8 + job->off_M + (int64_t)l * n * b;
            int jl = 0;
            for (int t = 0; t < b; ++t) {  // bin index, MSB-first digits of M_l^T k
              int dg = 0;
              for (int i = 0; i < n; ++i) dg += (int)Ml[i * b + t] * (int)kl[i];
              jl = jl * q + dg % q;
            }
            c2<T>* Ul = reinterpret_cast<c2<T>*>(plan.U) + job->off_U + (int64_t)l * RP * B + jl;
            const int8_t* Dl = plan.i8 + job->off_D + (int64_t)l * RP * n;
            if (sizeof(T) == 4) {
              const float rx = (float)rho.x, ry = (float)rho.y;
              for (int r = 0; r < RP; ++r) {
                const double2 w = root(plan.roots, q, row_phase(Dl + (int64_t)r * n, kl, n, words_ok, q));
                const float wx = (float)w.x, wy = (float)w.y;
                sub_entry(Ul + (int64_t)r * B, rx * wx - ry * wy, rx * wy + ry * wx);
              }
            } else {
              for (int r = 0; r < RP; ++r) {
                const double2 w = root(plan.roots, q, row_phase(Dl + (int64_t)r * n, kl, n, words_ok, q));
                sub_entry(Ul + (int64_t)r * B, rho.x * w.x - rho.y * w.y, rho.x * w.y + rho.y * w.x);
              }
            }
            lb = l * B + jl;
            fresh = atomicExch(plan.bin_stamp + job->off_bin + lb, iter) != iter;
          }
        } else {
          const bool active = it < cnt;
          const int u = active ? it / C : 0, l = active ? it - (it / C) * C : 0;
          const int bid = active ? __ldcg(plan.uniq + job->off_ball + u) : 0;
          const int64_t gball = job->off_ball + bid;
          const uint8_t* kl = plan.ball_k + gball * ks;
          const int8_t* Ml = plan.i8 + job->off_M + (int64_t)l * n * b;
          int part = 0;  // this thread's digits of the bin index
          if (active)
            for (int t = gi; t < b; t += G) {
              int dg = 0;
              for (int i = 0; i < n; ++i) dg += (int)Ml[i * b + t] * (int)kl[i];
              int pw = 1;
              for (int tt = t + 1; tt < b; ++tt) pw *= q;
              part += (dg % q) * pw;
            }
          const int jl = group_sum_g(part, gmask, G);
          if (active) {
            const unsigned long long best = __ldcg(reinterpret_cast<const unsigned long long*>(plan.ball_best) + gball);
            const int64_t gbest = job->off_bin + (int64_t)(best & 0xffffffffull);
            const double2 rho = make_double2(__ldcg(plan.rho + 2 * gbest), __ldcg(plan.rho + 2 * gbest + 1));
            c2<T>* Ul = reinterpret_cast<c2<T>*>(plan.U) + job->off_U + (int64_t)l * RP * B + jl;
            const int8_t* Dl = plan.i8 + job->off_D + (int64_t)l * RP * n;
            if (sizeof(T) == 4) {
              const float rx = (float)rho.x, ry = (float)rho.y;
              for (int r = gi; r < RP; r += G) {
                const float2 w = wq[row_phase(Dl + (int64_t)r * n, kl, n, words_ok, q)];
                sub_entry(Ul + (int64_t)r * B, rx * w.x - ry * w.y, rx * w.y + ry * w.x);
              }
            } else {
              for (int r = gi; r < RP; r += G) {
                const double2 w = root(plan.roots, q, row_phase(Dl + (int64_t)r * n, kl, n, words_ok, q));
                sub_entry(Ul + (int64_t)r * B, rho.x * w.x - rho.y * w.y, rho.x * w.y + rho.y * w.x);
              }
            }
            lb = l * B + jl;
            if (gi == 0) fresh = atomicExch(plan.bin_stamp + job->off_bin + lb, iter) != iter;
          }
        }
        const int pos = warp_append(fresh, jid, &ctl->n_dirty[parity]);  // once per bin per iteration
        if (fresh) list[pos] = lb;
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(PEEL_THREADS) peel_kernel(qsft_plan plan, cudaGraphConditionalHandle cond,
                                                           int set_cond, int max_iter) {
  if (__ldcg(plan.done_count) >= plan.njobs) return;  // every job has left the loop (the same in every block)
  peel_phase<T>(plan);
  // the block that finishes last closes the iteration (every other block's
  // subtractions, list entries and counters are visible to it)
  __shared__ int s_last, s_iter;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(plan.done_count + 1, 1) == (int)gridDim.x - 1;
    s_iter = 0;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  end_iteration(plan, &s_iter);
  __syncthreads();
  if (threadIdx.x == 0) {
    plan.done_count[1] = 0;  // the next iteration's tickets
    if (set_cond)
      cudaGraphSetConditional(cond, (__ldcg(plan.done_count) < plan.njobs && s_iter < max_iter) ? 1u : 0u);
  }
}

// ---------------------------------------------------------------- persistent loop
// The whole loop in one cooperative launch: every block runs the scan, decode
// and peel phases of an iteration in turn, separated by grid-wide barriers,
// block 0 closes the iteration between them, and the loop ends when every
// job has left it (or after max_iter).  The grid is what the GPU holds at once,
// so every block is resident.  Barrier waits are bounded in time: a wait that
// runs out records QSFT_ERR_TIMEOUT in plan.status and its block returns (the
// others then run out at the next barrier); the host reads the status.
constexpr int LOOP_THREADS = 128;
constexpr unsigned long long BARRIER_TIMEOUT_NS = 2000000000ull;  // 2 s

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// grid barrier on done_count[2] (arrivals) and done_count[3] (generation)
__device__ __forceinline__ bool grid_barrier(const qsft_plan& plan, int expected) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile int* gen = plan.done_count + 3;
    const int g = *gen;
    __threadfence();
    s_ok = 1;
    if (atomicAdd(plan.done_count + 2, 1) == expected - 1) {
      atomicExch(plan.done_count + 2, 0);
      __threadfence();
      atomicAdd(plan.done_count + 3, 1);
    } else {
      const unsigned long long t0 = global_ns();
      while (*gen == g) {
        if (global_ns() - t0 > BARRIER_TIMEOUT_NS) {
          s_ok = 0;
          atomicExch(plan.status, (int)QSFT_ERR_TIMEOUT);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return s_ok != 0;
}

template <typename T>
__global__ void __launch_bounds__(LOOP_THREADS, 4) peel_loop_kernel(qsft_plan plan, int max_iter) {
  // test only: a barrier that waits for one block more than the grid has
  const int expected = (int)gridDim.x + ((plan.flags & QSFT_PLAN_TEST_BARRIER_TIMEOUT) ? 1 : 0);
  __shared__ int s_iter;
  for (int it = 0; it < max_iter; ++it) {
    if (__ldcg(plan.done_count) >= plan.njobs) break;  // the same in every block: read after a barrier
    scan_phase<T>(plan, it == 0);
    if (!grid_barrier(plan, expected)) return;
    decode_phase<T, LOOP_THREADS, DEC_G>(plan);
    if (!grid_barrier(plan, expected)) return;
    peel_phase<T>(plan);
    if (!grid_barrier(plan, expected)) return;
    if (blockIdx.x == 0) {
      if (threadIdx.x == 0) s_iter = 0;
      __syncthreads();
      end_iteration(plan, &s_iter);
    }
    if (!grid_barrier(plan, expected)) return;
  }
}

template <typename T>
static int run_persistent(const qsft_plan* plan, int max_iter, cudaStream_t st) {
  static int sms[128], per[2][128];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128) return QSFT_ERR_CUDA;
  const int pi = sizeof(T) == 4 ? 0 : 1;
  if (!sms[dev] && cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return QSFT_ERR_CUDA;
  if (!per[pi][dev] &&
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[pi][dev], peel_loop_kernel<T>, LOOP_THREADS, 0) != cudaSuccess)
    return QSFT_ERR_CUDA;
  if (per[pi][dev] < 1) return QSFT_ERR_TOO_LARGE;
  qsft_plan pl = *plan;
  int mi = max_iter;
  void* args[] = {&pl, &mi};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(sms[dev] * per[pi][dev]));
  cfg.blockDim = dim3(LOOP_THREADS);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelExC(&cfg, (const void*)peel_loop_kernel<T>, args) != cudaSuccess) return QSFT_ERR_CUDA;
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
}

template <typename T>
static int iteration(const qsft_plan* plan, int first, cudaStream_t st, cudaGraphConditionalHandle cond = 0,
                     int set_cond = 0, int max_iter = 0) {
  scan_kernel<T><<<SCAN_BLOCKS, SCAN_THREADS, 0, st>>>(*plan, first);
  QSFT_CUDA_CHECK_LAUNCH();
  // groups of 8 lanes for the first iteration's many candidates, of 16 for the
  // later iterations' few (ms, 16 transforms: iteration 1 0.119 with 8, 0.140
  // with 16; iteration 2 0.055 with 8, 0.042 with 16)
  if (first)
    decode_kernel<T, DEC_G><<<DEC_BLOCKS, DEC_THREADS, 0, st>>>(*plan);
  else
    decode_kernel<T, DEC_G_LATER><<<DEC_BLOCKS, DEC_THREADS, 0, st>>>(*plan);
  QSFT_CUDA_CHECK_LAUNCH();
  peel_kernel<T><<<LIST_BLOCKS, PEEL_THREADS, 0, st>>>(*plan, cond, set_cond, max_iter);
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
}

// The body of the WHILE node: iterations 2.. as kernel nodes of `body`.
template <typename T>
static int add_body(const qsft_plan* plan, cudaGraph_t body, cudaGraphConditionalHandle cond, int max_iter) {
  qsft_plan pl = *plan;
  int first = 0, set = 1, mi = max_iter;
  void* a0[] = {&pl, &first};
  void* a1[] = {&pl};
  void* a2[] = {&pl, &cond, &set, &mi};
  struct K {
    void* f;
    unsigned grid, block;
    void** args;
  } ks[] = {{(void*)scan_kernel<T>, SCAN_BLOCKS, SCAN_THREADS, a0},
            {(void*)decode_kernel<T, DEC_G_LATER>, DEC_BLOCKS, DEC_THREADS, a1},
            {(void*)peel_kernel<T>, LIST_BLOCKS, PEEL_THREADS, a2}};
  cudaGraphNode_t prev = nullptr;
  for (const K& k : ks) {
    cudaKernelNodeParams kp = {};
    kp.func = k.f;
    kp.gridDim = dim3(k.grid);
    kp.blockDim = dim3(k.block);
    kp.sharedMemBytes = 0;
    kp.kernelParams = k.args;
    cudaGraphNode_t node;
    if (cudaGraphAddKernelNode(&node, body, prev ? &prev : nullptr, prev ? 1 : 0, &kp) != cudaSuccess)
      return QSFT_ERR_CUDA;
    count_launch();
    prev = node;
  }
  return QSFT_OK;
}

// Inside a stream capture: iteration 1 on the stream, then one WHILE node
// whose body runs further iterations only while some job is still in its
// loop -- finished batches cost no launches.
template <typename T>
static int run_graph(const qsft_plan* plan, int max_iter, cudaStream_t st) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  if (cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd) != cudaSuccess) return QSFT_ERR_CUDA;
  cudaGraphConditionalHandle cond;
  if (cudaGraphConditionalHandleCreate(&cond, g, 0, cudaGraphCondAssignDefault) != cudaSuccess) return QSFT_ERR_CUDA;
  int rc = iteration<T>(plan, 1, st, cond, 1, max_iter);
  if (rc != QSFT_OK || max_iter <= 1) return rc;
  if (cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd) != cudaSuccess) return QSFT_ERR_CUDA;
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = cond;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  if (cudaGraphAddNode(&node, g, deps, nullptr, nd, &np) != cudaSuccess) return QSFT_ERR_CUDA;
  rc = add_body<T>(plan, np.conditional.phGraph_out[0], cond, max_iter);
  if (rc != QSFT_OK) return rc;
  if (cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies) != cudaSuccess)
    return QSFT_ERR_CUDA;
  return QSFT_OK;
}

static int check_plan(const qsft_plan* p) {
  if (!p || p->njobs <= 0 || !p->jobs || !p->bin_prefix || !p->i8 || !p->U || !p->rho || !p->ball_best ||
      !p->uniq || !p->ball_tab || !p->ball_k || !p->ball_sum || !p->ball_cnt ||
      !p->ctrl || !p->roots || !p->bin_status || !p->bin_stamp || !p->dirty || !p->cand || !p->done_count)
    return QSFT_ERR_ARG;
  if (p->kstride < 16 || (p->kstride & 15) || p->kstride > 2 * QSFT_MAX_N) return QSFT_ERR_ARG;
  if (p->stage && (p->stage_rp < 1 || p->stage_rp > DEC_STAGE_RP)) return QSFT_ERR_ARG;
  if (p->max_q > QSFT_MAX_Q || p->max_n > QSFT_MAX_N) return QSFT_ERR_TOO_LARGE;
  if (p->prec != QSFT_F32 && p->prec != QSFT_F64) return QSFT_ERR_ARG;
  if (p->total_bins <= 0) return QSFT_ERR_ARG;
  return QSFT_OK;
}

}  // namespace qsft

using namespace qsft;

extern "C" int qsft_peel_init(const qsft_plan* plan, qsft_stream_t stream) {
  const int rc = check_plan(plan);
  if (rc != QSFT_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemsetAsync(plan->ctrl, 0, sizeof(qsft_ctrl) * plan->njobs, st) != cudaSuccess ||
      cudaMemsetAsync(plan->ball_tab, 0, sizeof(int64_t) * plan->total_slots, st) != cudaSuccess ||
      cudaMemsetAsync(plan->ball_best, 0, sizeof(int64_t) * plan->total_balls, st) != cudaSuccess ||
      cudaMemsetAsync(plan->ball_sum, 0, sizeof(double) * 2 * plan->total_balls, st) != cudaSuccess ||
      cudaMemsetAsync(plan->ball_cnt, 0, sizeof(int32_t) * plan->total_balls, st) != cudaSuccess ||
      cudaMemsetAsync(plan->bin_stamp, 0, sizeof(int32_t) * plan->total_bins, st) != cudaSuccess ||
      cudaMemsetAsync(plan->done_count, 0, 4 * sizeof(int32_t), st) != cudaSuccess)
    return QSFT_ERR_CUDA;
  return QSFT_OK;
}

extern "C" int qsft_peel_iteration(const qsft_plan* plan, int first, qsft_stream_t stream) {
  const int rc = check_plan(plan);
  if (rc != QSFT_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  return plan->prec == QSFT_F32 ? iteration<float>(plan, first, st) : iteration<double>(plan, first, st);
}

extern "C" int qsft_peel_run(const qsft_plan* plan, int max_iter, qsft_stream_t stream) {
  if (max_iter < 0) return QSFT_ERR_ARG;
  if (max_iter == 0) return QSFT_OK;
  const int rc = check_plan(plan);
  if (rc != QSFT_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  cudaStreamCaptureStatus cs;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) return QSFT_ERR_CUDA;
  if (cs == cudaStreamCaptureStatusActive)
    return plan->prec == QSFT_F32 ? run_graph<float>(plan, max_iter, st) : run_graph<double>(plan, max_iter, st);
  for (int i = 0; i < max_iter; ++i) {  // eager: finished jobs make the later launches no-ops
    const int r = plan->prec == QSFT_F32 ? iteration<float>(plan, i == 0, st) : iteration<double>(plan, i == 0, st);
    if (r != QSFT_OK) return r;
  }
  return QSFT_OK;
}

extern "C" int qsft_peel_persistent(const qsft_plan* plan, int max_iter, qsft_stream_t stream) {
  if (max_iter < 0) return QSFT_ERR_ARG;
  if (max_iter == 0) return QSFT_OK;
  const int rc = check_plan(plan);
  if (rc != QSFT_OK) return rc;
  if (!plan->status) return QSFT_ERR_ARG;  // a barrier that runs out reports there
  cudaStream_t st = (cudaStream_t)stream;
  return plan->prec == QSFT_F32 ? run_persistent<float>(plan, max_iter, st) : run_persistent<double>(plan, max_iter, st);
}
