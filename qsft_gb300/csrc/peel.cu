// Singleton detection and peeling: QSFT.transform's while-loop
// (qsft/qsft.py:151-255) for a batch of transforms.
//
// One iteration = four launches:
//   scan          thread per bin: the zeroton test ||col||^2 > cutoff*len
//                 (qsft/qsft.py:164); bins above it are queued.  The first
//                 iteration scans every bin; later ones only the bins that the
//                 previous subtractions changed (the rest keep their class:
//                 it is a function of the bin's unchanged values), and the
//                 multiton count is kept up to date as classes change.
//   decode        warp per queued bin: channel decoding of k (noiseless
//                 qsft/reconstruct.py:12-31 or NSO "nso1" :100-113, lanes over
//                 symbols), optional Reed-Solomon source decoding (:34-51),
//                 FP64 projection rho = <omega^(Dk), col>/len and FP64 residual
//                 (lanes over rows, warp reductions), bin-match test
//                 (qsft/qsft.py:174-190).  Singletons are deduplicated by k in a
//                 per-iteration hash table that keeps the largest (group, bin)
//                 -- the reference's dict order, `ball_values` (:209-216) -- and
//                 their rho goes to the job's result store (the `result` list
//                 and its running mean, :217, 247-255).
//   peel          warp per distinct k: subtract rho * omega^(D_l k) from bin
//                 M_l^T k (mod q) of every group l (qsft/qsft.py:223-241) and
//                 queue each changed bin for the next scan.
//   iter_end      per job: iteration count, cumulative peel count and the
//                 loop's stopping rules (qsft/qsft.py:151, 204-205).
//
// FP32 data path: bins are stored as float2.  Energy and phase decisions that
// fall within a small band of their thresholds are recomputed in FP64; the
// coefficient projection and residual energy are always computed in FP64.
#include "common.cuh"
#include "rs.cuh"

namespace qsft {

constexpr int SCAN_THREADS = 256;
constexpr int WARPS_PER_BLOCK = 8;
constexpr int MAX_SYMS = 256;  // channel symbols per bin (P - 1 <= 256)
constexpr int LIST_BLOCKS = 152 * 8;

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
// compare our row with a row another warp wrote (read through L2)
__device__ __forceinline__ bool row_eq(const uint8_t* mine, const uint8_t* other, int words) {
  const uint32_t* a = reinterpret_cast<const uint32_t*>(mine);
  const uint32_t* b = reinterpret_cast<const uint32_t*>(other);
  for (int i = 0; i < words; ++i)
    if (a[i] != __ldcg(b + i)) return false;
  return true;
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
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// ||col||^2 with the FP64 recomputation band of the FP32 path
template <typename T>
__device__ __forceinline__ double col_energy(const c2<T>* col, int RP, int B, double thr) {
  T e = 0;
  for (int r = 0; r < RP; ++r) {
    const c2<T> v = col[(int64_t)r * B];
    e += v.x * v.x + v.y * v.y;
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

// ---------------------------------------------------------------- scan
// first iteration: every bin of every active job
template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) scan_all_kernel(qsft_plan plan) {
  const int64_t gb = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool inrange = gb < plan.total_bins;
  const int jid = find_job(plan.bin_prefix, plan.njobs, inrange ? gb : plan.total_bins - 1);
  const qsft_job* __restrict__ job = plan.jobs + jid;
  qsft_ctrl* ctl = plan.ctrl + jid;
  const int B = job->B, RP = job->R * job->P;
  const int local = (int)(gb - job->off_bin);
  bool cand = false;
  if (inrange && !ctl->done) {
    const int c = local / B, jb = local - (local / B) * B;
    const c2<T>* col = reinterpret_cast<const c2<T>*>(plan.U) + job->off_U + (int64_t)c * RP * B + jb;
    const double thr = job->cutoff * RP;
    cand = col_energy<T>(col, RP, B, thr) > thr;
    plan.bin_status[gb] = 0;
  }
  const int pos = warp_append(cand, jid, &ctl->n_cand);
  if (cand) plan.cand[job->off_bin + pos] = local;
}

// later iterations: the bins the previous iteration's subtractions changed
template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) scan_dirty_kernel(qsft_plan plan) {
  if (__ldcg(plan.done_count) >= plan.njobs) return;  // every job has left the loop
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int gw = tid >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  int64_t chunk0 = 0;  // 32-entry chunks of all jobs' lists are dealt round-robin to the warps
  for (int jid = 0; jid < plan.njobs; ++jid) {
    qsft_ctrl* ctl = plan.ctrl + jid;
    if (ctl->done) continue;
    const int parity = (ctl->iter) & 1;  // written by the peel of iteration `iter`
    const int cnt = ctl->n_dirty[parity];
    const int nch = (cnt + 31) >> 5;
    const int start = (int)(((int64_t)gw - chunk0) % nw + nw) % nw;
    chunk0 += nch;
    if (start >= nch) continue;
    const qsft_job* __restrict__ job = plan.jobs + jid;
    const int B = job->B, RP = job->R * job->P;
    const double thr = job->cutoff * RP;
    const int32_t* list = plan.dirty + (int64_t)parity * plan.total_bins + job->off_bin;
    // all threads of a warp iterate together so that warp_append sees full warps
    for (int ch = start; ch < nch; ch += nw) {
      const int i = ch * 32 + (tid & 31);
      bool cand = false;
      int local = 0;
      if (i < cnt) {
        local = list[i];
        const int64_t gb = job->off_bin + local;
        if (plan.bin_status[gb] == 1) atomicSub(&ctl->n_multi, 1);
        plan.bin_status[gb] = 0;
        const int c = local / B, jb = local - (local / B) * B;
        const c2<T>* col = reinterpret_cast<const c2<T>*>(plan.U) + job->off_U + (int64_t)c * RP * B + jb;
        cand = col_energy<T>(col, RP, B, thr) > thr;
      }
      const int pos = warp_append(cand, jid, &ctl->n_cand);
      if (cand) plan.cand[job->off_bin + pos] = local;
    }
  }
}

// ---------------------------------------------------------------- decode
template <typename T>
__global__ void __launch_bounds__(WARPS_PER_BLOCK * 32) decode_kernel(qsft_plan plan) {
  if (__ldcg(plan.done_count) >= plan.njobs) return;  // every job has left the loop
  __shared__ __align__(16) uint8_t s_k[WARPS_PER_BLOCK][QSFT_MAX_N + 16];
  __shared__ uint8_t s_sym[WARPS_PER_BLOCK][MAX_SYMS];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int gw = blockIdx.x * WARPS_PER_BLOCK + wib;
  const int nw = gridDim.x * WARPS_PER_BLOCK;
  uint8_t* kl = s_k[wib];
  uint8_t* syms = s_sym[wib];
  int64_t base = 0;  // items of all jobs are dealt round-robin to the warps of the grid
  for (int jid = 0; jid < plan.njobs; ++jid) {
    qsft_ctrl* ctl = plan.ctrl + jid;
    if (ctl->done) continue;
    const int cnt = ctl->n_cand;
    const int start = (int)(((int64_t)gw - base) % nw + nw) % nw;
    base += cnt;
    if (start >= cnt) continue;
    const qsft_job* __restrict__ job = plan.jobs + jid;
    const int q = job->q, n = job->n, b = job->b, B = job->B, P = job->P, R = job->R;
    const int RP = R * P, nsym = P - 1;
    const double thr = job->cutoff * RP;
    const int ks = plan.kstride, words = ks / 4;
    const long long iter = (long long)ctl->iter + 1;
    for (int u = start; u < cnt; u += nw) {
      const int local = plan.cand[job->off_bin + u];
      const int c = local / B, jb = local - (local / B) * B;
      const int64_t gb = job->off_bin + local;
      const c2<T>* col = reinterpret_cast<const c2<T>*>(plan.U) + job->off_U + (int64_t)c * RP * B + jb;
      // ---- channel decoding, lanes over symbols
      if (job->chan == QSFT_CHAN_IDENTITY) {
        const c2<T> v0 = col[0];
        const T a0 = atan2(v0.y, v0.x);
        for (int i = lane + 1; i < RP && i <= nsym; i += 32) {
          const c2<T> vi = col[(int64_t)i * B];
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
        for (int i = lane + 1; i <= nsym; i += 32) {
          T zr = 0, zi = 0;
          for (int r = 0; r < R; ++r) {
            const c2<T> u0 = col[(int64_t)(r * P) * B];
            const c2<T> ui = col[(int64_t)(r * P + i) * B];
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
              const double2 u0 = to_d2(col[(int64_t)(r * P) * B]);
              const double2 ui = to_d2(col[(int64_t)(r * P + i) * B]);
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
      __syncwarp();
      // ---- source decoding
      if (job->src == QSFT_SRC_CODED) {
        if (lane == 0) {
          const GFt g = make_gf(plan.gf_tables + job->rs_gf_off, q, job->rs_s);
          rs_decode(g, q, job->rs_s, job->rs_t, n, syms, kl);
        }
      } else {
        for (int i = lane; i < n; i += 32) kl[i] = syms[i];
      }
      __syncwarp();
      for (int i = n + lane; i < ks; i += 32) kl[i] = 0;
      __syncwarp();
      // ---- FP64 projection and residual, lanes over rows (phases <d_r, k> mod q
      //      of the first 4*32 rows kept in registers between the two passes)
      const int8_t* Dc = plan.i8 + job->off_D + (int64_t)c * RP * n;
      const bool words_ok = (n & 3) == 0 && ((job->off_D & 3) == 0);
      auto phase = [&](int r) -> int {
        const int8_t* dr = Dc + (int64_t)r * n;
        int ph = 0;
        if (words_ok) {
          const uint32_t* dw = reinterpret_cast<const uint32_t*>(dr);
          const uint32_t* kw = reinterpret_cast<const uint32_t*>(kl);
          for (int w = 0; w < (n >> 2); ++w) ph = (int)__dp4a((unsigned)__ldg(dw + w), (unsigned)kw[w], (unsigned)ph);
        } else {
          for (int i = 0; i < n; ++i) ph += (int)dr[i] * (int)kl[i];
        }
        return ph % q;
      };
      int phc[4];
      double ar = 0, ai = 0;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int r = lane + 32 * k;
        phc[k] = 0;
        if (r < RP) {
          phc[k] = phase(r);
          const double2 w = root(plan.roots, q, phc[k]);
          const double2 v = to_d2(col[(int64_t)r * B]);
          ar += w.x * v.x + w.y * v.y;
          ai += w.x * v.y - w.y * v.x;
        }
      }
      for (int r = lane + 128; r < RP; r += 32) {
        const double2 w = root(plan.roots, q, phase(r));
        const double2 v = to_d2(col[(int64_t)r * B]);
        ar += w.x * v.x + w.y * v.y;
        ai += w.x * v.y - w.y * v.x;
      }
      ar = warp_sum(ar);
      ai = warp_sum(ai);
      const double2 rho = make_double2(ar / RP, ai / RP);
      double res = 0;
      auto resid = [&](int r, int ph) {
        const double2 w = root(plan.roots, q, ph);
        const double2 v = to_d2(col[(int64_t)r * B]);
        const double dx = v.x - (rho.x * w.x - rho.y * w.y);
        const double dy = v.y - (rho.x * w.y + rho.y * w.x);
        res += dx * dx + dy * dy;
      };
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int r = lane + 32 * k;
        if (r < RP) resid(r, phc[k]);
      }
      for (int r = lane + 128; r < RP; r += 32) resid(r, phase(r));
      res = warp_sum(res);
      // ---- bin match: M_c^T k = digits of j (MSB first), lanes over the b digits
      bool ok = true;
      if (lane < b) {
        const int8_t* Mc = plan.i8 + job->off_M + (int64_t)c * n * b;
        int dg = 0;
        for (int i = 0; i < n; ++i) dg += (int)Mc[i * b + lane] * (int)kl[i];
        int jr = jb;
        for (int t = b - 1; t > lane; --t) jr /= q;
        ok = (dg % q) == (jr % q);
      }
      const bool match = __all_sync(0xffffffffu, ok);
      const bool single = match && !(res > thr);
      if (lane == 0) plan.bin_status[gb] = single ? 2 : 1;
      if (!single) {
        if (lane == 0) atomicAdd(&ctl->n_multi, 1);
        __syncwarp();
        continue;
      }
      // ---- singleton: record k and rho, dedupe, add to the result store
      uint8_t* krow = plan.kbuf + gb * ks;
      for (int w = lane; w < words; w += 32)
        reinterpret_cast<uint32_t*>(krow)[w] = reinterpret_cast<const uint32_t*>(kl)[w];
      if (lane == 0) {
        plan.rho[2 * gb] = rho.x;
        plan.rho[2 * gb + 1] = rho.y;
      }
      __threadfence();
      __syncwarp();
      if (lane == 0) {
        atomicAdd(&ctl->n_single, 1);
        const uint32_t h = hash_row(kl, words);
        const int64_t cap = job->table_cap, mask = cap - 1;
        const long long stamp = iter << 32;
        unsigned long long* tk = reinterpret_cast<unsigned long long*>(plan.tab_key + job->off_slot);
        int64_t slot = h & mask;
        bool found = false, owner = false;
        for (int64_t probe = 0; probe < cap && !found; ++probe) {
          unsigned long long cur = atomicAdd(tk + slot, 0ull);
          if ((long long)(cur >> 32) != iter) {
            const unsigned long long mine = (unsigned long long)(stamp | (local + 1));
            const unsigned long long prev = atomicCAS(tk + slot, cur, mine);
            if (prev == cur) {
              owner = found = true;
              break;
            }
            cur = prev;
          }
          if ((long long)(cur >> 32) == iter) {
            const int64_t ob = (int64_t)(cur & 0xffffffffull) - 1;
            if (row_eq(kl, plan.kbuf + (job->off_bin + ob) * ks, words)) {
              found = true;
              break;
            }
            slot = (slot + 1) & mask;
          }
        }
        if (!found) {
          atomicExch(&ctl->err, (int)QSFT_ERR_OVERFLOW);
        } else {
          if (owner) {
            const int uix = atomicAdd(&ctl->n_unique, 1);
            plan.uniq[job->off_slot + uix] = (int32_t)slot;
          }
          atomicMax(reinterpret_cast<unsigned long long*>(plan.tab_best + job->off_slot + slot),
                    (unsigned long long)(stamp | local));
          int32_t* bt = plan.ball_tab + job->off_slot;
          int64_t s2 = h & mask;
          int myid = -1, bid = -1;
          for (int64_t probe = 0; probe < cap; ++probe) {
            int cur = atomicAdd(bt + s2, 0);
            if (cur == 0) {
              if (myid < 0) {
                myid = atomicAdd(&ctl->n_balls, 1);
                if (myid >= job->ball_cap) break;
                uint32_t* dst = reinterpret_cast<uint32_t*>(plan.ball_k + (job->off_ball + myid) * ks);
                for (int w = 0; w < words; ++w) dst[w] = reinterpret_cast<const uint32_t*>(kl)[w];
                __threadfence();
              }
              const int prev = atomicCAS(bt + s2, 0, myid + 1);
              if (prev == 0) {
                bid = myid;
                break;
              }
              cur = prev;
            }
            if (row_eq(kl, plan.ball_k + (job->off_ball + cur - 1) * ks, words)) {
              bid = cur - 1;
              break;
            }
            s2 = (s2 + 1) & mask;
          }
          if (bid < 0) {
            atomicExch(&ctl->err, (int)QSFT_ERR_OVERFLOW);
          } else {
            atomicAdd(plan.ball_sum + 2 * (job->off_ball + bid), rho.x);
            atomicAdd(plan.ball_sum + 2 * (job->off_ball + bid) + 1, rho.y);
            atomicAdd(plan.ball_cnt + job->off_ball + bid, 1);
          }
        }
      }
      __syncwarp();
    }
  }
}

// ---------------------------------------------------------------- peel
template <typename T>
__global__ void __launch_bounds__(WARPS_PER_BLOCK * 32) peel_kernel(qsft_plan plan) {
  if (__ldcg(plan.done_count) >= plan.njobs) return;  // every job has left the loop
  __shared__ uint8_t sk[WARPS_PER_BLOCK][QSFT_MAX_N];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int gw = blockIdx.x * WARPS_PER_BLOCK + wib;
  const int nw = gridDim.x * WARPS_PER_BLOCK;
  int64_t base = 0;  // balls of all jobs are dealt round-robin to the warps of the grid
  for (int jid = 0; jid < plan.njobs; ++jid) {
    qsft_ctrl* ctl = plan.ctrl + jid;
    if (ctl->done) continue;
    const int cnt = ctl->n_unique;
    const int start = (int)(((int64_t)gw - base) % nw + nw) % nw;
    base += cnt;
    if (start >= cnt) continue;
    const qsft_job* __restrict__ job = plan.jobs + jid;
    const int q = job->q, n = job->n, b = job->b, B = job->B, C = job->C;
    const int RP = job->R * job->P;
    const int iter = ctl->iter + 1;
    const int parity = iter & 1;
    int32_t* list = plan.dirty + (int64_t)parity * plan.total_bins + job->off_bin;
    for (int u = start; u < cnt; u += nw) {
      const int slot = plan.uniq[job->off_slot + u];
      const unsigned long long key = __ldcg(reinterpret_cast<const unsigned long long*>(plan.tab_key + job->off_slot) + slot);
      const unsigned long long best = __ldcg(reinterpret_cast<const unsigned long long*>(plan.tab_best + job->off_slot) + slot);
      const int64_t owner = (int64_t)(key & 0xffffffffull) - 1;
      const int64_t bestb = (int64_t)(best & 0xffffffffull);
      const uint8_t* krow = plan.kbuf + (job->off_bin + owner) * plan.kstride;
      for (int i = lane; i < n; i += 32) sk[wib][i] = __ldcg(krow + i);
      __syncwarp();
      const double2 rho = make_double2(__ldcg(plan.rho + 2 * (job->off_bin + bestb)),
                                       __ldcg(plan.rho + 2 * (job->off_bin + bestb) + 1));
      for (int l = 0; l < C; ++l) {
        const int8_t* Ml = plan.i8 + job->off_M + (int64_t)l * n * b;
        int contrib = 0;
        if (lane < b) {
          int dg = 0;
          for (int i = 0; i < n; ++i) dg += (int)Ml[i * b + lane] * (int)sk[wib][i];
          dg %= q;
          int pw = 1;
          for (int t = lane + 1; t < b; ++t) pw *= q;
          contrib = dg * pw;
        }
        const int jl = __reduce_add_sync(0xffffffffu, contrib);
        c2<T>* Ul = reinterpret_cast<c2<T>*>(plan.U) + job->off_U + (int64_t)l * RP * B + jl;
        const int8_t* Dl = plan.i8 + job->off_D + (int64_t)l * RP * n;
        for (int r = lane; r < RP; r += 32) {
          int ph = 0;
          for (int i = 0; i < n; ++i) ph += (int)Dl[(int64_t)r * n + i] * (int)sk[wib][i];
          const double2 w = root(plan.roots, q, ph % q);
          const double dx = rho.x * w.x - rho.y * w.y;
          const double dy = rho.x * w.y + rho.y * w.x;
          T* p = reinterpret_cast<T*>(Ul + (int64_t)r * B);
          atomicAdd(p, (T)(-dx));
          atomicAdd(p + 1, (T)(-dy));
        }
        if (lane == 0) {  // queue the changed bin for the next scan (once per iteration)
          const int lb = l * B + jl;
          if (atomicExch(plan.bin_stamp + job->off_bin + lb, iter) != iter) {
            const int pos = atomicAdd(&ctl->n_dirty[parity], 1);
            list[pos] = lb;
          }
        }
      }
      __syncwarp();
    }
  }
}

__global__ void iter_end_kernel(qsft_plan plan) {
  if (__ldcg(plan.done_count) >= plan.njobs) return;
  const int jid = blockIdx.x * blockDim.x + threadIdx.x;
  if (jid >= plan.njobs) return;
  qsft_ctrl* ctl = plan.ctrl + jid;
  const qsft_job* job = plan.jobs + jid;
  if (ctl->done) return;
  const int it = ctl->iter + 1;
  ctl->iter = it;
  ctl->num_peeling += ctl->n_unique;
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

template <typename T>
static int iteration(const qsft_plan* plan, int first, cudaStream_t st) {
  if (first) {
    const int64_t grid = (plan->total_bins + SCAN_THREADS - 1) / SCAN_THREADS;
    if (grid > 0x7fffffffLL) return QSFT_ERR_TOO_LARGE;
    scan_all_kernel<T><<<(unsigned)grid, SCAN_THREADS, 0, st>>>(*plan);
  } else {
    scan_dirty_kernel<T><<<LIST_BLOCKS, SCAN_THREADS, 0, st>>>(*plan);
  }
  QSFT_CUDA_CHECK_LAUNCH();
  decode_kernel<T><<<LIST_BLOCKS, WARPS_PER_BLOCK * 32, 0, st>>>(*plan);
  QSFT_CUDA_CHECK_LAUNCH();
  peel_kernel<T><<<LIST_BLOCKS, WARPS_PER_BLOCK * 32, 0, st>>>(*plan);
  QSFT_CUDA_CHECK_LAUNCH();
  iter_end_kernel<<<(plan->njobs + 127) / 128, 128, 0, st>>>(*plan);
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
}

static int check_plan(const qsft_plan* p) {
  if (!p || p->njobs <= 0 || !p->jobs || !p->bin_prefix || !p->i8 || !p->U || !p->kbuf || !p->rho ||
      !p->tab_key || !p->tab_best || !p->uniq || !p->ball_tab || !p->ball_k || !p->ball_sum || !p->ball_cnt ||
      !p->ctrl || !p->roots || !p->bin_status || !p->bin_stamp || !p->dirty || !p->cand || !p->done_count)
    return QSFT_ERR_ARG;
  if (p->kstride < 16 || (p->kstride & 15) || p->kstride > QSFT_MAX_N + 16) return QSFT_ERR_ARG;
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
      cudaMemsetAsync(plan->tab_key, 0, sizeof(int64_t) * plan->total_slots, st) != cudaSuccess ||
      cudaMemsetAsync(plan->tab_best, 0, sizeof(int64_t) * plan->total_slots, st) != cudaSuccess ||
      cudaMemsetAsync(plan->ball_tab, 0, sizeof(int32_t) * plan->total_slots, st) != cudaSuccess ||
      cudaMemsetAsync(plan->ball_sum, 0, sizeof(double) * 2 * plan->total_balls, st) != cudaSuccess ||
      cudaMemsetAsync(plan->ball_cnt, 0, sizeof(int32_t) * plan->total_balls, st) != cudaSuccess ||
      cudaMemsetAsync(plan->bin_stamp, 0, sizeof(int32_t) * plan->total_bins, st) != cudaSuccess ||
      cudaMemsetAsync(plan->done_count, 0, sizeof(int32_t), st) != cudaSuccess)
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
  for (int i = 0; i < max_iter; ++i) {
    const int rc = qsft_peel_iteration(plan, i == 0, stream);
    if (rc != QSFT_OK) return rc;
  }
  return QSFT_OK;
}
