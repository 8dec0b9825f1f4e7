// Singleton detection and peeling: QSFT.transform's while-loop
// (qsft/qsft.py:151-255) for a batch of transforms.
//
// One iteration = three launches:
//   detect_kernel   one thread per bin (group c, bin j) of every active job:
//                   zeroton test, channel decoding of k (noiseless / NSO
//                   "nso1"), optional Reed-Solomon source decoding, FP64
//                   re-projection of the coefficient rho, FP64 residual test,
//                   bin-match test; singletons are deduplicated by k in a
//                   per-iteration hash table (keeping the largest (c, j) as
//                   the reference's dict does) and their rho is added to the
//                   job's result store (the `result` list and its running
//                   mean, qsft/qsft.py:209-217, 247-255).
//   peel_kernel     one warp per distinct k: subtract rho * omega^(D_l k) from
//                   bin M_l^T k (mod q) of every group l (qsft/qsft.py:223-241).
//   iter_end_kernel per job: iteration count, cumulative peel count and the
//                   loop's stopping rules (qsft/qsft.py:151, 204-205).
//
// FP32 data path: bins are stored as float2.  Energy and phase decisions that
// fall within a small band of their thresholds are recomputed in FP64; the
// coefficient projection and residual energy are always computed in FP64.
#include "common.cuh"
#include "rs.cuh"

namespace qsft {

constexpr int DET_THREADS = 128;
constexpr int MAX_SYMS = 256;  // channel symbols per bin (P - 1 <= 256)

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
// compare our row (local) with a row another thread wrote (read through L2)
__device__ __forceinline__ bool row_eq(const uint8_t* mine, const uint8_t* other, int words) {
  const uint32_t* a = reinterpret_cast<const uint32_t*>(mine);
  const uint32_t* b = reinterpret_cast<const uint32_t*>(other);
  for (int i = 0; i < words; ++i)
    if (a[i] != __ldcg(b + i)) return false;
  return true;
}
__device__ __forceinline__ double2 root(const double* roots, int q, int m) {
  return make_double2(roots[(q * 32 + m) * 2], roots[(q * 32 + m) * 2 + 1]);
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

template <typename T>
__device__ __forceinline__ double2 ld_col(const c2<T>* col, int64_t r, int B) {
  return to_d2(col[r * B]);
}

// ---------------------------------------------------------------- detect
template <typename T>
__global__ void __launch_bounds__(DET_THREADS) detect_kernel(qsft_plan plan) {
  const int64_t gb = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool inrange = gb < plan.total_bins;
  const int jid = find_job(plan.bin_prefix, plan.njobs, inrange ? gb : plan.total_bins - 1);
  const qsft_job* __restrict__ job = plan.jobs + jid;
  qsft_ctrl* ctl = plan.ctrl + jid;
  int status = 0;  // 0 zeroton / inactive, 1 multiton, 2 singleton
  const int q = job->q, n = job->n, b = job->b, B = job->B, P = job->P;
  const int RP = job->R * P;
  const int64_t local = gb - job->off_bin;
  const int c = (int)(local / B);
  const int jb = (int)(local - (int64_t)c * B);
  uint8_t kl[QSFT_MAX_N + 16];
  double2 rho = make_double2(0.0, 0.0);
  const bool active = inrange && !ctl->done;
  const c2<T>* col = reinterpret_cast<const c2<T>*>(plan.U) + job->off_U + (int64_t)c * RP * B + jb;
  const double thr = job->cutoff * RP;

  if (active) {
    // zeroton test: ||col||^2 > cutoff * len(col)   (qsft/qsft.py:164)
    T e = 0;
    for (int r = 0; r < RP; ++r) {
      const c2<T> v = col[(int64_t)r * B];
      e += v.x * v.x + v.y * v.y;
    }
    double E = (double)e;
    if (sizeof(T) == 4 && fabs(E - thr) <= 1e-3 * thr) {
      E = 0.0;
      for (int r = 0; r < RP; ++r) {
        const double2 v = ld_col<T>(col, r, B);
        E += v.x * v.x + v.y * v.y;
      }
    }
    if (E > thr) {
      // ---- channel decoding (qsft/reconstruct.py:12-31, 100-113)
      uint8_t syms[MAX_SYMS];
      const int nsym = P - 1;
      if (job->chan == QSFT_CHAN_IDENTITY) {
        const double2 v0 = ld_col<T>(col, 0, B);
        const T a0 = atan2((T)v0.y, (T)v0.x);
        for (int i = 1; i < RP && i <= nsym; ++i) {
          const double2 vi = ld_col<T>(col, i, B);
          const T ai = atan2((T)vi.y, (T)vi.x);
          double a = (double)((T)q * (ai - a0) / (T)6.283185307179586);
          double fr = a - floor(a);
          if (sizeof(T) == 4 && fabs(fr - 0.5) < 1e-3) {
            a = (double)q * (atan2(vi.y, vi.x) - atan2(v0.y, v0.x)) / 6.283185307179586;
          }
          long long m = (long long)rint(a);  // round half to even, like np.round
          m %= q;
          if (m < 0) m += q;
          syms[i - 1] = (uint8_t)m;
        }
      } else {
        const int R = job->R;
        for (int i = 1; i <= nsym; ++i) {
          T zr = 0, zi = 0;
          for (int r = 0; r < R; ++r) {
            const c2<T> u0 = col[(int64_t)(r * P) * B];
            const c2<T> ui = col[(int64_t)(r * P + i) * B];
            zr += u0.x * ui.x + u0.y * ui.y;
            zi += u0.y * ui.x - u0.x * ui.y;
          }
          double ang = (double)atan2(zi, zr);
          if (ang < 0) ang += 6.283185307179586;
          double tq = ang * q / 6.283185307179586;
          if (sizeof(T) == 4 && fabs(tq - floor(tq) - 0.5) < 1e-3) {
            double dzr = 0, dzi = 0;
            for (int r = 0; r < R; ++r) {
              const double2 u0 = ld_col<T>(col, (int64_t)r * P, B);
              const double2 ui = ld_col<T>(col, (int64_t)r * P + i, B);
              dzr += u0.x * ui.x + u0.y * ui.y;
              dzi += u0.y * ui.x - u0.x * ui.y;
            }
            ang = atan2(dzi, dzr);
            if (ang < 0) ang += 6.283185307179586;
          }
          syms[i - 1] = (uint8_t)nearest_root(ang, q);
        }
      }
      // ---- source decoding
      if (job->src == QSFT_SRC_CODED) {
        const GFt g = make_gf(plan.gf_tables + job->rs_gf_off, q, job->rs_s);
        rs_decode(g, q, job->rs_s, job->rs_t, n, syms, kl);
      } else {
        for (int i = 0; i < n; ++i) kl[i] = syms[i];
      }
      for (int i = n; i < plan.kstride && i < QSFT_MAX_N + 16; ++i) kl[i] = 0;
      // ---- FP64 projection rho = <sig, col> / len, residual, bin match (qsft/qsft.py:174-183)
      const int8_t* Dc = plan.i8 + job->off_D + (int64_t)c * RP * n;
      double ar = 0, ai = 0;
      for (int r = 0; r < RP; ++r) {
        const int8_t* dr = Dc + (int64_t)r * n;
        int ph = 0;
        for (int i = 0; i < n; ++i) ph += (int)dr[i] * (int)kl[i];
        const double2 w = root(plan.roots, q, ph % q);
        const double2 v = ld_col<T>(col, r, B);
        ar += w.x * v.x + w.y * v.y;
        ai += w.x * v.y - w.y * v.x;
      }
      rho = make_double2(ar / RP, ai / RP);
      double res = 0;
      for (int r = 0; r < RP; ++r) {
        const int8_t* dr = Dc + (int64_t)r * n;
        int ph = 0;
        for (int i = 0; i < n; ++i) ph += (int)dr[i] * (int)kl[i];
        const double2 w = root(plan.roots, q, ph % q);
        const double2 v = ld_col<T>(col, r, B);
        const double dx = v.x - (rho.x * w.x - rho.y * w.y);
        const double dy = v.y - (rho.x * w.y + rho.y * w.x);
        res += dx * dx + dy * dy;
      }
      bool match = true;
      const int8_t* Mc = plan.i8 + job->off_M + (int64_t)c * n * b;
      int jr = jb;
      for (int t = b - 1; t >= 0; --t) {
        int dg = 0;
        for (int i = 0; i < n; ++i) dg += (int)Mc[i * b + t] * (int)kl[i];
        match &= (dg % q) == (jr % q);
        jr /= q;
      }
      status = (match && !(res > thr)) ? 2 : 1;
    }
  }

  // ---- per-job counters, aggregated per warp
  {
    const unsigned full = 0xffffffffu;
    const unsigned peers = __match_any_sync(full, jid);
    const unsigned singles = __ballot_sync(full, status == 2) & peers;
    const unsigned multis = __ballot_sync(full, status == 1) & peers;
    const int lane = threadIdx.x & 31;
    if (lane == __ffs(peers) - 1) {
      if (singles) atomicAdd(&ctl->n_single, __popc(singles));
      if (multis) atomicAdd(&ctl->n_multi, __popc(multis));
    }
  }
  if (status != 2) return;

  // ---- record the singleton: k row, rho
  const int ks = plan.kstride;
  const int words = ks / 4;
  uint8_t* krow = plan.kbuf + gb * ks;
  for (int w = 0; w < words; ++w) reinterpret_cast<uint32_t*>(krow)[w] = reinterpret_cast<const uint32_t*>(kl)[w];
  plan.rho[2 * gb] = rho.x;
  plan.rho[2 * gb + 1] = rho.y;
  __threadfence();
  const uint32_t h = hash_row(kl, words);
  const int64_t cap = job->table_cap;
  const int64_t mask = cap - 1;

  // ---- dedupe by k for this iteration (balls_to_peel / ball_values, qsft/qsft.py:209-216)
  const long long iter = (long long)ctl->iter + 1;
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
    return;
  }
  if (owner) {
    const int u = atomicAdd(&ctl->n_unique, 1);
    plan.uniq[job->off_slot + u] = (int32_t)slot;
  }
  atomicMax(reinterpret_cast<unsigned long long*>(plan.tab_best + job->off_slot + slot),
            (unsigned long long)(stamp | local));

  // ---- add rho to the result store (result list + running mean, qsft/qsft.py:217, 247-255)
  int32_t* bt = plan.ball_tab + job->off_slot;
  int64_t s2 = h & mask;
  int myid = -1, bid = -1;
  for (int64_t probe = 0; probe < cap; ++probe) {
    int cur = atomicAdd(bt + s2, 0);
    if (cur == 0) {
      if (myid < 0) {
        myid = atomicAdd(&ctl->n_balls, 1);
        if (myid >= job->ball_cap) {
          atomicExch(&ctl->err, (int)QSFT_ERR_OVERFLOW);
          return;
        }
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
    return;
  }
  atomicAdd(plan.ball_sum + 2 * (job->off_ball + bid), rho.x);
  atomicAdd(plan.ball_sum + 2 * (job->off_ball + bid) + 1, rho.y);
  atomicAdd(plan.ball_cnt + job->off_ball + bid, 1);
}

// ---------------------------------------------------------------- peel
template <typename T>
__global__ void __launch_bounds__(256) peel_kernel(qsft_plan plan) {
  __shared__ uint8_t sk[8][QSFT_MAX_N];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int gw = blockIdx.x * 8 + wib;
  const int nw = gridDim.x * 8;
  for (int jid = 0; jid < plan.njobs; ++jid) {
    const qsft_ctrl* ctl = plan.ctrl + jid;
    if (ctl->done) continue;
    const int cnt = ctl->n_unique;
    if (gw >= cnt) continue;
    const qsft_job* __restrict__ job = plan.jobs + jid;
    const int q = job->q, n = job->n, b = job->b, B = job->B, C = job->C;
    const int RP = job->R * job->P;
    for (int u = gw; u < cnt; u += nw) {
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
      }
      __syncwarp();
    }
  }
}

__global__ void iter_end_kernel(qsft_plan plan) {
  const int jid = blockIdx.x * blockDim.x + threadIdx.x;
  if (jid >= plan.njobs) return;
  qsft_ctrl* ctl = plan.ctrl + jid;
  const qsft_job* job = plan.jobs + jid;
  if (ctl->done) return;
  ctl->iter += 1;
  ctl->num_peeling += ctl->n_unique;
  if (ctl->n_multi == 0 || ctl->n_single == 0 || ctl->iter >= job->max_iter ||
      ctl->num_peeling >= job->peeling_max || ctl->err != 0)
    ctl->done = 1;
  ctl->n_single = 0;
  ctl->n_multi = 0;
  ctl->n_unique = 0;
}

template <typename T>
static int iteration(const qsft_plan* plan, cudaStream_t st) {
  const int64_t grid = (plan->total_bins + DET_THREADS - 1) / DET_THREADS;
  if (grid > 0x7fffffffLL) return QSFT_ERR_TOO_LARGE;
  detect_kernel<T><<<(unsigned)grid, DET_THREADS, 0, st>>>(*plan);
  QSFT_CUDA_CHECK_LAUNCH();
  peel_kernel<T><<<152 * 4, 256, 0, st>>>(*plan);
  QSFT_CUDA_CHECK_LAUNCH();
  iter_end_kernel<<<(plan->njobs + 127) / 128, 128, 0, st>>>(*plan);
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
}

static int check_plan(const qsft_plan* p) {
  if (!p || p->njobs <= 0 || !p->jobs || !p->bin_prefix || !p->i8 || !p->U || !p->kbuf || !p->rho ||
      !p->tab_key || !p->tab_best || !p->uniq || !p->ball_tab || !p->ball_k || !p->ball_sum || !p->ball_cnt ||
      !p->ctrl || !p->roots)
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
      cudaMemsetAsync(plan->ball_cnt, 0, sizeof(int32_t) * plan->total_balls, st) != cudaSuccess)
    return QSFT_ERR_CUDA;
  return QSFT_OK;
}

extern "C" int qsft_peel_iteration(const qsft_plan* plan, qsft_stream_t stream) {
  const int rc = check_plan(plan);
  if (rc != QSFT_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  return plan->prec == QSFT_F32 ? iteration<float>(plan, st) : iteration<double>(plan, st);
}

extern "C" int qsft_peel_run(const qsft_plan* plan, int max_iter, qsft_stream_t stream) {
  if (max_iter < 0) return QSFT_ERR_ARG;
  for (int i = 0; i < max_iter; ++i) {
    const int rc = qsft_peel_iteration(plan, stream);
    if (rc != QSFT_OK) return rc;
  }
  return QSFT_OK;
}
