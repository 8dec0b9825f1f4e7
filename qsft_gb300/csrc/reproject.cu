// Optional FP64 re-projection of the recovered coefficients against the raw
// bins.
//
// The reference's estimate of a coefficient is the running mean of the
// per-detection projections rho made while peeling (qsft/qsft.py:209-217,
// 247-255): each rho was taken from a bin after the balls peeled before it, so
// it carries their errors and the noise of that one bin.  Here every recovered
// coefficient is re-estimated from the bins as they were before any peeling:
//   1. subtract   every recovered (k, a) from a copy of the raw bins, in every
//                 group l at bin M_l^T k (mod q): raw_l[p][j] -= a omega^<d_p, k>
//   2. project    per recovered k, in FP64: for each group l,
//                 rho_l = a + <omega^(D_l k), raw_l[:, j_l]> / RP
//                 (the residual of its bin with its own contribution put back),
//                 and the new estimate is the mean of rho_l over the C groups.
// Step 2 is exact for a coefficient whose bins hold no other recovered one and
// one Jacobi step of the least-squares fit otherwise.  It changes the values
// the reference returns, so the parity path leaves it off.
#include "common.cuh"

namespace qsft {

constexpr int RP_THREADS = 256;
constexpr int RP_BLOCKS_X = 64;  // blocks per job (grid-stride over the job's rows)

__device__ __forceinline__ double2 rroot(const double* roots, int q, int m) {
  return make_double2(__ldg(roots + (q * 32 + m) * 2), __ldg(roots + (q * 32 + m) * 2 + 1));
}
// <d, k> mod q and M_l^T k (MSB-first digits) for the n-digit k row kr
__device__ __forceinline__ int dot_mod(const int8_t* d, const uint8_t* kr, int n, int q) {
  int s = 0;
  for (int i = 0; i < n; ++i) s += (int)d[i] * (int)kr[i];
  return s % q;
}
__device__ __forceinline__ int bin_of(const int8_t* Ml, const uint8_t* kr, int n, int b, int q) {
  int j = 0;
  for (int t = 0; t < b; ++t) {
    int dg = 0;
    for (int i = 0; i < n; ++i) dg += (int)Ml[i * b + t] * (int)kr[i];
    j = j * q + dg % q;
  }
  return j;
}
__device__ __forceinline__ void sub_c(float2* p, double dx, double dy) {
  asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"((float)-dx), "f"((float)-dy) : "memory");
}
__device__ __forceinline__ void sub_c(double2* p, double dx, double dy) {
  atomicAdd(&p->x, -dx);
  atomicAdd(&p->y, -dy);
}

// 1. per (row of job blockIdx.y, group l): raw_l[:, M_l^T k] -= a omega^(D_l k)
template <typename T>
__global__ void __launch_bounds__(RP_THREADS) reproj_subtract_kernel(qsft_plan plan, c2<T>* raw, const uint8_t* out_k,
                                                                     const double* out_val,
                                                                     const int64_t* out_index) {
  const int jid = blockIdx.y;
  const qsft_job* __restrict__ job = plan.jobs + jid;
  const int q = job->q, n = job->n, b = job->b, C = job->C, RP = job->R * job->P;
  const int64_t B = job->B;
  const int64_t first = out_index[2 * jid], count = out_index[2 * jid + 1];
  const int ks = plan.kstride;
  for (int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; it < count * C;
       it += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = first + it / C;
    const int l = (int)(it % C);
    const uint8_t* kr = out_k + row * ks;
    const double ax = out_val[2 * row], ay = out_val[2 * row + 1];
    const int j = bin_of(plan.i8 + job->off_M + (int64_t)l * n * b, kr, n, b, q);
    const int8_t* Dl = plan.i8 + job->off_D + (int64_t)l * RP * n;
    c2<T>* col = raw + job->off_U + (int64_t)l * RP * B + j;
    for (int p = 0; p < RP; ++p) {
      const double2 w = rroot(plan.roots, q, dot_mod(Dl + (int64_t)p * n, kr, n, q));
      sub_c(col + p * B, ax * w.x - ay * w.y, ax * w.y + ay * w.x);
    }
  }
}

// 2. per row of job blockIdx.y: the mean over the groups of
//    a + <omega^(D_l k), raw_l[:, j_l]> / RP, in FP64
template <typename T>
__global__ void __launch_bounds__(RP_THREADS) reproj_project_kernel(qsft_plan plan, const c2<T>* raw,
                                                                    const uint8_t* out_k, double* out_val,
                                                                    const int64_t* out_index) {
  const int jid = blockIdx.y;
  const qsft_job* __restrict__ job = plan.jobs + jid;
  const int q = job->q, n = job->n, b = job->b, C = job->C, RP = job->R * job->P;
  const int64_t B = job->B;
  const int64_t first = out_index[2 * jid], count = out_index[2 * jid + 1];
  const int ks = plan.kstride;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < count; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = first + r;
    const uint8_t* kr = out_k + row * ks;
    const double ax = out_val[2 * row], ay = out_val[2 * row + 1];
    double sx = 0.0, sy = 0.0;
    for (int l = 0; l < C; ++l) {
      const int j = bin_of(plan.i8 + job->off_M + (int64_t)l * n * b, kr, n, b, q);
      const int8_t* Dl = plan.i8 + job->off_D + (int64_t)l * RP * n;
      const c2<T>* col = raw + job->off_U + (int64_t)l * RP * B + j;
      double px = 0.0, py = 0.0;  // <omega^(D_l k), residual column> = sum conj(w) v
      for (int p = 0; p < RP; ++p) {
        const double2 w = rroot(plan.roots, q, dot_mod(Dl + (int64_t)p * n, kr, n, q));
        const double2 v = to_d2(col[p * B]);
        px += w.x * v.x + w.y * v.y;
        py += w.x * v.y - w.y * v.x;
      }
      sx += ax + px / RP;
      sy += ay + py / RP;
    }
    out_val[2 * row] = sx / C;
    out_val[2 * row + 1] = sy / C;
  }
}

template <typename T>
static int reproject(const qsft_plan* p, void* raw, const uint8_t* out_k, double* out_val, const int64_t* out_index,
                     cudaStream_t st) {
  const dim3 grid(RP_BLOCKS_X, (unsigned)p->njobs);
  reproj_subtract_kernel<T><<<grid, RP_THREADS, 0, st>>>(*p, reinterpret_cast<c2<T>*>(raw), out_k, out_val, out_index);
  QSFT_CUDA_CHECK_LAUNCH();
  reproj_project_kernel<T><<<grid, RP_THREADS, 0, st>>>(*p, reinterpret_cast<const c2<T>*>(raw), out_k, out_val,
                                                        out_index);
  QSFT_CUDA_CHECK_LAUNCH();
  return QSFT_OK;
}

}  // namespace qsft

using namespace qsft;

extern "C" int qsft_reproject(const qsft_plan* plan, void* raw, const uint8_t* out_k, double* out_val,
                              const int64_t* out_index, qsft_stream_t stream) {
  if (!plan || plan->njobs <= 0 || plan->njobs > 65535 || !plan->jobs || !plan->i8 || !plan->roots || !raw || !out_k ||
      !out_val || !out_index)
    return QSFT_ERR_ARG;
  if (plan->kstride < 16 || (plan->kstride & 15)) return QSFT_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (plan->prec == QSFT_F32) return reproject<float>(plan, raw, out_k, out_val, out_index, st);
  if (plan->prec == QSFT_F64) return reproject<double>(plan, raw, out_k, out_val, out_index, st);
  return QSFT_ERR_ARG;
}
