// Peeling of one transform without any device allocation.
//
// Some callers cannot allocate device memory when they run the transform:
// serving threads that must not hit cudaMalloc's implicit device-wide
// synchronisation while other streams are busy, and host applications that
// own every buffer (a fixed memory budget or a pool of their own) and hand a
// library only its inputs and outputs.  For them qsft_peel_noalloc runs
// QSFT.transform's peeling loop for one job with all of its scratch in
// g_scratch below, a statically sized device array that every GPU loading
// this library holds until the process exits.
//
// Limits: C*B <= QSFT_NOALLOC_MAX_BINS bins and k rows of at most
// QSFT_NOALLOC_KSTRIDE bytes (n <= 32; n <= 16 for a coded source).
// Every call shares the array, and it keeps the last call's contents:
// qsft_peel_init clears what must start at zero, and calls that overlap on
// the GPU (different streams, threads or processes' contexts on one device)
// race and corrupt each other's results; serialise them.  The first call on a
// device takes the array's device address (cudaGetSymbolAddress) with that
// device current, so make that first call before any stream capture.  The
// job's control record is copied to the caller's out_ctrl at the end, so a
// table overflow (ctrl.err) reaches the caller like on the workspace path.
#include <mutex>

#include "common.cuh"

namespace qsft {
namespace noalloc {

constexpr int64_t MAX_BINS = QSFT_NOALLOC_MAX_BINS;
constexpr int KSTRIDE = QSFT_NOALLOC_KSTRIDE;
constexpr int64_t MAX_SLOTS = 2 * MAX_BINS;  // next power of two >= 2 * bins
constexpr int64_t MAX_BALLS = MAX_BINS + 64;

constexpr size_t al(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t OFF_JOB = 0;
constexpr size_t OFF_PREFIX = al(OFF_JOB + sizeof(qsft_job));
constexpr size_t OFF_ROOTS = al(OFF_PREFIX + 2 * sizeof(int64_t));
constexpr size_t OFF_INDEX = al(OFF_ROOTS + 33 * 32 * 2 * sizeof(double));
constexpr size_t OFF_CTRL = al(OFF_INDEX + 2 * sizeof(int64_t));
constexpr size_t OFF_DONE = al(OFF_CTRL + sizeof(qsft_ctrl));
constexpr size_t OFF_RHO = al(OFF_DONE + 4 * sizeof(int32_t));
constexpr size_t OFF_BALLTAB = al(OFF_RHO + MAX_BINS * 2 * sizeof(double));
constexpr size_t OFF_BALLBEST = al(OFF_BALLTAB + MAX_SLOTS * sizeof(int64_t));
constexpr size_t OFF_UNIQ = al(OFF_BALLBEST + MAX_BALLS * sizeof(int64_t));
constexpr size_t OFF_BALLK = al(OFF_UNIQ + MAX_BALLS * sizeof(int32_t));
constexpr size_t OFF_BALLSUM = al(OFF_BALLK + MAX_BALLS * KSTRIDE);
constexpr size_t OFF_BALLCNT = al(OFF_BALLSUM + MAX_BALLS * 2 * sizeof(double));
constexpr size_t OFF_STATUS = al(OFF_BALLCNT + MAX_BALLS * sizeof(int32_t));
constexpr size_t OFF_STAMP = al(OFF_STATUS + MAX_BINS);
constexpr size_t OFF_DIRTY = al(OFF_STAMP + MAX_BINS * sizeof(int32_t));
constexpr size_t OFF_CAND = al(OFF_DIRTY + 2 * MAX_BINS * sizeof(int32_t));
constexpr size_t TOTAL = al(OFF_CAND + MAX_BINS * sizeof(int32_t));

// the scratch: held by every GPU that loads the library, shared by every call
static __device__ __align__(256) unsigned char g_scratch[TOTAL];

// per-call set-up inside the scratch: the job record, its bin prefix [0, C*B]
// and the table of roots exp(2 pi i m / q) at (q*32 + m)
__global__ void setup_kernel(qsft_job job, unsigned char* base) {
  if (threadIdx.x == 0) {
    *reinterpret_cast<qsft_job*>(base + OFF_JOB) = job;
    int64_t* pre = reinterpret_cast<int64_t*>(base + OFF_PREFIX);
    pre[0] = 0;
    pre[1] = (int64_t)job.C * job.B;
  }
  double* roots = reinterpret_cast<double*>(base + OFF_ROOTS);
  for (int i = threadIdx.x; i < 33 * 32; i += blockDim.x) {
    const int q = i / 32, m = i % 32;
    double2 w = make_double2(0.0, 0.0);
    if (q >= 2 && m < q) w = root_of_unity(m, q);
    roots[2 * i] = w.x;
    roots[2 * i + 1] = w.y;
  }
}

// device address of g_scratch on the current device, taken once per device
static int scratch_base(unsigned char** out) {
  static std::mutex mu;
  static void* addr[128];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return QSFT_ERR_CUDA;
  if (dev < 0 || dev >= 128) return QSFT_ERR_ARG;
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return QSFT_ERR_CUDA;
    addr[dev] = p;
  }
  *out = static_cast<unsigned char*>(addr[dev]);
  return QSFT_OK;
}

}  // namespace noalloc
}  // namespace qsft

using namespace qsft;
using namespace qsft::noalloc;

extern "C" int qsft_peel_noalloc(int prec, const qsft_job* job_in, const int8_t* i8, void* U,
                                 const int32_t* gf_tables, uint8_t* out_k, double* out_val, int32_t* out_cnt,
                                 int64_t* out_total, int32_t max_out, qsft_ctrl* out_ctrl,
                                 qsft_stream_t stream) {
  if (!job_in || !i8 || !U || !out_k || !out_val || !out_cnt || !out_total || !out_ctrl) return QSFT_ERR_ARG;
  if (prec != QSFT_F32 && prec != QSFT_F64) return QSFT_ERR_ARG;
  qsft_job job = *job_in;
  int64_t bins = 0, slots = 0, balls = 0;
  int32_t ks = 0;
  const int rc0 = qsft_workspace_layout(&job, 1, &bins, &slots, &balls, &ks);
  if (rc0 != QSFT_OK) return rc0;
  if (bins > MAX_BINS || slots > MAX_SLOTS || balls > MAX_BALLS || ks > KSTRIDE) return QSFT_ERR_TOO_LARGE;
  if (max_out < job.ball_cap) return QSFT_ERR_ARG;  // output rows the collection may write
  if (job.src == QSFT_SRC_CODED && !gf_tables) return QSFT_ERR_ARG;
  unsigned char* base = nullptr;
  const int rc1 = scratch_base(&base);
  if (rc1 != QSFT_OK) return rc1;
  cudaStream_t st = (cudaStream_t)stream;
  setup_kernel<<<1, 256, 0, st>>>(job, base);
  QSFT_CUDA_CHECK_LAUNCH();

  qsft_plan p = {};
  p.njobs = 1;
  p.prec = prec;
  p.kstride = KSTRIDE;
  p.total_bins = bins;
  p.total_slots = slots;
  p.total_balls = balls;
  p.max_q = p.min_q = job.q;
  p.max_n = job.n;
  p.all_q_pow2 = (job.q & (job.q - 1)) == 0;
  p.max_rp = job.R * job.P;
  p.jobs = reinterpret_cast<const qsft_job*>(base + OFF_JOB);
  p.bin_prefix = reinterpret_cast<const int64_t*>(base + OFF_PREFIX);
  p.i8 = i8;
  p.U = U;
  p.gf_tables = gf_tables;
  p.roots = reinterpret_cast<const double*>(base + OFF_ROOTS);
  p.rho = reinterpret_cast<double*>(base + OFF_RHO);
  p.ball_tab = reinterpret_cast<int64_t*>(base + OFF_BALLTAB);
  p.ball_best = reinterpret_cast<int64_t*>(base + OFF_BALLBEST);
  p.uniq = reinterpret_cast<int32_t*>(base + OFF_UNIQ);
  p.ball_k = base + OFF_BALLK;
  p.ball_sum = reinterpret_cast<double*>(base + OFF_BALLSUM);
  p.ball_cnt = reinterpret_cast<int32_t*>(base + OFF_BALLCNT);
  p.ctrl = reinterpret_cast<qsft_ctrl*>(base + OFF_CTRL);
  p.bin_status = base + OFF_STATUS;
  p.bin_stamp = reinterpret_cast<int32_t*>(base + OFF_STAMP);
  p.dirty = reinterpret_cast<int32_t*>(base + OFF_DIRTY);
  p.cand = reinterpret_cast<int32_t*>(base + OFF_CAND);
  p.stage = nullptr;  // no staging copies: the decoder reads the candidates' columns from U
  p.done_count = reinterpret_cast<int32_t*>(base + OFF_DONE);

  // qsft_peel_init zeroes everything that must start at zero (control record,
  // hash tables, ball store, stamps, done count); the other regions are
  // written before they are read.
  int rc = qsft_peel_init(&p, stream);
  if (rc != QSFT_OK) return rc;
  rc = qsft_peel_run(&p, job.max_iter, stream);
  if (rc != QSFT_OK) return rc;
  rc = qsft_collect(&p, out_k, out_val, out_cnt, reinterpret_cast<int64_t*>(base + OFF_INDEX), out_total, stream);
  if (rc != QSFT_OK) return rc;
  // the control record (err, iter, n_balls, num_peeling) to the caller: a
  // device-to-device copy on the stream, no allocation
  if (cudaMemcpyAsync(out_ctrl, base + OFF_CTRL, sizeof(qsft_ctrl), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return QSFT_ERR_CUDA;
  return QSFT_OK;
}
