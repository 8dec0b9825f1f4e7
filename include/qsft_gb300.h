/*
 * qsft_gb300.h -- C ABI of the GB300 (sm_103a) q-SFT hot path.
 *
 * The reference (basics-lab/qsft) is a Python package whose hot path is:
 *   coset query generation + function evaluation  (SubsampledSignal._subsample_qsft,
 *       qsft/input_signal_subsampled.py:107-155,183-206; SyntheticSubsampledSignal
 *       .subsample / sampling_function, synt_exp/synt_src/synthetic_signal.py:100-118)
 *   q^b-point GWHT per (group, delay)              (qsft/utils.py:31-36; :264-266)
 *   bin-domain AWGN                                (synthetic_signal.py:120-130)
 *   singleton detection + peeling                  (qsft/qsft.py:151-255;
 *       qsft/reconstruct.py:12-168; qsft/ReedSolomon.py:26-48)
 * Each entry point below replaces one of those steps.  All entry points take
 * plain device pointers and sizes (no framework types), run on the caller's
 * CUDA stream, never synchronise, never allocate, and return a qsft_status.
 * Every buffer is owned by the caller; qsft_workspace_layout() tells the
 * caller how large the scratch regions must be.
 *
 * Batching: a call processes a batch of independent transform "jobs" that may
 * have different shapes (q, n, b, C, R, P, S).  Jobs are described by an array
 * of qsft_job records in device memory; packed operand arrays are addressed by
 * the per-job offsets.  A batch of one job is the plain single-transform case.
 */
#ifndef QSFT_GB300_H
#define QSFT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void* qsft_stream_t; /* a cudaStream_t (0 = legacy default stream) */

typedef enum {
  QSFT_OK = 0,
  QSFT_ERR_ARG = -1,          /* bad shape / null pointer / unsupported parameter  */
  QSFT_ERR_CUDA = -2,         /* a CUDA launch or runtime call failed               */
  QSFT_ERR_TOO_LARGE = -3,    /* a shape exceeds a compiled limit (see QSFT_MAX_*)  */
  QSFT_ERR_OVERFLOW = -4,     /* a device table overflowed (reported via qsft_ctrl) */
  QSFT_ERR_TIMEOUT = -5       /* a bounded device wait gave up (reported via status) */
} qsft_status;

/* compiled limits */
#define QSFT_MAX_Q 32         /* alphabet size q (2..32)                              */
#define QSFT_MAX_N 128        /* query length n                                       */
#define QSFT_MAX_RS_T 16      /* Reed-Solomon correction radius t                     */
#define QSFT_MAX_GF 4096      /* order q^s of the RS symbol field                      */

/* qsft_eval_cosets works in tiles of this many samples of a job's C*R*P*B
 * flattened samples; qsft_plan.eval_prefix counts these tiles               */
#define QSFT_EVAL_TILE 1024

/* precision of the complex data (float2 / double2 interleaved re,im) */
#define QSFT_F32 4
#define QSFT_F64 8

/* channel / source decoding methods (QSFT reconstruct_method_channel / _source) */
#define QSFT_CHAN_IDENTITY 0  /* noiseless [0;I] delays, qsft/reconstruct.py:12-31       */
#define QSFT_CHAN_NSO 1       /* NSO soft decoding "nso1", qsft/reconstruct.py:100-113   */
#define QSFT_SRC_IDENTITY 0
#define QSFT_SRC_CODED 1      /* Reed-Solomon syndrome source code, reconstruct.py:34-51 */

/*
 * One transform.  Offsets are in ELEMENTS of the packed array they index.
 *   M  (int8,  C x n x b, row-major per group)      -- Ms after get_MDU's permutation
 *   D  (int8,  C x RP x n; RP = R*P, repeat-major)   -- np.vstack(Ds[c]) per group
 *   K  (int8,  S x n)                                -- support k_s (synthetic signal)
 *   A  (complex, S)                                  -- coefficients a_s
 *   U  (complex, C x RP x B)                         -- samples, then bins
 * The peeling workspace of a job starts at off_bin (bins), off_slot (hash
 * slots) and off_ball (result balls) in the workspace arrays.
 */
typedef struct qsft_job {
  int32_t q, n, b, C;
  int32_t R, P, S, B;          /* B = q^b bins per row                              */
  int32_t chan, src;           /* QSFT_CHAN_*, QSFT_SRC_*                           */
  int32_t rs_s, rs_t;          /* RS: symbol field GF(q^s), radius t                */
  int32_t rs_gf_off;           /* offset of this job's GF tables in gf_tables       */
  int32_t max_iter;            /* peeling iteration cap (15 in the reference)       */
  int32_t table_cap;           /* hash slots, power of two, >= 2*C*B                */
  int32_t ball_cap;            /* capacity of the result ball store                 */
  double cutoff;               /* energy threshold per bin entry (x RP)             */
  int64_t peeling_max;         /* min(q^n, 2^62)                                    */
  int64_t off_M, off_D, off_K, off_A, off_U;
  int64_t off_bin, off_slot, off_ball;
  uint64_t noise_seed;         /* device-noise key (qsft_add_noise_philox)          */
  double noise_nu;             /* per-component noise sigma (0 = none)              */
} qsft_job;

/* per-job peeling state, device resident (zeroed by qsft_peel_init) */
typedef struct qsft_ctrl {
  int32_t done;                /* 1 once the reference's while-loop would exit      */
  int32_t iter;                /* iterations run                                    */
  int32_t n_single;            /* singletons found in the current iteration         */
  int32_t n_multi;             /* multitons among all bins (kept up to date)        */
  int32_t n_unique;            /* distinct balls peeled in the current iteration    */
  int32_t n_balls;             /* distinct balls recorded so far (result size)      */
  int32_t err;                 /* QSFT_ERR_OVERFLOW when a table filled up          */
  int32_t n_cand;              /* bins above the energy cutoff in this iteration    */
  int32_t n_dirty[2];          /* bins changed by the peel of an iteration (parity) */
  int64_t num_peeling;         /* cumulative balls peeled                           */
} qsft_ctrl;

/*
 * Everything a batched call needs.  All pointers are device pointers.  The
 * struct itself lives in host memory and is passed by pointer.
 */
typedef struct qsft_plan {
  int32_t njobs;
  int32_t prec;                /* QSFT_F32 or QSFT_F64                              */
  int32_t kstride;             /* bytes per k row in ball_k and the outputs (>= n;
                                * >= 2n with a coded source, qsft_workspace_layout) */
  int32_t flags;               /* QSFT_PLAN_* bits                                  */
  int64_t total_bins;          /* sum of C*B over jobs                              */
  int64_t total_slots;         /* sum of table_cap over jobs                        */
  int64_t total_balls;         /* sum of ball_cap over jobs                         */
  int64_t total_eval_tiles;    /* eval_prefix[njobs]                                */
  int32_t max_q, max_n;        /* largest q and n over the jobs (launch sizing)     */
  int32_t all_q_pow2;          /* 1 when every job's q is a power of two            */
  int32_t max_rp;              /* largest R*P over the jobs                         */
  const qsft_job* jobs;        /* [njobs]                                           */
  const int64_t* eval_prefix;  /* [njobs+1] cumulative evaluation tiles             */
  const int64_t* bin_prefix;   /* [njobs+1] cumulative C*B (== jobs[i].off_bin)     */
  const int8_t* i8;            /* packed M, D, K                                    */
  const void* A;               /* packed coefficients                               */
  void* U;                     /* packed samples / bins                             */
  const int32_t* gf_tables;    /* RS: exp | log | zech tables per field             */
  const double* roots;         /* exp(2 pi i m / q) at ((q*32 + m)*2), q <= 32      */
  /* peeling workspace (sizes from qsft_workspace_layout) */
  double* rho;                 /* [total_bins * 2]   FP64 coefficient per singleton bin */
  /* persistent hash table k -> ball: (tag << 32) | (ball id + 1), tag a
   * nonzero 32-bit hash of k, so that probes compare k rows only on a tag hit */
  int64_t* ball_tab;           /* [total_slots]                                     */
  /* (iteration << 32) | largest local bin among the iteration's detections of
   * the ball: no clearing between iterations, and the atomicMax that records
   * a detection also tells whether it is the ball's first in the iteration   */
  int64_t* ball_best;          /* [total_balls]                                     */
  int32_t* uniq;               /* [total_balls]  balls detected in this iteration   */
  uint8_t* ball_k;             /* [total_balls * kstride]                           */
  double* ball_sum;            /* [total_balls * 2]                                 */
  int32_t* ball_cnt;           /* [total_balls]                                     */
  qsft_ctrl* ctrl;             /* [njobs]                                           */
  uint8_t* bin_status;         /* [total_bins] 0 zeroton, 1 multiton, 2 singleton  */
  int32_t* bin_stamp;          /* [total_bins] last iteration that changed the bin  */
  int32_t* dirty;              /* [2 * total_bins] changed bins, by iteration parity */
  int32_t* cand;               /* [total_bins] bins above the energy cutoff in this
                                * iteration, job j's list at jobs[j].off_bin       */
  /* staged copies of the candidates' columns, for the decoder: job j owns the
   * columns [bin_prefix[j] / 8, bin_prefix[j+1] / 8) of stage_rp complex values
   * (prec); candidates beyond that share, or jobs with R*P > stage_rp, are read
   * from U.  NULL: no staging.                                                  */
  void* stage;                 /* [(total_bins / 8) * stage_rp] complex             */
  int32_t* done_count;         /* [4]: [0] jobs whose loop has ended (the peeling
                                * kernels exit at once when it reaches njobs);
                                * [1] blocks of the running peel launch that have
                                * finished (the last one closes the iteration);
                                * [2], [3] the grid barrier of qsft_peel_persistent */
  /* tensor-core evaluation (FP32 plans): work items are (job, support chunk of
   * tc_smax entries, group of QSFT_TC_TILES tiles of 128 samples)              */
  const int64_t* tc_prefix;    /* [njobs+1] cumulative work items, or NULL          */
  int64_t total_tc_work;       /* tc_prefix[njobs]                                  */
  int32_t tc_smax;             /* support entries per chunk                         */
  int32_t tc_npad;             /* K extent: max n rounded up to 32, 64 or 128       */
  int32_t min_q;               /* smallest q over the jobs                          */
  int32_t tc_table_bytes;      /* max over jobs of C*b*q*tc_npad + C*R*P*tc_npad    */
  int32_t tc_entry_bytes;      /* shared-memory table bytes per support entry:
                                * q*q*4 when every job has the same q in {2, 4}
                                * (pair table), else max_q*8                        */
  int32_t stage_rp;            /* column length of `stage` (1..64; min(max R*P, 64)) */
  int32_t* status;             /* [1] device word, 0 = ok, else a qsft_status       */
  /* coset-factored tensor-core evaluation (qsft_eval_cosets_gemm); the gm_*
   * sizes and counts are filled in by qsft_gemm_layout                         */
  void* gm_ws;                 /* operand workspace of gm_ws_bytes                  */
  const int64_t* gm_index;     /* [3*njobs+2]: work-unit prefix [njobs+1] |
                                * operand-block prefix [njobs+1] | byte offset of
                                * each job's region in gm_ws [njobs]                */
  int64_t total_gm_work;       /* work units of the GEMM kernel (job, group, chunk
                                * of delay rows, block of gm_mt*128 rows)           */
  int64_t total_gm_prep;       /* blocks of the operand kernel                      */
  int64_t gm_ws_bytes;
  int32_t gm_mt;               /* 128-row MMA tiles per work unit (1 or 2)          */
  int32_t gm_kps;              /* K entries per support vector: 2 when every q is 2
                                * or 4 (exact FP16 characters), else 4             */
  int32_t gm_nw;               /* 32-bit words of packed b-digit vectors (1, 2, 4)  */
  int32_t gm_npmax;            /* largest N extent: 4 columns per delay row of a
                                * chunk (<= 56 rows, equal chunks), rounded to 16   */
  int32_t gm_jt_bytes;         /* shared-memory bytes of the largest group table    */
  int32_t gm_nacc;             /* accumulator buffers in tensor memory (1 or 2)     */
} qsft_plan;

/* tiles of 128 samples per tensor-core work item */
#define QSFT_TC_TILES 16

#define QSFT_PLAN_DETERMINISTIC 1  /* reserved */
/* test only: the grid barriers of qsft_peel_persistent wait for one block more
 * than the grid has, so that their bounded wait runs out and reports
 * QSFT_ERR_TIMEOUT in plan->status (the failure path, without a GPU fault) */
#define QSFT_PLAN_TEST_BARRIER_TIMEOUT 2

/* ---- library ---------------------------------------------------------- */
int qsft_abi_version(void);                 /* returns 1 */
const char* qsft_status_string(int status);
/* device architecture the library was built for, e.g. 103 */
int qsft_built_arch(void);
/* number of kernels this library has launched in this process (all threads) */
int64_t qsft_launch_count(void);

/* ---- query generation + evaluation ------------------------------------- */
/*
 * Replaces SubsampledSignal._subsample_qsft's sampling of every coset
 * (qsft/input_signal_subsampled.py:119-149) with the synthetic evaluation of
 * SyntheticSubsampledSignal.sampling_function (synthetic_signal.py:100-102):
 * U[c][r*P+p][l] = sum_s a_s * omega^(<(M_c l + d_{r,p}) mod q, k_s> mod q),
 * omega = exp(2 pi i / q), l enumerated MSB-first (qsft/utils.py:107-108).
 * Query points are never converted to decimal indices.
 */
int qsft_eval_cosets(const qsft_plan* plan, qsft_stream_t stream);
/*
 * Same result as qsft_eval_cosets for FP32 plans, with the integer dot
 * products <x, k_s> computed by the 5th-generation tensor cores
 * (tcgen05.mma kind::f16: digits are exact in FP16 and the sums exact in the
 * FP32 accumulator) into tensor memory; CUDA cores then reduce
 * a_s * omega^(dot mod q).  Needs plan->tc_prefix / tc_smax / tc_npad, and U
 * zeroed beforehand: partial sums (two column halves per sample, and one per
 * support chunk) are added into U with vector reductions.
 */
int qsft_eval_cosets_tc(const qsft_plan* plan, qsft_stream_t stream);

/*
 * Same result as qsft_eval_cosets for FP32 plans, computed as one complex GEMM
 * per (job, group) on the tensor cores.  With x = M_c l + d and
 * j_s = M_c^T k_s (mod q),
 *   U[c][rp][l] = sum_s omega^(<l, j_s>) * (a_s omega^(<d_rp, k_s>))
 *               = (W C)[l][rp],
 * W the q^b x S character matrix of the j_s (exact in FP16 for q in {2, 4};
 * hi + lo FP16 halves otherwise) and C the S x R*P coefficient matrix (hi + lo
 * FP16 halves of a per-job power-of-two scaling, as separate N columns).  An operand kernel builds C
 * and the j_s into gm_ws; the persistent GEMM kernel (one CTA per SM) generates
 * W tiles in tensor memory and runs tcgen05.mma kind::f16 into tensor-memory
 * accumulators.  U needs no zeroing.
 * Needs the plan's gm_* fields from qsft_gemm_layout.
 */
int qsft_eval_cosets_gemm(const qsft_plan* plan, qsft_stream_t stream);
/*
 * Host-side sizing for qsft_eval_cosets_gemm: from the jobs' shapes (q, n, b,
 * C, R, P, S, B), fills plan->gm_mt, gm_nacc, gm_kps, gm_nw, gm_npmax,
 * gm_jt_bytes, total_gm_work, total_gm_prep, gm_ws_bytes and
 * index_host[3*njobs+2] (to be uploaded to plan->gm_index).  A plan->gm_mt of 1
 * on entry caps the 128-row tiles per work unit (default 2), a plan->gm_nacc of
 * 1 keeps a single accumulator buffer (default: two when tensor memory allows).  QSFT_ERR_TOO_LARGE when a job is outside the
 * kernel's limits (q > 32, b > 16, R*P > 128, S > 8192): use
 * qsft_eval_cosets_tc for such batches.
 */
int qsft_gemm_layout(const qsft_job* jobs_host, int njobs, qsft_plan* plan, int64_t* index_host);

/*
 * Replaces SyntheticSubsampledSignal.subsample(query_indices)
 * (synthetic_signal.py:108-118) for arbitrary query points given as q-ary
 * digit rows X (npoints x n, int8, MSB-first like dec_to_qary_vec,
 * qsft/utils.py:79-84).  out[i] = sum_s a_s omega^(<X_i, k_s> mod q).
 */
int qsft_eval_points(int prec, int q, int n, int S, const int8_t* X, int64_t npoints,
                     const int8_t* K, const void* A, void* out, qsft_stream_t stream);

/* ---- GWHT --------------------------------------------------------------- */
/*
 * Replaces gwht(x, q, b) = fftn(reshape(x,[q]*b)) / q^b (qsft/utils.py:31-36)
 * as applied by _compute_subtransform (qsft/input_signal_subsampled.py:264-266),
 * in place, on nrows rows of q^b complex values starting at data + row_off[i]
 * (element offsets, device array).
 */
int qsft_gwht(int prec, int q, int b, void* data, const int64_t* row_off, int64_t nrows,
              qsft_stream_t stream);

/*
 * qsft_gwht over rows of plan->U (row_off as for qsft_gwht) with the device bin
 * noise of qsft_add_noise_philox for those rows added in the transform's last
 * pass, for every shape (the row kernel draws once per entry pair, the other
 * kernels once per entry; the values are those of the separate noise pass):
 * no extra read and write of the bins.  row_meta[2i], row_meta[2i+1] = the job
 * of row i and the row's index within that job (c*R*P + r*P + p).  Jobs with
 * noise_nu = 0 get the plain transform.
 */
int qsft_gwht_noise(const qsft_plan* plan, int q, int b, const int64_t* row_off, const int32_t* row_meta,
                    int64_t nrows, qsft_stream_t stream);

/*
 * GWHT schedules: the kernels that can transform rows of one (q, b) shape.
 *   QSFT_GWHT_ROW           q in {2, 4}, q^b = 2^8..2^14 (FP64 2^13): a CTA per
 *                           row, whole row in shared memory
 *   QSFT_GWHT_ROWC          q in {2, 4}, q^b = 2^13..2^15: a thread-block
 *                           cluster of 4096-value slices per row, the top bits
 *                           across the cluster through distributed shared memory
 *   QSFT_GWHT_CLUSTER       rows above 48 KB whose q^k-way split fits 64 KB per
 *                           CTA (q^k <= 8): any q, radix-q passes per slice
 *   QSFT_GWHT_PASSES        tile passes through global memory, tiles up to 200 KB
 *   QSFT_GWHT_PASSES_SMALL  the same with tiles up to 48 KB (more CTAs per SM),
 *                           for rows above 48 KB
 * Every schedule gives the same transform (and the same fused noise values).
 * qsft_gwht and qsft_gwht_noise use the schedule selected for the shape and
 * precision (process-wide, all devices), else the built-in rule (the first
 * valid of ROWC, ROW, CLUSTER, PASSES).  No counterpart in the reference,
 * whose gwht is scipy's fftn: this is the GWHT schedule choice the batched
 * path makes, normally from a timing of every valid schedule on the device
 * (qsft_gb300/autotune.py).
 */
#define QSFT_GWHT_AUTO 0
#define QSFT_GWHT_ROW 1
#define QSFT_GWHT_ROWC 2
#define QSFT_GWHT_CLUSTER 3
#define QSFT_GWHT_PASSES 4
#define QSFT_GWHT_PASSES_SMALL 5
/* the valid schedules of a shape: their count, the first max_ids written to ids */
int qsft_gwht_schedules(int prec, int q, int b, int32_t* ids, int max_ids);
/* select `schedule` (or QSFT_GWHT_AUTO: the built-in rule) for a shape;
 * QSFT_ERR_ARG when it is not valid for the shape */
int qsft_gwht_select(int prec, int q, int b, int schedule);
/* the schedule qsft_gwht and qsft_gwht_noise use for a shape now */
int qsft_gwht_selected(int prec, int q, int b);

/* ---- bin noise ---------------------------------------------------------- */
/*
 * Replaces the bin-domain AWGN of SyntheticSubsampledSignal.get_MDU
 * (synthetic_signal.py:126-129): U += N(0, nu^2) + i N(0, nu^2) per entry,
 * nu = jobs[j].noise_nu, drawn from a counter-based Philox-4x32-10 stream keyed
 * by jobs[j].noise_seed: draw row*half + e (half = ceil(q^b / 2)) gives entries
 * e and e + half of the job's row `row` (not numpy's stream: for
 * reference-identical noise the host draws it and adds it with qsft_add_bins).
 */
int qsft_add_noise_philox(const qsft_plan* plan, qsft_stream_t stream);
/* U[i] += X[i] for count complex values (host-drawn noise, uploaded) */
int qsft_add_bins(int prec, void* U, const void* X, int64_t count, qsft_stream_t stream);

/* ---- peeling ------------------------------------------------------------ */
/* zero ctrl, the result ball store and its index (start of QSFT.transform) */
int qsft_peel_init(const qsft_plan* plan, qsft_stream_t stream);
/*
 * One iteration of QSFT.transform's while-loop (qsft/qsft.py:151-241) for every
 * job not yet done: classify every bin of every group as zero/single/multiton
 * (qsft/qsft.py:162-193 with singleton_detection, qsft/reconstruct.py:132-168),
 * record each singleton's coefficient (the `result` list, :209-217), dedupe
 * singletons by k keeping the coefficient of the last (group, bin) in
 * (i, j) order (`ball_values`, :216), subtract every ball from every group
 * (:223-241), and apply the loop's stopping rules (:151, :204-205).
 * `first` = 1 for the first iteration after qsft_peel_init (every bin is
 * classified); later iterations re-classify only the bins the previous
 * iteration's subtractions changed -- the others keep their class, which is a
 * function of the bin's unchanged values, so the outcome is the same.
 */
int qsft_peel_iteration(const qsft_plan* plan, int first, qsft_stream_t stream);
/* kernels one peeling iteration launches (scan: zeroton test; decode: decoding
 * and recording of singletons; peel: subtraction and the iteration's end) */
#define QSFT_PEEL_LAUNCHES_PER_ITER 3
/*
 * Up to max_iter iterations.  Issued eagerly, all max_iter are launched
 * (iterations of finished jobs are no-ops).  Inside a stream capture,
 * iteration 1 is captured and iterations 2.. become one conditional WHILE
 * node of the graph whose body runs only while some job is still in its loop
 * (the condition is set on the device at the end of every iteration).
 */
int qsft_peel_run(const qsft_plan* plan, int max_iter, qsft_stream_t stream);
/*
 * The same loop as one persistent cooperative launch: every block of a grid
 * the GPU holds at once runs an iteration's scan, decode and peel phases in
 * turn, with grid-wide barriers between them, and block 0 applies the
 * stopping rules; the loop ends on the device when every job has left it (or
 * after max_iter iterations).  No graph node per iteration, no launch between
 * phases.  Each barrier wait is bounded (2 s): when it runs out the kernel
 * records QSFT_ERR_TIMEOUT in plan->status (required) and returns.
 */
int qsft_peel_persistent(const qsft_plan* plan, int max_iter, qsft_stream_t stream);

/*
 * Gather the result of QSFT.transform for every job: the distinct k recorded
 * by the peeling loop and the mean of their coefficients (the `gwht` dict,
 * qsft/qsft.py:247-255).  Results of job j are written contiguously:
 * out_index[2j] = first row, out_index[2j+1] = count; rows hold k in
 * out_k[row*kstride ..] (n bytes used), the mean in out_val[2*row .. 2*row+1]
 * and the number of singleton detections averaged in out_cnt[row].  For a
 * job with a coded source, k entry i is out_k[.. + i] + q * out_k[.. + n + i]:
 * the reference keeps a decoded error value outside GF(q) as an entry >= q
 * (see qsft_rs_decode); every other job has zeros there.
 * *out_total (device int64) receives the row count (the call zeroes it first).
 * Output capacity: plan->total_balls rows.
 */
int qsft_collect(const qsft_plan* plan, uint8_t* out_k, double* out_val, int32_t* out_cnt,
                 int64_t* out_index, int64_t* out_total, qsft_stream_t stream);

/*
 * Optional FP64 re-projection of every coefficient qsft_collect wrote.  No
 * counterpart in the reference, whose estimate is the running mean of the
 * peeling's per-detection projections (qsft/qsft.py:209-217, 247-255): here
 * every recovered (k, a) is first subtracted from `raw` (a copy of the bins
 * taken before qsft_peel_init, same layout as plan->U, used as scratch), then
 * each coefficient becomes the mean over the C groups of
 * a + <omega^(D_l k), raw_l[:, M_l^T k]> / RP, computed in FP64: the
 * projection against the raw samples with every other recovered coefficient
 * removed.  out_k / out_index as qsft_collect wrote them; out_val is
 * overwritten.  It changes the values the reference returns: the parity path
 * leaves it off.
 */
int qsft_reproject(const qsft_plan* plan, void* raw, const uint8_t* out_k, double* out_val,
                   const int64_t* out_index, qsft_stream_t stream);

/* ---- Reed-Solomon syndrome decoding ------------------------------------- */
/*
 * Replaces ReedSolomon.syndrome_decode (qsft/ReedSolomon.py:26-48) for nrows
 * syndromes at once: syms[row*2ts ..] holds the 2ts q-ary channel symbols of a
 * row (2t GF(q^s) syndromes, MSB-first digits); k_out[row*n ..] receives the
 * error values on the last n code positions as the integer form of their
 * GF(q^s) elements (sum of coefficient c_m times q^m), like the reference,
 * whose k has entries >= q for values outside GF(q); zero on a decoding
 * failure.
 * gf_tables: exp | log | zech tables of GF(q^s) (the layout qsft_job.rs_gf_off
 * points at).
 */
int qsft_rs_decode(int q, int s, int t, int n, const int32_t* gf_tables, const uint8_t* syms,
                   int64_t nrows, int16_t* k_out, qsft_stream_t stream);

/* ---- peeling without device allocation ------------------------------------ */
#define QSFT_NOALLOC_MAX_BINS 16384  /* largest C * q^b of a qsft_peel_noalloc job       */
#define QSFT_NOALLOC_KSTRIDE 32      /* out_k row bytes: n <= 32 (n <= 16, coded source)  */
/*
 * No counterpart in the reference: the peeling loop of qsft_peel_init +
 * qsft_peel_run + qsft_collect for ONE job, for callers that cannot allocate
 * device memory: serving threads that must not stall on cudaMalloc's
 * device-wide synchronisation while other streams are busy, and host
 * applications that own every buffer (a fixed memory budget or a pool of
 * their own) and hand a library only its inputs and outputs.  All scratch
 * (hash tables, result store, lists, roots table, control record) lives in a
 * statically sized device array inside the library (about 1.9 MB, held by
 * every GPU that loads the library until the process exits), so the call
 * allocates nothing.  `job` is a host record (offsets off_M/off_D into i8,
 * off_U into U; qsft_workspace_layout's fields are filled in by the call); U
 * holds the job's bins and is peeled in place.  Results as qsft_collect, rows
 * of QSFT_NOALLOC_KSTRIDE bytes; max_out must be at least C*q^b + 64.
 * out_ctrl (device memory, required) receives the job's control record when
 * the loop has ended: out_ctrl->err != 0 (QSFT_ERR_OVERFLOW) means a device
 * table filled up and the results are incomplete; iter, n_balls and
 * num_peeling are those of the workspace path.  Limits: C*q^b <=
 * QSFT_NOALLOC_MAX_BINS and k rows of at most QSFT_NOALLOC_KSTRIDE bytes (n <=
 * 32; n <= 16 for a coded source), else QSFT_ERR_TOO_LARGE.  Every call shares
 * the one array and its contents stay from the last call: calls that overlap
 * on the GPU race; serialise them.  The first call on a device looks up the
 * array's address with that device current; make it before any stream
 * capture.
 */
int qsft_peel_noalloc(int prec, const qsft_job* job, const int8_t* i8, void* U, const int32_t* gf_tables,
                      uint8_t* out_k, double* out_val, int32_t* out_cnt, int64_t* out_total, int32_t max_out,
                      qsft_ctrl* out_ctrl, qsft_stream_t stream);

/*
 * Scratch sizes for a batch: given the jobs' (q, n, b, C, B, src) on the host,
 * writes the counts of bins, hash slots, balls and the kstride (the k row
 * bytes: n, or 2n for a coded source, rounded up to 16, largest over the
 * jobs), and fills the per-job offsets off_bin / off_slot / off_ball,
 * table_cap and ball_cap.
 */
int qsft_workspace_layout(qsft_job* jobs_host, int njobs, int64_t* total_bins,
                          int64_t* total_slots, int64_t* total_balls, int32_t* kstride);

#ifdef __cplusplus
}
#endif
#endif /* QSFT_GB300_H */
