"""ctypes binding of the C ABI in ``include/qsft_gb300.h``.

The shared library is built in-tree (``qsft_gb300/build.py``) and loaded from
``qsft_gb300/lib/``.  There is no fallback: if the library is missing or was
built for another architecture, every GPU entry point raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libqsft_gb300.so")

QSFT_F32 = 4
QSFT_F64 = 8
CHAN = {"identity": 0, "nso": 1}
SRC = {"identity": 0, "coded": 1}
MAX_Q = 32
MAX_N = 128
MAX_RS_T = 16
MAX_GF = 4096
TC_TILES = 16     # QSFT_TC_TILES
TC_TILE_M = 128
NOALLOC_MAX_BINS = 16384   # QSFT_NOALLOC_MAX_BINS
NOALLOC_KSTRIDE = 32       # QSFT_NOALLOC_KSTRIDE
TC_SUB_N = 128
PEEL_LAUNCHES_PER_ITER = 3   # QSFT_PEEL_LAUNCHES_PER_ITER
PLAN_TEST_BARRIER_TIMEOUT = 2   # QSFT_PLAN_TEST_BARRIER_TIMEOUT
GWHT_SCHEDULES = {1: "row", 2: "rowc", 3: "cluster", 4: "passes", 5: "passes_small"}   # QSFT_GWHT_*

# exported symbols, in header order
SYMBOLS = [
    "qsft_abi_version", "qsft_status_string", "qsft_built_arch", "qsft_launch_count", "qsft_eval_cosets",
    "qsft_eval_cosets_tc", "qsft_eval_cosets_gemm", "qsft_gemm_layout", "qsft_eval_points",
    "qsft_gwht_noise", "qsft_gwht", "qsft_gwht_schedules", "qsft_gwht_select", "qsft_gwht_selected",
    "qsft_add_noise_philox", "qsft_add_bins", "qsft_peel_init", "qsft_peel_iteration",
    "qsft_peel_run", "qsft_peel_persistent", "qsft_collect", "qsft_reproject", "qsft_rs_decode", "qsft_peel_noalloc", "qsft_workspace_layout",
]


class QsftError(RuntimeError):
    pass


class QsftJob(ctypes.Structure):
    _fields_ = [
        ("q", ctypes.c_int32), ("n", ctypes.c_int32), ("b", ctypes.c_int32), ("C", ctypes.c_int32),
        ("R", ctypes.c_int32), ("P", ctypes.c_int32), ("S", ctypes.c_int32), ("B", ctypes.c_int32),
        ("chan", ctypes.c_int32), ("src", ctypes.c_int32),
        ("rs_s", ctypes.c_int32), ("rs_t", ctypes.c_int32),
        ("rs_gf_off", ctypes.c_int32), ("max_iter", ctypes.c_int32),
        ("table_cap", ctypes.c_int32), ("ball_cap", ctypes.c_int32),
        ("cutoff", ctypes.c_double),
        ("peeling_max", ctypes.c_int64),
        ("off_M", ctypes.c_int64), ("off_D", ctypes.c_int64), ("off_K", ctypes.c_int64),
        ("off_A", ctypes.c_int64), ("off_U", ctypes.c_int64),
        ("off_bin", ctypes.c_int64), ("off_slot", ctypes.c_int64), ("off_ball", ctypes.c_int64),
        ("noise_seed", ctypes.c_uint64),
        ("noise_nu", ctypes.c_double),
    ]


class QsftCtrl(ctypes.Structure):
    _fields_ = [
        ("done", ctypes.c_int32), ("iter", ctypes.c_int32), ("n_single", ctypes.c_int32),
        ("n_multi", ctypes.c_int32), ("n_unique", ctypes.c_int32), ("n_balls", ctypes.c_int32),
        ("err", ctypes.c_int32), ("n_cand", ctypes.c_int32), ("n_dirty", ctypes.c_int32 * 2),
        ("num_peeling", ctypes.c_int64),
    ]


_P = ctypes.c_void_p


class QsftPlan(ctypes.Structure):
    _fields_ = [
        ("njobs", ctypes.c_int32), ("prec", ctypes.c_int32), ("kstride", ctypes.c_int32), ("flags", ctypes.c_int32),
        ("total_bins", ctypes.c_int64), ("total_slots", ctypes.c_int64), ("total_balls", ctypes.c_int64),
        ("total_eval_tiles", ctypes.c_int64),
        ("max_q", ctypes.c_int32), ("max_n", ctypes.c_int32), ("all_q_pow2", ctypes.c_int32),
        ("max_rp", ctypes.c_int32),
        ("jobs", _P), ("eval_prefix", _P), ("bin_prefix", _P), ("i8", _P), ("A", _P), ("U", _P),
        ("gf_tables", _P), ("roots", _P),
        ("rho", _P), ("ball_tab", _P), ("ball_best", _P), ("uniq", _P),
        ("ball_k", _P), ("ball_sum", _P), ("ball_cnt", _P), ("ctrl", _P),
        ("bin_status", _P), ("bin_stamp", _P), ("dirty", _P), ("cand", _P), ("stage", _P), ("done_count", _P),
        ("tc_prefix", _P), ("total_tc_work", ctypes.c_int64), ("tc_smax", ctypes.c_int32),
        ("tc_npad", ctypes.c_int32), ("min_q", ctypes.c_int32), ("tc_table_bytes", ctypes.c_int32),
        ("tc_entry_bytes", ctypes.c_int32), ("stage_rp", ctypes.c_int32), ("status", _P),
        ("gm_ws", _P), ("gm_index", _P), ("total_gm_work", ctypes.c_int64), ("total_gm_prep", ctypes.c_int64),
        ("gm_ws_bytes", ctypes.c_int64), ("gm_mt", ctypes.c_int32), ("gm_kps", ctypes.c_int32),
        ("gm_nw", ctypes.c_int32), ("gm_npmax", ctypes.c_int32), ("gm_jt_bytes", ctypes.c_int32),
        ("gm_nacc", ctypes.c_int32),
    ]


_lib = None


def load():
    """Load the in-tree library (once) and declare the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise QsftError(f"{LIB_PATH} is missing: build it with `python qsft_gb300/build.py` "
                        "(or __graft_entry__.build()); there is no CPU fallback")
    L = ctypes.CDLL(LIB_PATH)
    i32, i64, vp = ctypes.c_int, ctypes.c_int64, ctypes.c_void_p
    plan_p = ctypes.POINTER(QsftPlan)
    sig = {
        "qsft_abi_version": ([], i32),
        "qsft_status_string": ([i32], ctypes.c_char_p),
        "qsft_built_arch": ([], i32),
        "qsft_launch_count": ([], i64),
        "qsft_eval_cosets": ([plan_p, vp], i32),
        "qsft_eval_cosets_tc": ([plan_p, vp], i32),
        "qsft_eval_cosets_gemm": ([plan_p, vp], i32),
        "qsft_gemm_layout": ([ctypes.POINTER(QsftJob), i32, plan_p, ctypes.POINTER(i64)], i32),
        "qsft_eval_points": ([i32, i32, i32, i32, vp, i64, vp, vp, vp, vp], i32),
        "qsft_gwht": ([i32, i32, i32, vp, vp, i64, vp], i32),
        "qsft_gwht_noise": ([plan_p, i32, i32, vp, vp, i64, vp], i32),
        "qsft_gwht_schedules": ([i32, i32, i32, ctypes.POINTER(ctypes.c_int32), i32], i32),
        "qsft_gwht_select": ([i32, i32, i32, i32], i32),
        "qsft_gwht_selected": ([i32, i32, i32], i32),
        "qsft_add_noise_philox": ([plan_p, vp], i32),
        "qsft_add_bins": ([i32, vp, vp, i64, vp], i32),
        "qsft_peel_init": ([plan_p, vp], i32),
        "qsft_peel_iteration": ([plan_p, i32, vp], i32),
        "qsft_peel_run": ([plan_p, i32, vp], i32),
        "qsft_peel_persistent": ([plan_p, i32, vp], i32),
        "qsft_collect": ([plan_p, vp, vp, vp, vp, vp, vp], i32),
        "qsft_reproject": ([plan_p, vp, vp, vp, vp, vp], i32),
        "qsft_rs_decode": ([i32, i32, i32, i32, vp, vp, i64, vp, vp], i32),
        "qsft_peel_noalloc": ([i32, ctypes.POINTER(QsftJob), vp, vp, vp, vp, vp, vp, vp, i32, vp, vp], i32),
        "qsft_workspace_layout": ([ctypes.POINTER(QsftJob), i32, ctypes.POINTER(i64), ctypes.POINTER(i64),
                                   ctypes.POINTER(i64), ctypes.POINTER(ctypes.c_int32)], i32),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    if L.qsft_abi_version() != 1:
        raise QsftError("libqsft_gb300.so ABI version mismatch")
    _lib = L
    return L


def check(rc, what):
    if rc != 0:
        msg = load().qsft_status_string(rc).decode()
        raise QsftError(f"{what} failed: {msg} ({rc})")


def stream_handle(stream=None):
    """cudaStream_t of a torch stream (default: the current stream)."""
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)
