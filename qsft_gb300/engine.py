"""Batched execution of the q-SFT hot path on one GPU.

A :class:`Batch` packs any number of independent transforms ("jobs", possibly
of different shapes) into device buffers laid out as the C ABI expects
(``include/qsft_gb300.h``), and drives the CUDA library through it:

    eval_cosets -> gwht -> noise -> peel (detect / dedupe / subtract, looped) -> collect

PyTorch only provides device memory and the stream; every step of the path is
one of the library's kernels.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import QSFT_F32, QSFT_F64, QsftJob, QsftPlan, QsftCtrl, check, load, stream_handle

EVAL_TILE = 1024  # QSFT_EVAL_TILE
MAX_ITER = 15     # qsft/qsft.py:142

_ROOTS = {}


def roots_table(device):
    """exp(2 pi i m / q) for q <= 32 at index (q*32 + m), computed as the
    reference does: omega ** m with omega = exp(2 pi i / q) (qsft/qsft.py:102,174)."""
    key = str(device)
    if key not in _ROOTS:
        t = np.zeros((33, 32, 2))
        for q in range(2, 33):
            w = np.exp(2j * np.pi / q) ** np.arange(q)
            t[q, :q, 0] = w.real
            t[q, :q, 1] = w.imag
        _ROOTS[key] = torch.from_numpy(t.ravel()).to(device)
    return _ROOTS[key]


def precision_code(precision):
    if precision in ("fp32", "float32", torch.complex64, QSFT_F32):
        return QSFT_F32
    if precision in ("fp64", "float64", torch.complex128, QSFT_F64):
        return QSFT_F64
    raise ValueError(f"unknown precision {precision!r}")


def complex_dtype(prec):
    return torch.complex64 if prec == QSFT_F32 else torch.complex128


class JobSpec:
    """One transform.

    M: (C, n, b) ints; D: (C, R*P, n) ints (the vstacked delays of each group);
    K: (S, n) support and A: (S,) coefficients of a synthetic signal to
    evaluate on the device, or U: a (C, R*P, q^b) complex device tensor of
    precomputed samples/bins; cutoff: the per-entry energy threshold.
    """

    def __init__(self, q, n, b, M, D, R, P, chan="identity", src="identity", cutoff=1e-9, K=None, A=None,
                 U=None, rs=None, max_iter=MAX_ITER, noise_nu=0.0, noise_seed=0):
        self.q, self.n, self.b, self.R, self.P = int(q), int(n), int(b), int(R), int(P)
        self.M = np.ascontiguousarray(np.asarray(M, dtype=np.int64).reshape(-1, self.n, self.b))
        self.C = self.M.shape[0]
        self.D = np.ascontiguousarray(np.asarray(D, dtype=np.int64).reshape(self.C, self.R * self.P, self.n))
        self.chan, self.src, self.rs = chan, src, rs
        self.cutoff = float(cutoff)
        self.K = None if K is None else np.ascontiguousarray(np.asarray(K, dtype=np.int64).reshape(-1, self.n))
        self.A = None if A is None else np.asarray(A, dtype=np.complex128).reshape(-1)
        self.S = 0 if self.K is None else self.K.shape[0]
        self.U = U
        self.max_iter = int(max_iter)
        self.noise_nu = float(noise_nu)
        self.noise_seed = int(noise_seed) & ((1 << 64) - 1)
        self.B = self.q ** self.b
        if not (2 <= self.q <= _lib.MAX_Q) or not (1 <= self.n <= _lib.MAX_N):
            raise ValueError("q must be in 2..32 and n in 1..128")
        if self.B > (1 << 22):
            raise ValueError("q^b above 2^22 bins is not supported")
        for arr in (self.M, self.D) + ((self.K,) if self.K is not None else ()):
            if arr.size and (arr.min() < 0 or arr.max() > 127):
                raise ValueError("M, D and K entries must be non-negative q-ary digits")
        if src == "coded" and rs is None:
            raise ValueError("coded source needs a ReedSolomon description")


class Batch:
    """Device-resident state of a batch of transforms (see module docstring)."""

    def __init__(self, specs, precision="fp32", device=None):
        self.lib = load()
        self.specs = list(specs)
        if not self.specs:
            raise ValueError("empty batch")
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.prec = precision_code(precision)
        cdt = complex_dtype(self.prec)
        J = len(self.specs)
        jobs = (QsftJob * J)()
        i8_parts, a_parts, gf_parts = [], [], []
        off_i8 = off_a = off_u = off_gf = 0
        gf_index = {}
        eval_prefix = [0]
        for j, sp in enumerate(self.specs):
            jb = jobs[j]
            jb.q, jb.n, jb.b, jb.C = sp.q, sp.n, sp.b, sp.C
            jb.R, jb.P, jb.S, jb.B = sp.R, sp.P, sp.S, sp.B
            jb.chan = _lib.CHAN[sp.chan]
            jb.src = _lib.SRC[sp.src]
            jb.max_iter = sp.max_iter
            jb.cutoff = sp.cutoff
            jb.peeling_max = min(sp.q ** sp.n, 1 << 62)
            jb.noise_nu = sp.noise_nu
            jb.noise_seed = sp.noise_seed
            if sp.src == "coded":
                key = (sp.q, sp.rs.s)
                if key not in gf_index:
                    tb = sp.rs.gf_tables()
                    gf_index[key] = off_gf
                    gf_parts.append(tb)
                    off_gf += tb.size
                jb.rs_s, jb.rs_t, jb.rs_gf_off = sp.rs.s, sp.rs.t, gf_index[key]
            for name, arr in (("off_M", sp.M), ("off_D", sp.D), ("off_K", sp.K)):
                setattr(jb, name, off_i8)
                if arr is not None:
                    i8_parts.append(arr.astype(np.int8).ravel())
                    off_i8 += arr.size
            jb.off_A = off_a
            if sp.A is not None:
                a_parts.append(sp.A)
                off_a += sp.A.size
            jb.off_U = off_u
            off_u += sp.C * sp.R * sp.P * sp.B
            eval_prefix.append(eval_prefix[-1] + (sp.C * sp.R * sp.P * sp.B + EVAL_TILE - 1) // EVAL_TILE)
        tb_, ts_, tl_ = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        ks_ = ctypes.c_int32()
        check(self.lib.qsft_workspace_layout(jobs, J, ctypes.byref(tb_), ctypes.byref(ts_), ctypes.byref(tl_),
                                             ctypes.byref(ks_)), "qsft_workspace_layout")
        self.total_bins, self.total_slots, self.total_balls = tb_.value, ts_.value, tl_.value
        self.kstride = ks_.value
        self.jobs_host = jobs
        dev = self.device

        def dt(a, dtype):
            return torch.from_numpy(np.ascontiguousarray(a)).to(dev, dtype=dtype)

        self.i8 = dt(np.concatenate(i8_parts) if i8_parts else np.zeros(1, np.int8), torch.int8)
        a = np.concatenate(a_parts) if a_parts else np.zeros(1, np.complex128)
        self.A = torch.from_numpy(a).to(dev).to(cdt)
        self.U = torch.empty(max(off_u, 1), dtype=cdt, device=dev)
        for j, sp in enumerate(self.specs):
            if sp.U is not None:
                n_el = sp.C * sp.R * sp.P * sp.B
                self.U[jobs[j].off_U:jobs[j].off_U + n_el].copy_(sp.U.reshape(-1).to(cdt))
        self.jobs_dev = torch.frombuffer(bytearray(bytes(jobs)), dtype=torch.uint8).to(dev)
        self.eval_prefix = dt(np.array(eval_prefix, dtype=np.int64), torch.int64)
        self.bin_prefix = dt(np.array([jobs[j].off_bin for j in range(J)] + [self.total_bins], dtype=np.int64),
                             torch.int64)
        self.gf = dt(np.concatenate(gf_parts) if gf_parts else np.zeros(1, np.int32), torch.int32)
        self.roots = roots_table(dev)
        z = lambda n, d: torch.zeros(max(int(n), 1), dtype=d, device=dev)  # noqa: E731
        self.kbuf = z(self.total_bins * self.kstride, torch.uint8)
        self.rho = z(self.total_bins * 2, torch.float64)
        self.tab_key = z(self.total_slots, torch.int64)
        self.tab_best = z(self.total_slots, torch.int64)
        self.uniq = z(self.total_slots, torch.int32)
        self.ball_tab = z(self.total_slots, torch.int32)
        self.ball_k = z(self.total_balls * self.kstride, torch.uint8)
        self.ball_sum = z(self.total_balls * 2, torch.float64)
        self.ball_cnt = z(self.total_balls, torch.int32)
        self.ctrl = z(J * ctypes.sizeof(QsftCtrl), torch.uint8)
        self.out_k = z(self.total_balls * self.kstride, torch.uint8)
        self.out_val = z(self.total_balls * 2, torch.float64)
        self.out_cnt = z(self.total_balls, torch.int32)
        self.out_index = z(2 * J, torch.int64)
        self.out_total = z(1, torch.int64)
        p = QsftPlan()
        p.njobs, p.prec, p.kstride, p.flags = J, self.prec, self.kstride, 0
        p.total_bins, p.total_slots, p.total_balls = self.total_bins, self.total_slots, self.total_balls
        p.total_eval_tiles = eval_prefix[-1]
        p.max_q = max(sp.q for sp in self.specs)
        p.max_n = max(sp.n for sp in self.specs)
        p.all_q_pow2 = int(all((sp.q & (sp.q - 1)) == 0 for sp in self.specs))
        p.max_rp = max(sp.R * sp.P for sp in self.specs)
        ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
        p.jobs, p.eval_prefix, p.bin_prefix = ptr(self.jobs_dev), ptr(self.eval_prefix), ptr(self.bin_prefix)
        p.i8, p.A, p.U, p.gf_tables, p.roots = ptr(self.i8), ptr(self.A), ptr(self.U), ptr(self.gf), ptr(self.roots)
        p.kbuf, p.rho, p.tab_key, p.tab_best = ptr(self.kbuf), ptr(self.rho), ptr(self.tab_key), ptr(self.tab_best)
        p.uniq, p.ball_tab, p.ball_k = ptr(self.uniq), ptr(self.ball_tab), ptr(self.ball_k)
        p.ball_sum, p.ball_cnt, p.ctrl = ptr(self.ball_sum), ptr(self.ball_cnt), ptr(self.ctrl)
        self.plan = p
        # rows per (q, b) size class for the GWHT
        groups = {}
        for j, sp in enumerate(self.specs):
            rows = jobs[j].off_U + np.arange(sp.C * sp.R * sp.P, dtype=np.int64) * sp.B
            groups.setdefault((sp.q, sp.b), []).append(rows)
        self.gwht_groups = {k: dt(np.concatenate(v), torch.int64) for k, v in groups.items()}

    # ------------------------------------------------------------ steps
    def job_U(self, j):
        """The (C, R*P, B) view of job j's samples / bins."""
        sp, jb = self.specs[j], self.jobs_host[j]
        n_el = sp.C * sp.R * sp.P * sp.B
        return self.U[jb.off_U:jb.off_U + n_el].view(sp.C, sp.R * sp.P, sp.B)

    def eval(self, stream=None):
        check(self.lib.qsft_eval_cosets(ctypes.byref(self.plan), stream_handle(stream)), "qsft_eval_cosets")

    def gwht(self, stream=None):
        for (q, b), rows in self.gwht_groups.items():
            check(self.lib.qsft_gwht(self.prec, q, b, ctypes.c_void_p(self.U.data_ptr()),
                                     ctypes.c_void_p(rows.data_ptr()), rows.numel(), stream_handle(stream)),
                  "qsft_gwht")

    def add_noise(self, stream=None):
        check(self.lib.qsft_add_noise_philox(ctypes.byref(self.plan), stream_handle(stream)), "qsft_add_noise")

    def add_bins(self, j, X, stream=None):
        """U_j += X (host-drawn noise uploaded as a device tensor of U_j's shape)."""
        Uj = self.job_U(j)
        X = X.to(self.device, dtype=Uj.dtype).contiguous()
        check(self.lib.qsft_add_bins(self.prec, ctypes.c_void_p(Uj.data_ptr()), ctypes.c_void_p(X.data_ptr()),
                                     Uj.numel(), stream_handle(stream)), "qsft_add_bins")

    def peel(self, max_iter=MAX_ITER, stream=None):
        sh = stream_handle(stream)
        check(self.lib.qsft_peel_init(ctypes.byref(self.plan), sh), "qsft_peel_init")
        check(self.lib.qsft_peel_run(ctypes.byref(self.plan), int(max_iter), sh), "qsft_peel_run")

    def collect_async(self, stream=None):
        self.out_total.zero_()
        check(self.lib.qsft_collect(ctypes.byref(self.plan), ctypes.c_void_p(self.out_k.data_ptr()),
                                    ctypes.c_void_p(self.out_val.data_ptr()), ctypes.c_void_p(self.out_cnt.data_ptr()),
                                    ctypes.c_void_p(self.out_index.data_ptr()),
                                    ctypes.c_void_p(self.out_total.data_ptr()), stream_handle(stream)),
              "qsft_collect")

    def ctrl_host(self):
        raw = self.ctrl.cpu().numpy().tobytes()
        return [QsftCtrl.from_buffer_copy(raw, j * ctypes.sizeof(QsftCtrl)) for j in range(len(self.specs))]

    def results(self):
        """Per job: (keys (m, n) int64, values complex128 (m,), counts int32 (m,), ctrl)."""
        self.collect_async()
        total = int(self.out_total.item())
        idx = self.out_index.cpu().numpy().reshape(-1, 2)
        ks = self.out_k[:max(total, 1) * self.kstride].cpu().numpy().reshape(-1, self.kstride)
        vals = self.out_val[:max(total, 1) * 2].cpu().numpy().reshape(-1, 2)
        cnts = self.out_cnt[:max(total, 1)].cpu().numpy()
        ctrls = self.ctrl_host()
        out = []
        for j, sp in enumerate(self.specs):
            s, c = int(idx[j, 0]), int(idx[j, 1])
            keys = ks[s:s + c, :sp.n].astype(np.int64)
            v = vals[s:s + c, 0] + 1j * vals[s:s + c, 1]
            if ctrls[j].err:
                raise _lib.QsftError(f"job {j}: device table overflow during peeling")
            out.append((keys, v, cnts[s:s + c].copy(), ctrls[j]))
        return out


def to_dict(keys, vals):
    return {tuple(int(x) for x in k): complex(v) for k, v in zip(keys, vals)}


def gwht_device(x, q, b, precision=None):
    """In-place q-ary GWHT of the rows of a contiguous complex CUDA tensor (..., q^b)."""
    lib = load()
    prec = QSFT_F64 if x.dtype == torch.complex128 else QSFT_F32
    if precision is not None and precision_code(precision) != prec:
        raise ValueError("tensor dtype does not match precision")
    if not x.is_cuda or not x.is_contiguous() or x.shape[-1] != q ** b:
        raise ValueError("expected a contiguous CUDA tensor whose last dim is q^b")
    nrows = x.numel() // (q ** b)
    rows = torch.arange(nrows, dtype=torch.int64, device=x.device) * (q ** b)
    check(lib.qsft_gwht(prec, q, b, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(rows.data_ptr()), nrows,
                        stream_handle()), "qsft_gwht")
    return x


def add_bins_(U, X):
    """U += X on the device with the library's kernel (U contiguous, X converted to U's dtype)."""
    lib = load()
    prec = QSFT_F64 if U.dtype == torch.complex128 else QSFT_F32
    if not U.is_contiguous():
        raise ValueError("U must be contiguous")
    X = X.to(U.device, dtype=U.dtype).contiguous()
    if X.numel() != U.numel():
        raise ValueError("shape mismatch")
    check(lib.qsft_add_bins(prec, ctypes.c_void_p(U.data_ptr()), ctypes.c_void_p(X.data_ptr()), U.numel(),
                            stream_handle()), "qsft_add_bins")
    return U


def eval_points_device(X, K, A, q, precision="fp64"):
    """f(x) = sum_s a_s omega^(<x,k_s> mod q) for digit rows X (N, n) on the device."""
    lib = load()
    prec = precision_code(precision)
    cdt = complex_dtype(prec)
    dev = torch.device("cuda", torch.cuda.current_device())
    X = torch.as_tensor(np.ascontiguousarray(X, dtype=np.int8)).to(dev)
    K = torch.as_tensor(np.ascontiguousarray(K, dtype=np.int8)).to(dev)
    A = torch.as_tensor(np.asarray(A, dtype=np.complex128)).to(dev).to(cdt)
    N, n = X.shape
    out = torch.empty(max(N, 1), dtype=cdt, device=dev)
    check(lib.qsft_eval_points(prec, int(q), int(n), int(K.shape[0]), ctypes.c_void_p(X.data_ptr()), N,
                               ctypes.c_void_p(K.data_ptr()), ctypes.c_void_p(A.data_ptr()),
                               ctypes.c_void_p(out.data_ptr()), stream_handle()), "qsft_eval_points")
    return out[:N]


def rs_decode_batch(rs, syndromes):
    """Decode rows of 2ts q-ary syndrome symbols on the GPU; returns (rows, n) int64."""
    lib = load()
    dev = torch.device("cuda", torch.cuda.current_device())
    syn = np.ascontiguousarray(np.asarray(syndromes, dtype=np.int64) % rs.q, dtype=np.uint8)
    nrows = syn.shape[0]
    gf = torch.from_numpy(rs.gf_tables()).to(dev)
    sy = torch.from_numpy(syn).to(dev)
    out = torch.zeros(max(nrows * rs.ns, 1), dtype=torch.uint8, device=dev)
    check(lib.qsft_rs_decode(rs.q, rs.s, rs.t, rs.ns, ctypes.c_void_p(gf.data_ptr()), ctypes.c_void_p(sy.data_ptr()),
                             nrows, ctypes.c_void_p(out.data_ptr()), stream_handle()), "qsft_rs_decode")
    return out[:nrows * rs.ns].cpu().numpy().reshape(nrows, rs.ns).astype(np.int64)
