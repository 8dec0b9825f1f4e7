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

from . import _lib, autotune
from ._lib import QSFT_F32, QSFT_F64, QsftJob, QsftPlan, QsftCtrl, check, load, stream_handle

EVAL_TILE = 1024  # QSFT_EVAL_TILE
TC_TILE_M = 128   # samples per tensor-core tile
TC_SUB_N = 128    # support entries per MMA sub-tile
TC_SMEM_TARGET = 110 * 1024   # two CTAs per SM


def tc_entry_bytes(qs):
    """Table bytes per support entry of the tensor-core kernel: a pair table
    (q*q entries per two support entries) when every job has the same q in {2, 4}."""
    qs = set(qs)
    if len(qs) == 1 and next(iter(qs)) in (2, 4):
        q = next(iter(qs))
        return q * q * 4
    return max(qs) * 8


def tc_smem_bytes(npad, smax, entry_bytes, table_bytes=0):
    """Shared memory of the tensor-core evaluation kernel (mirrors eval_tc.cu)."""
    return max(2048 + 128 * npad * 2 + smax * npad * 2 + smax * entry_bytes + table_bytes, 80 * 1024)
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

    @classmethod
    def trusted(cls, q, n, b, M, D, R, P, chan, src, cutoff, K, A, rs, max_iter, noise_nu, noise_seed):
        """A JobSpec from arrays that already passed __init__'s conversions and
        checks (M (C, n, b), D (C, R*P, n), K (S, n) as int64 or int8 digits;
        complex128 A): the per-submit path of a request whose arrays were
        validated once."""
        sp = cls.__new__(cls)
        sp.q, sp.n, sp.b, sp.R, sp.P = q, n, b, R, P
        sp.M, sp.D, sp.C = M, D, M.shape[0]
        sp.chan, sp.src, sp.rs, sp.cutoff = chan, src, rs, float(cutoff)
        sp.K, sp.A = K, A
        sp.S = 0 if K is None else K.shape[0]
        sp.U = None
        sp.max_iter = int(max_iter)
        sp.noise_nu = float(noise_nu)
        sp.noise_seed = int(noise_seed) & ((1 << 64) - 1)
        sp.B = q ** b
        return sp


def workspace_bytes(specs, precision="fp32", reproject=False):
    """Device bytes a :class:`Batch` of `specs` allocates (its workspace, inputs
    and outputs; not the per-device roots table): the admission footprint of a
    serving loop.  Host-only -- the library's layout functions, no GPU."""
    b = Batch.__new__(Batch)
    b.lib = load()
    b.reproject = bool(reproject)
    b.prec = precision_code(precision)
    b._build_layout(list(specs))
    return b.planned_bytes()


def layout_key(spec):
    """Everything that fixes a job's place in the device workspace."""
    rs = (spec.rs.s, spec.rs.t) if spec.rs is not None else None
    return (spec.q, spec.n, spec.b, spec.C, spec.R, spec.P, spec.S, spec.chan, spec.src, rs)


class Batch:
    """Device-resident state of a batch of transforms (see module docstring).

    The workspace is allocated once per layout (the jobs' shapes); ``load``
    replaces the inputs of a batch with the same layout through pinned host
    staging buffers, so a serving loop re-uses one Batch per layout."""

    def __init__(self, specs, precision="fp32", device=None, reproject=False, peel_mode="graph"):
        self.lib = load()
        self.reproject = bool(reproject)
        if peel_mode not in ("graph", "persistent"):
            raise ValueError(f"unknown peel_mode {peel_mode!r}")
        self.peel_mode = peel_mode
        specs = list(specs)
        if not specs:
            raise ValueError("empty batch")
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.prec = precision_code(precision)
        self.cdt = complex_dtype(self.prec)
        self.layout = tuple(layout_key(sp) for sp in specs)
        self._build_layout(specs)
        self._allocate()
        self.load(specs)

    # ------------------------------------------------------------ layout
    def _build_layout(self, specs):
        J = len(specs)
        jobs = (QsftJob * J)()
        off_i8 = off_a = off_u = off_gf = 0
        gf_index, gf_parts = {}, []
        eval_prefix = [0]
        for j, sp in enumerate(specs):
            jb = jobs[j]
            jb.q, jb.n, jb.b, jb.C = sp.q, sp.n, sp.b, sp.C
            jb.R, jb.P, jb.S, jb.B = sp.R, sp.P, sp.S, sp.B
            jb.chan = _lib.CHAN[sp.chan]
            jb.src = _lib.SRC[sp.src]
            jb.peeling_max = min(sp.q ** sp.n, 1 << 62)
            if sp.src == "coded":
                key = (sp.q, sp.rs.s)
                if key not in gf_index:
                    tb = sp.rs.gf_tables()
                    gf_index[key] = off_gf
                    gf_parts.append(tb)
                    off_gf += tb.size
                jb.rs_s, jb.rs_t, jb.rs_gf_off = sp.rs.s, sp.rs.t, gf_index[key]
            # 16-byte aligned sub-arrays (word loads of the delay rows in detection)
            jb.off_M = off_i8
            off_i8 = (off_i8 + sp.M.size + 15) & ~15
            jb.off_D = off_i8
            off_i8 = (off_i8 + sp.D.size + 15) & ~15
            jb.off_K = off_i8
            off_i8 = (off_i8 + (0 if sp.K is None else sp.K.size) + 15) & ~15
            jb.off_A = off_a
            off_a += 0 if sp.A is None else sp.A.size
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
        self.n_i8, self.n_a, self.n_u = off_i8, off_a, off_u
        # the padding after each job's M, D and K rows (zeros), so that `load`
        # writes the whole digit buffer with one concatenation
        self._pads = []
        for jb, sp in zip(jobs, specs):
            ends = (jb.off_M + sp.M.size, jb.off_D + sp.D.size, jb.off_K + (0 if sp.K is None else sp.K.size))
            nxt = (jb.off_D, jb.off_K, (ends[2] + 15) & ~15)
            self._pads.append([np.zeros(b - a, np.int8) for a, b in zip(ends, nxt)])
        self.eval_prefix_host = eval_prefix
        self.gf_host = np.concatenate(gf_parts) if gf_parts else np.zeros(1, np.int32)
        self.njobs = J
        self.shapes = [(sp.q, sp.n, sp.b, sp.C, sp.R, sp.P, sp.S, sp.B) for sp in specs]
        # coded sources keep each k entry's high part (v // q of a decoded RS
        # value v outside GF(q)) in the n bytes after the digits of a k row
        self.coded = [sp.src == "coded" for sp in specs]
        # tensor-core evaluation: K extent, support chunk, work items
        maxn = max(sp.n for sp in specs)
        self.tc_npad = 32 if maxn <= 32 else (64 if maxn <= 64 else 128)
        self.tc_entry_bytes = tc_entry_bytes([sp.q for sp in specs])
        self.tc_table_bytes = max(sp.C * (sp.b * sp.q + sp.R * sp.P) * self.tc_npad for sp in specs)
        smax = TC_SUB_N
        while tc_smem_bytes(self.tc_npad, smax + TC_SUB_N, self.tc_entry_bytes,
                            self.tc_table_bytes) <= TC_SMEM_TARGET:
            smax += TC_SUB_N
        self.tc_smax = smax
        # the tensor-core kernel needs its tables and one 128-entry support chunk in shared memory
        self.tc_ok = tc_smem_bytes(self.tc_npad, smax, self.tc_entry_bytes, self.tc_table_bytes) <= 227 * 1024
        tc_prefix = [0]
        self.tc_needs_zero = False
        for sp in specs:
            tiles = -(-(sp.C * sp.R * sp.P * sp.B) // TC_TILE_M)
            groups = -(-tiles // _lib.TC_TILES)
            chunks = -(-sp.S // smax)
            self.tc_needs_zero |= chunks != 1
            tc_prefix.append(tc_prefix[-1] + chunks * groups)
        self.tc_prefix_host = tc_prefix
        rows, meta = {}, {}
        for j, sp in enumerate(specs):
            idx = np.arange(sp.C * sp.R * sp.P, dtype=np.int64)
            rows.setdefault((sp.q, sp.b), []).append(jobs[j].off_U + idx * sp.B)
            # (job, row within the job) per row: the key of the row's device noise
            meta.setdefault((sp.q, sp.b), []).append(np.stack([np.full_like(idx, j), idx], axis=1).astype(np.int32))
        self.gwht_rows_host = {k: np.concatenate(v) for k, v in rows.items()}
        self.gwht_meta_host = {k: np.concatenate(v).ravel() for k, v in meta.items()}
        self.max_iter = max(sp.max_iter for sp in specs)

    def _index_block(self):
        """The small index arrays the kernels read (job prefixes, GF tables, GWHT
        row offsets and row metadata, the GEMM work index), packed into one int64
        host array so that they reach the device in one copy: (array,
        {name: (word offset, length, dtype)}, GEMM work index or None).  Every
        segment starts 16 bytes after a multiple of 16."""
        J = self.njobs
        segs = [("eval_prefix", np.asarray(self.eval_prefix_host, dtype=np.int64), torch.int64),
                ("bin_prefix", np.array([self.jobs_host[j].off_bin for j in range(J)] + [self.total_bins],
                                        dtype=np.int64), torch.int64),
                ("tc_prefix", np.asarray(self.tc_prefix_host, dtype=np.int64), torch.int64),
                ("gf", np.ascontiguousarray(self.gf_host, dtype=np.int32), torch.int32)]
        for k, v in self.gwht_rows_host.items():
            segs.append((("rows", k), np.ascontiguousarray(v, dtype=np.int64), torch.int64))
        for k, v in self.gwht_meta_host.items():
            segs.append((("meta", k), np.ascontiguousarray(v, dtype=np.int32), torch.int32))
        gm_index = None
        if self.prec == QSFT_F32:
            index = (ctypes.c_int64 * (3 * J + 2))()
            if self.lib.qsft_gemm_layout(self.jobs_host, J, ctypes.byref(QsftPlan()), index) == 0:
                gm_index = np.frombuffer(index, dtype=np.int64).copy()
                segs.append(("gm_index", gm_index, torch.int64))
        place, words = {}, 0
        for name, arr, dt in segs:
            place[name] = (words, arr.size, dt)
            words += max(2, (arr.nbytes + 15) // 16 * 2)
        block = np.zeros(words, dtype=np.int64)
        raw = block.view(np.uint8)
        for name, arr, _ in segs:
            off = place[name][0] * 8
            raw[off:off + arr.nbytes] = arr.view(np.uint8)
        return block, place, gm_index

    def planned_bytes(self):
        """Bytes ``_allocate`` takes for this layout, each buffer rounded up to the
        caching allocator's 512-byte blocks."""
        J, es = self.njobs, (8 if self.prec == QSFT_F32 else 16)
        bins, slots, balls, ks = self.total_bins, self.total_slots, self.total_balls, self.kstride
        cs = ctypes.sizeof(QsftCtrl) // 8
        block, _, _ = self._index_block()
        sizes = [max(self.n_i8, 1), max(self.n_a, 1) * es, max(self.n_u, 1) * es, ctypes.sizeof(QsftJob) * J,
                 block.nbytes,                                                      # packed index arrays
                 bins * 16, slots * 8, balls * 8, balls * 4,                        # rho, ball table, best, uniq
                 balls * ks, balls * 16, balls * 4,                                 # ball k, sum, count
                 bins, bins * 4, 2 * bins * 4, bins * 4,                            # status, stamp, dirty, cand
                 (bins // 8) * self.stage_rp() * es,                                # staged candidate columns
                 balls * ks, balls * 16, balls * 4, (2 + 2 * J + cs * J) * 8, 16]   # outputs, metadata, done
        if getattr(self, "reproject", False):
            sizes.append(max(self.n_u, 1) * es)                                      # raw bins copy
        if self.prec == QSFT_F32:
            p = QsftPlan()
            index = (ctypes.c_int64 * (3 * J + 2))()
            if self.lib.qsft_gemm_layout(self.jobs_host, J, ctypes.byref(p), index) == 0:
                sizes.append(max(int(p.gm_ws_bytes), 256))
        return int(sum((s + 511) // 512 * 512 for s in sizes))

    def stage_rp(self):
        """Column length of the peeling's staging buffer: the longest R*P, at most 64."""
        return max(1, min(max(s[4] * s[5] for s in self.shapes), 64))

    def device_bytes(self):
        """Bytes of this batch's device tensors (what ``planned_bytes`` predicts)."""
        seen, total = {self.roots.untyped_storage().data_ptr()}, 0
        for v in vars(self).values():
            ts = v.values() if isinstance(v, dict) else [v]
            for t in ts:
                if isinstance(t, torch.Tensor) and t.device.type == "cuda":
                    key = t.untyped_storage().data_ptr()
                    if key not in seen:
                        seen.add(key)
                        total += (t.untyped_storage().nbytes() + 511) // 512 * 512
        return total

    def _allocate(self):
        dev, J = self.device, self.njobs
        z = lambda n, d: torch.zeros(max(int(n), 1), dtype=d, device=dev)  # noqa: E731
        self.i8 = z(self.n_i8, torch.int8)
        self.A = z(self.n_a, self.cdt)
        self.U = torch.empty(max(self.n_u, 1), dtype=self.cdt, device=dev)
        self.jobs_dev = z(ctypes.sizeof(QsftJob) * J, torch.uint8)
        # the small index arrays: one pinned staging buffer, one copy on the current
        # stream, typed views into one device buffer
        block, place, gm_index = self._index_block()
        self._index_host = torch.from_numpy(block).pin_memory()
        self.index_dev = torch.empty(block.size, dtype=torch.int64, device=dev)
        self.index_dev.copy_(self._index_host, non_blocking=True)

        def view(name):
            w, n, dt = place[name]
            if dt == torch.int64:
                return self.index_dev[w:w + n]
            return self.index_dev[w:w + (n + 1) // 2].view(torch.int32)[:n]

        self.eval_prefix, self.bin_prefix = view("eval_prefix"), view("bin_prefix")
        self.tc_prefix, self.gf = view("tc_prefix"), view("gf")
        self.gwht_groups = {k: view(("rows", k)) for k in self.gwht_rows_host}
        self.gwht_meta = {k: view(("meta", k)) for k in self.gwht_meta_host}
        self.roots = roots_table(dev)
        self.rho = z(self.total_bins * 2, torch.float64)
        self.ball_tab = z(self.total_slots, torch.int64)
        self.ball_best = z(self.total_balls, torch.int64)
        self.uniq = z(self.total_balls, torch.int32)
        self.ball_k = z(self.total_balls * self.kstride, torch.uint8)
        self.ball_sum = z(self.total_balls * 2, torch.float64)
        self.ball_cnt = z(self.total_balls, torch.int32)
        self.bin_status = z(self.total_bins, torch.uint8)
        self.bin_stamp = z(self.total_bins, torch.int32)
        self.dirty = z(2 * self.total_bins, torch.int32)
        self.out_k = z(self.total_balls * self.kstride, torch.uint8)
        self.out_val = z(self.total_balls * 2, torch.float64)
        self.out_cnt = z(self.total_balls, torch.int32)
        # metadata read back after a run, in one copy: total | index[2J] | ctrl[J] | status
        cs = ctypes.sizeof(QsftCtrl) // 8
        self.meta = z(1 + 2 * J + cs * J + 1, torch.int64)
        self.out_total = self.meta[0:1]
        self.out_index = self.meta[1:1 + 2 * J]
        self.ctrl = self.meta[1 + 2 * J:1 + 2 * J + cs * J].view(torch.uint8)
        self.status = self.meta[1 + 2 * J + cs * J:].view(torch.int32)
        self.meta_host = torch.empty_like(self.meta, device="cpu").pin_memory()
        # pinned staging for inputs
        self.i8_host = torch.empty(self.i8.numel(), dtype=torch.int8).pin_memory()
        self.A_host = torch.empty(self.A.numel(), dtype=self.cdt).pin_memory()
        self.jobs_host_t = torch.empty(self.jobs_dev.numel(), dtype=torch.uint8).pin_memory()
        p = QsftPlan()
        p.njobs, p.prec, p.kstride, p.flags = J, self.prec, self.kstride, 0
        p.total_bins, p.total_slots, p.total_balls = self.total_bins, self.total_slots, self.total_balls
        p.total_eval_tiles = self.eval_prefix_host[-1]
        qs = [s[0] for s in self.shapes]
        p.max_q, p.min_q = max(qs), min(qs)
        p.max_n = max(s[1] for s in self.shapes)
        p.all_q_pow2 = int(all((q & (q - 1)) == 0 for q in qs))
        p.max_rp = max(s[4] * s[5] for s in self.shapes)
        ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
        p.jobs, p.eval_prefix, p.bin_prefix = ptr(self.jobs_dev), ptr(self.eval_prefix), ptr(self.bin_prefix)
        p.i8, p.A, p.U, p.gf_tables, p.roots = ptr(self.i8), ptr(self.A), ptr(self.U), ptr(self.gf), ptr(self.roots)
        p.rho, p.ball_tab, p.ball_best = ptr(self.rho), ptr(self.ball_tab), ptr(self.ball_best)
        p.uniq, p.ball_k = ptr(self.uniq), ptr(self.ball_k)
        p.ball_sum, p.ball_cnt, p.ctrl = ptr(self.ball_sum), ptr(self.ball_cnt), ptr(self.ctrl)
        p.bin_status, p.bin_stamp = ptr(self.bin_status), ptr(self.bin_stamp)
        p.dirty = ptr(self.dirty)
        self.cand = z(self.total_bins, torch.int32)
        p.cand = ptr(self.cand)
        # copies of the candidates' columns (1/8 of the bins, R*P <= 64 only)
        p.stage_rp = self.stage_rp()
        self.stage = torch.empty(max((self.total_bins // 8) * p.stage_rp, 1), dtype=self.cdt, device=dev)
        p.stage = ptr(self.stage)
        self.done_count = z(4, torch.int32)
        p.done_count = ptr(self.done_count)
        p.tc_prefix, p.total_tc_work = ptr(self.tc_prefix), self.tc_prefix_host[-1]
        p.tc_smax, p.tc_npad, p.tc_table_bytes = self.tc_smax, self.tc_npad, self.tc_table_bytes
        p.tc_entry_bytes = self.tc_entry_bytes
        p.status = ptr(self.status)
        # coset-factored GEMM evaluation (FP32): operand workspace and work index
        # (the layout call fills the plan's gm_* fields; its index is in the block)
        index = (ctypes.c_int64 * (3 * J + 2))()
        # the bins as they were before the peeling, for the optional re-projection
        self.U_raw = torch.empty_like(self.U) if getattr(self, "reproject", False) else None
        self.gm_ok = (gm_index is not None and
                      self.lib.qsft_gemm_layout(self.jobs_host, J, ctypes.byref(p), index) == 0)
        if self.gm_ok:
            self.gm_ws = torch.empty(max(int(p.gm_ws_bytes), 256), dtype=torch.uint8, device=dev)
            self.gm_index = view("gm_index")
            p.gm_ws, p.gm_index = ptr(self.gm_ws), ptr(self.gm_index)
        self.plan = p

    # ------------------------------------------------------------ inputs
    def load(self, specs, stream=None):
        """Copy the inputs of `specs` (same layout as this batch) to the device."""
        specs = list(specs)
        if tuple(layout_key(sp) for sp in specs) != self.layout:
            raise ValueError("specs do not match this batch's layout")
        self.specs = specs
        jobs = self.jobs_host
        self._pack_host(specs, self.i8_host.numpy(), self.A_host.numpy())
        self.jobs_host_t.numpy()[:] = np.frombuffer(bytes(jobs), dtype=np.uint8)
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.stream(st):
            self.i8.copy_(self.i8_host, non_blocking=True)
            self.A.copy_(self.A_host, non_blocking=True)
            self.jobs_dev.copy_(self.jobs_host_t, non_blocking=True)
            for j, sp in enumerate(specs):
                if sp.U is not None:
                    n_el = sp.C * sp.R * sp.P * sp.B
                    self.U[jobs[j].off_U:jobs[j].off_U + n_el].copy_(sp.U.reshape(-1).to(self.cdt))
        self.h2d_bytes = self.i8.numel() + self.A.numel() * self.A.element_size() + self.jobs_dev.numel()

    def _pack_host(self, specs, i8, a):
        """The jobs' per-step fields into the host job records, and their M, D, K
        digits and coefficients into the host arrays `i8` and `a` at the
        layout's offsets (one concatenation per array: each job's M, D and K
        rows followed by the zeros up to the next 16-byte boundary)."""
        pieces, apieces = [], []
        empty = np.zeros(0, np.int8)
        for j, sp in enumerate(specs):
            jb = self.jobs_host[j]
            jb.max_iter = sp.max_iter
            jb.cutoff = sp.cutoff
            jb.noise_nu = sp.noise_nu
            jb.noise_seed = sp.noise_seed
            pm, pd, pk = self._pads[j]
            pieces += [sp.M.ravel(), pm, sp.D.ravel(), pd, empty if sp.K is None else sp.K.ravel(), pk]
            if sp.A is not None:
                apieces.append(sp.A.ravel())
        if self.n_i8:
            np.concatenate(pieces, out=i8[:self.n_i8], casting="same_kind")
        if apieces:
            np.concatenate(apieces, out=a[:self.n_a], casting="same_kind")

    # ------------------------------------------------------------ steps
    def job_U(self, j):
        """The (C, R*P, B) view of job j's samples / bins."""
        sp, jb = self.specs[j], self.jobs_host[j]
        n_el = sp.C * sp.R * sp.P * sp.B
        return self.U[jb.off_U:jb.off_U + n_el].view(sp.C, sp.R * sp.P, sp.B)

    def eval_method(self):
        """The evaluation kernel ``eval`` picks: "gemm" (coset-factored tensor-core
        GEMM), "tc" (tensor-core dot products + CUDA-core reduction) or "cuda"."""
        if self.prec != QSFT_F32:
            return "cuda"
        return "gemm" if self.gm_ok else ("tc" if self.tc_ok else "cuda")

    def eval(self, stream=None, method=None):
        """Coset evaluation into U with `method` (default: ``eval_method()``)."""
        method = method or self.eval_method()
        if method == "gemm":
            if not self.gm_ok:
                raise ValueError("this batch is outside the GEMM evaluation's limits")
            check(self.lib.qsft_eval_cosets_gemm(ctypes.byref(self.plan), stream_handle(stream)),
                  "qsft_eval_cosets_gemm")
        elif method == "tc":
            self.U.zero_()   # the tensor-core kernel accumulates partial sums into U
            check(self.lib.qsft_eval_cosets_tc(ctypes.byref(self.plan), stream_handle(stream)), "qsft_eval_cosets_tc")
        elif method == "cuda":
            check(self.lib.qsft_eval_cosets(ctypes.byref(self.plan), stream_handle(stream)), "qsft_eval_cosets")
        else:
            raise ValueError(f"unknown evaluation method {method!r}")

    def gwht_noise(self, stream=None):
        """GWHT of every row, with each job's device bin noise added in the same pass
        (each shape's schedule tuned on its first use, see autotune.ensure)."""
        for (q, b), rows in self.gwht_groups.items():
            autotune.ensure(q, b, self.prec, self.device)
            check(self.lib.qsft_gwht_noise(ctypes.byref(self.plan), q, b, ctypes.c_void_p(rows.data_ptr()),
                                           ctypes.c_void_p(self.gwht_meta[(q, b)].data_ptr()), rows.numel(),
                                           stream_handle(stream)), "qsft_gwht_noise")

    def gwht(self, stream=None):
        for (q, b), rows in self.gwht_groups.items():
            autotune.ensure(q, b, self.prec, self.device)
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
        if self.U_raw is not None:
            st = stream if stream is not None else torch.cuda.current_stream(self.device)
            with torch.cuda.stream(st):
                self.U_raw.copy_(self.U)
        check(self.lib.qsft_peel_init(ctypes.byref(self.plan), sh), "qsft_peel_init")
        if self.peel_mode == "persistent":   # the loop in one cooperative launch
            check(self.lib.qsft_peel_persistent(ctypes.byref(self.plan), int(max_iter), sh), "qsft_peel_persistent")
        else:                                # a launch per phase; a WHILE node when captured
            check(self.lib.qsft_peel_run(ctypes.byref(self.plan), int(max_iter), sh), "qsft_peel_run")

    # ------------------------------------------------------------ whole step
    def step(self, max_iter=None, stream=None):
        """eval -> gwht + noise -> peel -> collect, issued on the stream."""
        self.eval(stream)
        self.gwht_noise(stream)
        self.peel(self.max_iter if max_iter is None else max_iter, stream)
        self.collect_async(stream)

    def capture(self, max_iter=None):
        """Record one step into a CUDA graph (replayed by run()); the graph reads
        the workspace buffers, so later load()s need no re-capture."""
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            self.step(max_iter)            # warm-up: kernel attributes, lazy loads
        torch.cuda.current_stream(self.device).wait_stream(side)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        l0 = self.lib.qsft_launch_count()
        with torch.cuda.graph(g):
            self.step(max_iter)
        self.graph_launches = self.lib.qsft_launch_count() - l0
        self.graph = g
        return g

    def launches_per_run(self, ctrl=None):
        """Library kernels one graph replay executed: the captured launches, with
        the peeling loop's body (captured once) counted once per iteration
        after the first that the jobs actually ran (read from the control records)."""
        ctrl = self.ctrl_host() if ctrl is None else ctrl
        extra = max(max(int(c.iter) for c in ctrl) - 2, -1)
        return self.graph_launches + _lib.PEEL_LAUNCHES_PER_ITER * extra

    def run(self, stream=None):
        """One step on `stream` (default: the current stream): graph replay when
        captured, else direct launches."""
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.stream(st):
            g = getattr(self, "graph", None)
            if g is not None:
                g.replay()
            else:
                self.step()

    def fetch_async(self, stream=None, rows_hint=None):
        """Queue the result read-back on `stream` without waiting: the metadata and
        the first `rows_hint` output rows go to pinned host buffers, and an event
        marks their arrival (``results_fetched`` waits on it)."""
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        if not hasattr(self, "out_k_host"):
            self.out_k_host = torch.empty_like(self.out_k, device="cpu").pin_memory()
            self.out_val_host = torch.empty_like(self.out_val, device="cpu").pin_memory()
            self.out_cnt_host = torch.empty_like(self.out_cnt, device="cpu").pin_memory()
            self.fetched_event = torch.cuda.Event()
        rows = self.total_balls if rows_hint is None else int(min(max(rows_hint, 1), self.total_balls))
        with torch.cuda.stream(st):
            self.meta_host.copy_(self.meta, non_blocking=True)
            self.out_k_host[:rows * self.kstride].copy_(self.out_k[:rows * self.kstride], non_blocking=True)
            self.out_val_host[:rows * 2].copy_(self.out_val[:rows * 2], non_blocking=True)
            self.out_cnt_host[:rows].copy_(self.out_cnt[:rows], non_blocking=True)
            self.fetched_event.record(st)
        self.fetched_rows = rows

    def results_fetched(self):
        """``results()`` from the buffers ``fetch_async`` filled: waits for its event;
        rows beyond the prefix it copied (rare: more recovered keys than the hint)
        are read now."""
        self.fetched_event.synchronize()
        meta = self.meta_host.numpy()
        total = int(meta[0])
        if total > self.fetched_rows:
            a, z = self.fetched_rows, total
            self.out_k_host[a * self.kstride:z * self.kstride].copy_(self.out_k[a * self.kstride:z * self.kstride])
            self.out_val_host[a * 2:z * 2].copy_(self.out_val[a * 2:z * 2])
            self.out_cnt_host[a:z].copy_(self.out_cnt[a:z])
        return self._parse(meta, self.out_k_host.numpy(), self.out_val_host.numpy(), self.out_cnt_host.numpy())

    def collect_async(self, stream=None):
        check(self.lib.qsft_collect(ctypes.byref(self.plan), ctypes.c_void_p(self.out_k.data_ptr()),
                                    ctypes.c_void_p(self.out_val.data_ptr()), ctypes.c_void_p(self.out_cnt.data_ptr()),
                                    ctypes.c_void_p(self.out_index.data_ptr()),
                                    ctypes.c_void_p(self.out_total.data_ptr()), stream_handle(stream)),
              "qsft_collect")
        if self.U_raw is not None:   # FP64 re-projection against the raw bins (off on the parity path)
            # its scratch is a copy of the raw bins in U (free once the peeling is
            # collected), so the pristine copy serves every later collection too
            st = stream if stream is not None else torch.cuda.current_stream(self.device)
            with torch.cuda.stream(st):
                self.U.copy_(self.U_raw)
            check(self.lib.qsft_reproject(ctypes.byref(self.plan), ctypes.c_void_p(self.U.data_ptr()),
                                          ctypes.c_void_p(self.out_k.data_ptr()), ctypes.c_void_p(self.out_val.data_ptr()),
                                          ctypes.c_void_p(self.out_index.data_ptr()), stream_handle(stream)),
                  "qsft_reproject")

    def ctrl_host(self, meta=None):
        meta = self._read_meta() if meta is None else meta
        J = self.njobs
        raw = meta[1 + 2 * J:1 + 2 * J + (ctypes.sizeof(QsftCtrl) // 8) * J].tobytes()
        return [QsftCtrl.from_buffer_copy(raw, j * ctypes.sizeof(QsftCtrl)) for j in range(J)]

    def _read_meta(self):
        self.meta_host.copy_(self.meta)   # synchronises with the stream
        return self.meta_host.numpy()

    def results(self, stream=None, collected=False):
        """Per job: (keys (m, n) int64, values complex128 (m,), counts int32 (m,), ctrl).

        Two device->host copies: the metadata, then the used rows of the output.
        collected=True skips the collect launch (a captured step already did it)."""
        if not collected:
            self.collect_async(stream)
        meta = self._read_meta()
        rows = max(int(meta[0]), 1)
        return self._parse(meta, self.out_k[:rows * self.kstride].cpu().numpy(),
                           self.out_val[:rows * 2].cpu().numpy(), self.out_cnt[:rows].cpu().numpy())

    def _parse(self, meta, out_k, out_val, out_cnt):
        J = self.njobs
        total = int(meta[0])
        idx = meta[1:1 + 2 * J].reshape(-1, 2)
        ctrls = self.ctrl_host(meta)
        st = int(np.int64(meta[-1]).astype(np.int64) & 0xffffffff)
        if st != 0:
            st = st - (1 << 32) if st >= (1 << 31) else st
            raise _lib.QsftError(f"device status {st}: {self.lib.qsft_status_string(st).decode()}")
        rows = max(total, 1)
        ks = out_k[:rows * self.kstride].reshape(-1, self.kstride)
        vals = out_val[:rows * 2].reshape(-1, 2)
        cnts = out_cnt[:rows]
        self.d2h_bytes = self.meta.numel() * 8 + rows * (self.kstride + 16 + 4)
        # every row converted at once (copies: the buffers may be staging memory
        # that the next read-back overwrites), then a view per job
        v_all = vals.view(np.complex128).reshape(-1).copy()
        c_all = cnts.copy()
        n0 = self.shapes[0][1]
        same_n = not any(self.coded) and all(sh[1] == n0 for sh in self.shapes)
        k_all = ks[:, :n0].astype(np.int64) if same_n else None
        out = []
        for j, shape in enumerate(self.shapes):
            if ctrls[j].err:
                raise _lib.QsftError(f"job {j}: device table overflow during peeling")
            s, c = int(idx[j, 0]), int(idx[j, 1])
            n = shape[1]
            if same_n:
                keys = k_all[s:s + c]
            else:
                keys = ks[s:s + c, :n].astype(np.int64)
                if self.coded[j]:
                    keys += shape[0] * ks[s:s + c, n:2 * n].astype(np.int64)
            out.append((keys, v_all[s:s + c], c_all[s:s + c], ctrls[j]))
        return out

    def device_status(self):
        """The kernels' status word (a bounded wait that gave up sets QSFT_ERR_TIMEOUT)."""
        return int(self.status[0].item())


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
    autotune.ensure(q, b, prec, x.device)
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
    """Decode rows of 2ts q-ary syndrome symbols on the GPU; returns (rows, n) int64
    error values, each the integer form of its GF(q^s) element (>= q outside GF(q),
    as the reference's ReedSolomon.syndrome_decode returns them)."""
    lib = load()
    dev = torch.device("cuda", torch.cuda.current_device())
    syn = np.ascontiguousarray(np.asarray(syndromes, dtype=np.int64) % rs.q, dtype=np.uint8)
    nrows = syn.shape[0]
    gf = torch.from_numpy(rs.gf_tables()).to(dev)
    sy = torch.from_numpy(syn).to(dev)
    out = torch.zeros(max(nrows * rs.ns, 1), dtype=torch.int16, device=dev)
    check(lib.qsft_rs_decode(rs.q, rs.s, rs.t, rs.ns, ctypes.c_void_p(gf.data_ptr()), ctypes.c_void_p(sy.data_ptr()),
                             nrows, ctypes.c_void_p(out.data_ptr()), stream_handle()), "qsft_rs_decode")
    return out[:nrows * rs.ns].cpu().numpy().reshape(nrows, rs.ns).astype(np.int64)
