"""GWHT schedule autotuner.

Several kernels can transform rows of one (q, b) shape (the library's GWHT
schedules, ``QSFT_GWHT_*`` in ``include/qsft_gb300.h``): a CTA per row with the
whole row in shared memory, a thread-block cluster of slices per row, a
generic cluster with radix-q passes, tile passes through global memory with
large or small tiles.  Which is fastest depends on q, b, the precision and the
GPU.  ``tune`` times every valid schedule of a shape on the device -- the
transform with the device bin noise fused in, as the batched path runs it, on
rows that together exceed L2 -- selects the fastest in the library
(``qsft_gwht_select``) and caches the choice for the process.  ``ensure`` is
what :class:`~qsft_gb300.engine.Batch` calls on a shape's first use (outside a
stream capture; ``QSFT_GWHT_AUTOTUNE=0`` turns it off and keeps the built-in
rule).

The reference computes each sub-transform with scipy's ``fftn``
(qsft/utils.py:31-36, called per row from qsft/input_signal_subsampled.py:
150-153, 264-266); the choice of schedule has no counterpart there.
"""
import ctypes
import os
import threading

import numpy as np

from . import _lib

TUNE_BYTES = 256 << 20     # bins timed per schedule: more than the 129 MB L2
TUNE_REPS = 3

_CACHE = {}                # (device key, precision code, q, b) -> record
_LOCK = threading.Lock()


def _prec(precision):
    from .engine import precision_code
    return precision_code(precision)


def schedules(q, b, precision="fp32"):
    """The library's valid GWHT schedules for rows of q^b values."""
    lib = _lib.load()
    ids = (ctypes.c_int32 * 8)()
    n = lib.qsft_gwht_schedules(_prec(precision), int(q), int(b), ids, 8)
    if n < 0:
        raise _lib.QsftError(f"no GWHT schedule for q={q}, b={b}")
    return [int(ids[i]) for i in range(min(n, 8))]


def select(q, b, precision, schedule):
    _lib.check(_lib.load().qsft_gwht_select(_prec(precision), int(q), int(b), int(schedule)), "qsft_gwht_select")


def selected(q, b, precision="fp32"):
    return int(_lib.load().qsft_gwht_selected(_prec(precision), int(q), int(b)))


def pick(times_ms):
    """The fastest schedule; ties go to the lower id (the built-in order)."""
    return min(times_ms, key=lambda s: (times_ms[s], s))


def enabled():
    return os.environ.get("QSFT_GWHT_AUTOTUNE", "1") != "0"


def _device_key(device):
    import torch
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    return f"{torch.cuda.get_device_name(dev)}:{dev.index}", dev


class _DeviceTimer:
    """Times qsft_gwht_noise over rows of one shape: random bins, one job whose
    device noise is on, every row of it (row_meta = (0, row))."""

    def __init__(self, q, b, prec, dev):
        import torch
        self.torch = torch
        self.q, self.b, self.prec, self.dev = q, b, prec, dev
        B = q ** b
        es = 8 if prec == _lib.QSFT_F32 else 16
        self.nrows = max(1, -(-TUNE_BYTES // (B * es)))
        cdt = torch.complex64 if prec == _lib.QSFT_F32 else torch.complex128
        g = torch.Generator(device=dev).manual_seed(1)
        self.U = torch.randn(self.nrows * B, dtype=cdt, device=dev, generator=g)
        job = _lib.QsftJob()
        job.q, job.b, job.B = q, b, B
        job.noise_nu, job.noise_seed = 1.0, 12345
        self.jobs = torch.from_numpy(np.frombuffer(bytes(job), dtype=np.uint8).copy()).to(dev)
        self.rows = torch.arange(self.nrows, dtype=torch.int64, device=dev) * B
        meta = np.zeros((self.nrows, 2), dtype=np.int32)
        meta[:, 1] = np.arange(self.nrows)
        self.meta = torch.from_numpy(meta.ravel()).to(dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        p = _lib.QsftPlan()
        p.njobs, p.prec = 1, prec
        p.jobs, p.U, p.status = (ctypes.c_void_p(t.data_ptr()) for t in (self.jobs, self.U, self.status))
        self.plan = p

    def launch(self):
        _lib.check(_lib.load().qsft_gwht_noise(ctypes.byref(self.plan), self.q, self.b,
                                               ctypes.c_void_p(self.rows.data_ptr()),
                                               ctypes.c_void_p(self.meta.data_ptr()), self.nrows,
                                               _lib.stream_handle()), "qsft_gwht_noise")

    def __call__(self, schedule):
        torch = self.torch
        select(self.q, self.b, self.prec, schedule)
        self.launch()                                   # warm-up: attributes, first-touch
        torch.cuda.synchronize(self.dev)
        a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(TUNE_REPS):
            self.launch()
        z.record()
        z.synchronize()
        if int(self.status.item()) != 0:
            raise _lib.QsftError(f"GWHT schedule {schedule} reported device status {int(self.status.item())}")
        return a.elapsed_time(z) / TUNE_REPS


def tune(q, b, precision="fp32", device=None, timer=None):
    """Time every valid schedule of (q, b) at `precision`, select the fastest
    and cache it.  `timer(schedule) -> ms` replaces the device timing (tests).
    Returns {"schedule", "name", "times_ms", "rows"}."""
    prec = _prec(precision)
    cands = schedules(q, b, prec)
    key_dev, dev = _device_key(device) if timer is None else ("timer", None)
    t = timer if timer is not None else _DeviceTimer(q, b, prec, dev)
    times = {s: float(t(s)) for s in cands}
    best = pick(times)
    select(q, b, prec, best)
    rec = {"schedule": best, "name": _lib.GWHT_SCHEDULES.get(best, str(best)),
           "times_ms": {_lib.GWHT_SCHEDULES.get(s, str(s)): v for s, v in times.items()},
           "rows": getattr(t, "nrows", None)}
    with _LOCK:
        _CACHE[(key_dev, prec, int(q), int(b))] = rec
    return rec


def ensure(q, b, precision="fp32", device=None, timer=None):
    """Tune (q, b, precision) once per process and device; a shape with one
    valid schedule, a disabled tuner or an active stream capture (kernels may
    not be timed there) keep the selection as it is."""
    if not enabled():
        return None
    import torch
    if timer is None and torch.cuda.is_current_stream_capturing():
        return None
    prec = _prec(precision)
    key_dev = _device_key(device)[0] if timer is None else "timer"
    with _LOCK:
        rec = _CACHE.get((key_dev, prec, int(q), int(b)))
    if rec is not None:
        return rec
    if len(schedules(q, b, prec)) < 2:
        rec = {"schedule": selected(q, b, prec), "name": "only", "times_ms": {}, "rows": None}
        with _LOCK:
            _CACHE[(key_dev, prec, int(q), int(b))] = rec
        return rec
    return tune(q, b, prec, device, timer)


def table():
    """The tuned shapes: {"fp32 q=4 b=7": record, ...}."""
    with _LOCK:
        return {f"{'fp32' if p == _lib.QSFT_F32 else 'fp64'} q={q} b={b}": dict(r)
                for (_, p, q, b), r in _CACHE.items()}


def clear():
    """Forget the tuned shapes and return every shape to the built-in rule."""
    lib = _lib.load()
    with _LOCK:
        keys = list(_CACHE)
        _CACHE.clear()
    for (_, p, q, b) in keys:
        lib.qsft_gwht_select(p, q, b, 0)
