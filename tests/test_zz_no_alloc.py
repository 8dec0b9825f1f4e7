"""qsft_peel_noalloc: the peeling loop for callers that cannot allocate device
memory (serving threads that must not stall on cudaMalloc's device-wide
synchronisation, host applications that own every buffer and give a library
only its inputs and outputs).  Called through the C ABI and checked against
the workspace path (qsft_peel_init/run/collect on a Batch) on the same bins,
twice in a row since every call reuses the library's one static scratch
array: same support, coefficients within the FP32 / FP64 tolerances of the
other parity tests, and the same control record (no table error, the same
iteration count and peel count).  This file sorts last so that a
stop-at-first-failure run has executed every other test first."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dict(keys, vals):
    return {tuple(int(x) for x in k): complex(v) for k, v in zip(keys, vals)}


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_peel_noalloc_matches_workspace_path(cuda, prec):
    import torch
    from qsft_gb300 import _lib
    from qsft_gb300.engine import Batch, precision_code
    from qsft_gb300.serve import random_request

    np.random.seed(7)
    req = random_request(4, 10, 4, 40, C=3, R=2, snr_db=20.0)     # C*B = 768 bins, n = 10
    bt = Batch([req.spec()], precision=prec)
    bt.eval()
    bt.gwht()
    bt.add_noise()
    U0 = bt.job_U(0).clone()                                       # the bins before peeling
    bt.peel()
    keys, vals, _, ctrl_ws = bt.results()[0]
    want = _dict(keys, vals)
    assert len(want) >= 38

    lib = _lib.load()
    job = _lib.QsftJob.from_buffer_copy(bytes(bt.jobs_host[0]))
    job.off_U = 0                                                  # U below is this job's bins alone
    cap = job.C * job.B + 64
    csz = ctypes.sizeof(_lib.QsftCtrl)
    for call in range(2):                                          # the static scratch is reused
        U = U0.clone()
        out_k = torch.zeros(cap * _lib.NOALLOC_KSTRIDE, dtype=torch.uint8, device=cuda)
        out_val = torch.zeros(cap * 2, dtype=torch.float64, device=cuda)
        out_cnt = torch.zeros(cap, dtype=torch.int32, device=cuda)
        out_total = torch.zeros(1, dtype=torch.int64, device=cuda)
        out_ctrl = torch.full((csz,), 0xff, dtype=torch.uint8, device=cuda)   # must be overwritten
        rc = lib.qsft_peel_noalloc(precision_code(prec), ctypes.byref(job), ctypes.c_void_p(bt.i8.data_ptr()),
                                   ctypes.c_void_p(U.data_ptr()), None, ctypes.c_void_p(out_k.data_ptr()),
                                   ctypes.c_void_p(out_val.data_ptr()), ctypes.c_void_p(out_cnt.data_ptr()),
                                   ctypes.c_void_p(out_total.data_ptr()), cap, ctypes.c_void_p(out_ctrl.data_ptr()),
                                   _lib.stream_handle())
        assert rc == 0, lib.qsft_status_string(rc)
        torch.cuda.synchronize()
        ctrl = _lib.QsftCtrl.from_buffer_copy(out_ctrl.cpu().numpy().tobytes())
        assert ctrl.err == 0, f"call {call}: device table error {ctrl.err}"
        assert ctrl.done == 1 and ctrl.iter == ctrl_ws.iter, f"call {call}: {ctrl.iter} vs {ctrl_ws.iter} iterations"
        assert ctrl.num_peeling == ctrl_ws.num_peeling
        m = int(out_total.item())
        # ball ids handed out: one per distinct k, plus any that two threads inserting
        # the same k at once allocated (left empty, skipped by the collection)
        assert ctrl.n_balls >= m
        k = out_k[:m * _lib.NOALLOC_KSTRIDE].cpu().numpy().reshape(m, -1)[:, :job.n]
        v = out_val[:2 * m].cpu().numpy().reshape(m, 2)
        got = _dict(k, v[:, 0] + 1j * v[:, 1])
        assert set(got) == set(want), f"call {call}: support differs"
        err = max(abs(got[x] - want[x]) / abs(want[x]) for x in want)
        assert err < (1e-10 if prec == "fp64" else 1e-5), f"call {call}: relative error {err:.2e}"


def test_peel_noalloc_rejects_bad_calls(cuda):
    from qsft_gb300 import _lib
    lib = _lib.load()
    job = _lib.QsftJob()
    job.q, job.n, job.b, job.C, job.R, job.P, job.B = 4, 20, 7, 3, 2, 21, 4 ** 7   # 49152 bins > 16384
    job.chan, job.src, job.max_iter = 1, 0, 15
    p = ctypes.c_void_p(16)
    rc = lib.qsft_peel_noalloc(4, ctypes.byref(job), p, p, None, p, p, p, p, 1 << 20, p, None)
    assert rc == -3   # QSFT_ERR_TOO_LARGE, before touching any pointer
    rc = lib.qsft_peel_noalloc(4, ctypes.byref(job), p, p, None, p, p, p, p, 1 << 20, None, None)
    assert rc == -1   # QSFT_ERR_ARG: the control-record output is required
