"""The peeling loop as one persistent cooperative launch (qsft_peel_persistent):
the same results as the launch-per-phase path, which the other tests pin to
the reference -- identical support and iteration counts, coefficients within
the FP32 / FP64 tolerances -- on a batch of the benchmark's shape, a batch of
mixed shapes and a Reed-Solomon-coded job; the same inside a captured CUDA
graph; and its bounded grid-barrier wait: when it runs out (a test flag makes
every barrier wait for one block more than the grid has) the kernel returns
and reports QSFT_ERR_TIMEOUT, and the GPU context stays usable."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _specs(kind):
    from qsft_gb300.serve import random_request
    from qsft_gb300.server import random_mix_request
    np.random.seed(31)
    if kind == "bench":
        return [random_request(4, 20, 7, 1000, C=3, R=2, snr_db=10.0).spec() for _ in range(4)]
    if kind == "mixed":
        return [random_mix_request(max_bins=1 << 14).spec() for _ in range(12)]
    return [random_request(5, 40, 3, 25, C=3, R=2, snr_db=20.0, src="coded", t=4, max_weight=4).spec()
            for _ in range(3)]


def _run(specs, prec, mode, capture=False):
    import torch
    from qsft_gb300.engine import Batch
    b = Batch(specs, precision=prec, peel_mode=mode)
    if capture:
        b.capture()
        b.run()
        torch.cuda.synchronize()
        return b.results(collected=True)
    b.step()
    return b.results(collected=True)


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("kind", ["bench", "mixed", "coded"])
def test_persistent_loop_equals_launch_per_phase(cuda, prec, kind):
    specs = _specs(kind)
    want = _run(specs, prec, "graph")
    for capture in (False, True):
        got = _run(specs, prec, "persistent", capture)
        for (k0, v0, _, c0), (k1, v1, _, c1) in zip(want, got):
            d0 = {tuple(x): y for x, y in zip(k0.tolist(), v0)}
            d1 = {tuple(x): y for x, y in zip(k1.tolist(), v1)}
            assert set(d0) == set(d1)
            assert int(c0.iter) == int(c1.iter) and int(c0.num_peeling) == int(c1.num_peeling)
            if d0:
                l2 = np.sqrt(sum(abs(d0[x] - d1[x]) ** 2 for x in d0) / sum(abs(y) ** 2 for y in d0.values()))
                assert l2 < (1e-10 if prec == "fp64" else 1e-5)


def test_persistent_barrier_timeout_is_reported(cuda):
    import torch
    from qsft_gb300 import _lib
    from qsft_gb300.engine import Batch
    specs = _specs("bench")[:2]
    b = Batch(specs, peel_mode="persistent")
    b.eval(); b.gwht_noise()
    b.plan.flags |= _lib.PLAN_TEST_BARRIER_TIMEOUT        # every barrier waits for a block that never comes
    b.peel()
    b.collect_async()
    torch.cuda.synchronize()
    assert b.device_status() == -5                          # QSFT_ERR_TIMEOUT, read from the device
    with pytest.raises(_lib.QsftError):
        b.results(collected=True)
    # the context is still usable: a fresh batch runs and agrees with the other path
    got = _run(specs, "fp32", "persistent")
    want = _run(specs, "fp32", "graph")
    assert all(set(map(tuple, g[0].tolist())) == set(map(tuple, w[0].tolist())) for g, w in zip(got, want))
