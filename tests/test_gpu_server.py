"""The continuous-batching loop on the GPU: every request of a serving mix gives
the same result in the mix (packed with others, several batches in flight on
separate streams) as alone, and the admission footprint is what a batch
allocates.

Tolerance: identical recovered support and iteration count; coefficients
within 1e-4 relative (the mix packs requests of other alphabets, which
changes the evaluation GEMM's K split for q in {2, 4}: FP32 rounding only).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _small_mix(count, seed):
    from qsft_gb300.server import random_mix_request
    np.random.seed(seed)
    return [random_mix_request(n_range=(8, 24), s_range=(10, 300), max_bins=1 << 14) for _ in range(count)]


def test_footprint_is_the_batch_allocation(cuda):
    from qsft_gb300.engine import Batch, workspace_bytes
    reqs = _small_mix(9, 3)
    for group in (reqs[:1], reqs[1:4], reqs):
        specs = [r.spec() for r in group]
        for prec in ("fp32", "fp64"):
            b = Batch(specs, precision=prec)
            assert b.device_bytes() == workspace_bytes(specs, prec)


def test_serving_mix_equals_alone(cuda):
    import torch
    from qsft_gb300.serve import transform_batch
    from qsft_gb300.server import GpuExecutor, Server
    reqs = _small_mix(24, 17)
    ex = GpuExecutor(max_inflight=3)
    rep = Server(ex, budget_bytes=4 << 30, max_jobs=4, max_inflight=3).run(reqs, np.zeros(len(reqs)))
    torch.cuda.synchronize()
    assert rep.completed() == len(reqs) and all(e is None for e in rep.errors)
    assert rep.max_inflight_seen == 3 and len(rep.batches) == 6
    assert any(len({reqs[i].q for i in idx}) > 1 for _, idx, _ in rep.batches)   # mixed alphabets in a batch
    for r, got in zip(reqs, rep.results):
        want = transform_batch([r])[0]
        dg, dw = got.to_dict(), want.to_dict()
        assert set(dg) == set(dw) and len(dw) > 0
        assert got.iterations == want.iterations
        ref = max(abs(v) for v in dw.values())
        assert max(abs(dg[k] - dw[k]) for k in dw) <= 1e-4 * ref
        if r.noise_sd == 0:   # noiseless: the exact support
            assert set(dw) == set(map(tuple, r.locq.T.astype(np.int64).tolist()))


def test_serving_poisson_arrivals_with_a_tight_budget(cuda):
    """Poisson arrivals and a budget of three requests' footprint: batches stay
    within it, every request completes, latencies are positive."""
    from qsft_gb300.engine import workspace_bytes
    from qsft_gb300.server import GpuExecutor, Server, poisson_arrivals
    reqs = _small_mix(40, 29)
    foot = [workspace_bytes([r.spec()]) for r in reqs]
    budget = 3 * max(foot)
    arr = poisson_arrivals(len(reqs), 4000.0, np.random.RandomState(1))
    rep = Server(GpuExecutor(max_inflight=4), budget_bytes=budget, max_jobs=8, max_inflight=4).run(reqs, arr)
    assert rep.completed() == len(reqs)
    assert rep.peak_bytes <= budget
    assert np.all(rep.latency > 0)
    p = rep.percentiles()
    assert p["p50"] <= p["p99"]
