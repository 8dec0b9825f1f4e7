"""The serving mix pinned to the oracle: requests drawn like the benchmark's
serving mix (q in {2,3,4,5,20}, n in [8,60], b in [3,8], S up to q^b/4, SNR in
{10, 20, inf} dB; seed 7) run through the GPU path and through the oracle on
the same host-drawn bin noise (bench.pin_vs_oracle).  The GPU's sampling + GWHT
must give the oracle's closed-form bins, and the peeling the oracle's result:
identical support and iteration count, coefficients within relative L2 1e-5
(FP32) / 1e-10 (FP64), hence the same NMSE against the truth.

Besides the first requests of the mix, the sample holds the ten whose oracle
NMSE was worst among the first 400 of the mix (found by running the oracle on
all of them that fit, on CPU): q=20, b=3 requests at high load and 10 dB, and
small noiseless requests whose peeling stalls -- where the algorithm itself
misses NMSE 1e-4, the GPU must miss it the same way."""
import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

WORST = [247, 69, 358, 15, 344, 24, 182, 396, 65, 301]   # indices in the seed-7 mix
CAP = 1 << 22                                            # bin entries C*R*P*q^b per request


def _mix(count):
    from qsft_gb300.server import random_mix_request
    np.random.seed(7)
    return [random_mix_request() for _ in range(count)]


def _fits(r):
    return len(r.Ms) * len(r.Ds[0]) * r.Ds[0][0].shape[0] * r.q ** r.b <= CAP


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_serving_mix_matches_oracle(cuda, prec):
    import sys
    sys.path.insert(0, ROOT)
    import bench
    reqs = _mix(400)
    fit = [i for i in range(len(reqs)) if _fits(reqs[i])]
    pick = fit[:60 if prec == "fp32" else 15] + [i for i in WORST if _fits(reqs[i])]
    recs = bench.pin_vs_oracle([reqs[i] for i in pick], cuda, precision=prec, max_entries=CAP)
    assert len(recs) == len(pick)
    bad = [(pick[x["index"]], x) for x in recs if not x["same_support"] or not x["same_iterations"]]
    assert not bad, bad[:3]
    tol = 1e-10 if prec == "fp64" else 1e-5
    worst = max(recs, key=lambda x: x["coef_rel_l2"])
    assert worst["coef_rel_l2"] < tol, worst
    assert max(x["bins_rel_err"] for x in recs) < (1e-12 if prec == "fp64" else 5e-5)
    for x in recs:
        if x["noisy"] and x["nmse_oracle"] > 0:
            assert abs(x["nmse_gpu"] - x["nmse_oracle"]) <= 0.01 * x["nmse_oracle"], x
    # the hard cases are in the sample: noisy requests far above NMSE 1e-4 and a
    # noiseless one that the peeling leaves incomplete, in the oracle too
    assert max(x["nmse_oracle"] for x in recs if x["noisy"]) > 1e-2
    assert max(x["nmse_oracle"] for x in recs if not x["noisy"]) > 1e-4
