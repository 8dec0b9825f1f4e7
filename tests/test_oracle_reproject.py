"""The oracle's checker of the optional FP64 re-projection (no counterpart in
the reference): on noiseless closed-form bins, coefficients whose bins hold
no other coefficient in some group come back exactly from perturbed estimates,
and every estimate moves towards the truth."""
import numpy as np

import oracle as O


def test_reproject_recovers_isolated_coefficients():
    rs = np.random.RandomState(4)
    q, n, b, S, C = 4, 12, 5, 60, 3
    locq = rs.randint(q, size=(n, S))
    a = rs.uniform(1, 10, S) * np.exp(2j * np.pi * rs.uniform(size=S))
    Ms = [rs.randint(q, size=(n, b)) for _ in range(C)]
    D = np.vstack((np.zeros(n), np.eye(n))).astype(int)
    U = O.closed_form_bins(Ms, [D] * C, locq, a, q)
    truth = {tuple(int(x) for x in locq[:, s]): a[s] for s in range(S)}
    est = {k: v * (1 + 0.01 * (rs.randn() + 1j * rs.randn())) for k, v in truth.items()}
    new = O.reproject([U[c] for c in range(C)], Ms, [D] * C, q, est)
    err_old = sum(abs(est[k] - truth[k]) ** 2 for k in truth)
    err_new = sum(abs(new[k] - truth[k]) ** 2 for k in truth)
    assert err_new < 0.1 * err_old
    K = locq.T
    alone = 0
    for s, k in enumerate(truth):
        shared = [sum(1 for t in range(S) if t != s and all(((K[t] - K[s]) @ M) % q == 0)) for M in Ms]
        if max(shared) == 0:                      # no other coefficient in any of its bins: exact
            assert abs(new[k] - truth[k]) < 1e-9 * abs(truth[k])
            alone += 1
    assert alone >= S // 2
