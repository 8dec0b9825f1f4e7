"""Parity of the CUDA path (through the C ABI) with the oracle and with the
reference's own outputs (golden fixtures).

Tolerances: integer / index results (support sets, decoded k, bins chosen)
must be identical.  Complex values: FP64 path relative error <= 1e-10;
FP32 path relative error <= 2e-5 for samples / bins, and for recovered
coefficients relative L2 <= 1e-5 against the reference's (noiseless and noisy
alike, since the host draws the reference's noise), NMSE within 1% of the
reference's NMSE.
"""
import os

import numpy as np
import pytest

import oracle as O
from conftest import case_query_args, golden_cases, golden_dict, load_golden, transform_b

pytestmark = pytest.mark.gpu

PRECS = ["fp64", "fp32"]
REL = {"fp64": 1e-10, "fp32": 2e-5}


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("prec", PRECS)
def test_gwht_matches_reference_pins(cuda, prec):
    from qsft_gb300 import utils as U
    z = load_golden("gwht_pins")
    for key in z:
        if key.startswith("x_"):
            q, b = (int(t[1:]) for t in key[2:].split("_"))
            assert rel_err(U.gwht(z[key], q, b, precision=prec), z["y" + key[1:]]) < REL[prec], key


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("q,b", [(2, 14), (2, 15), (3, 9), (4, 7), (4, 8), (5, 6), (7, 4), (8, 5), (20, 3), (20, 4), (16, 4), (32, 3)])
def test_gwht_sizes_vs_oracle(cuda, prec, q, b):
    """Single-pass and multi-pass (rows above the shared-memory budget) transforms."""
    import torch
    from qsft_gb300.engine import gwht_device
    rs = np.random.RandomState(q * 100 + b)
    x = rs.randn(3, q ** b) + 1j * rs.randn(3, q ** b)
    t = torch.from_numpy(x).to(cuda).to(torch.complex128 if prec == "fp64" else torch.complex64)
    got = gwht_device(t, q, b).cpu().numpy()
    want = np.stack([O.gwht(r, q, b) for r in x])
    assert rel_err(got, want) < REL[prec] * (3 if q == 20 else 1)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("q,b", [(4, 11), (2, 22)])
def test_gwht_largest_rows_vs_oracle(cuda, prec, q, b):
    """Rows of q^b = 2^22 values, the largest the C ABI takes (passes through global memory)."""
    import torch
    from qsft_gb300.engine import gwht_device
    rs = np.random.RandomState(b)
    x = rs.randn(1, q ** b) + 1j * rs.randn(1, q ** b)
    t = torch.from_numpy(x).to(cuda).to(torch.complex128 if prec == "fp64" else torch.complex64)
    got = gwht_device(t, q, b).cpu().numpy()
    want = O.gwht(x[0], q, b)[None]
    assert rel_err(got, want) < REL[prec] * 3


def _small_qsft(prec, a_min, a_max, S, seed):
    import qsft_gb300 as Q
    q, n, b, C = 4, 10, 4, 3
    qa = dict(query_method="complex", num_subsample=C, delays_method_source="identity",
              subsampling_method="qsft", delays_method_channel="identity", num_repeat=1, b=b)
    np.random.seed(seed)
    sig = Q.get_random_subsampled_signal(n=n, q=q, sparsity=S, a_min=a_min, a_max=a_max, noise_sd=0.0,
                                         query_args=dict(qa), precision=prec)
    res = Q.QSFT(num_subsample=C, num_repeat=1, b=b, reconstruct_method_source="identity",
                 reconstruct_method_channel="identity").transform(sig, report=True)
    np.random.seed(seed)
    osig = O.OracleSignal(n, q, S, a_min, a_max, 0.0, dict(qa))
    want = O.OracleQSFT(num_subsample=C, num_repeat=1, b=b, reconstruct_method_source="identity",
                        reconstruct_method_channel="identity").transform(osig)
    return res, {tuple(int(x) for x in k): v for k, v in want.items()}


@pytest.mark.parametrize("prec", PRECS)
def test_zero_signal_gives_empty_result(cuda, prec):
    """Every coefficient zero: no bin passes the energy test, the loop stops after
    its first iteration and the result is empty (the report as the reference's:
    no locations, Hamming weights 0)."""
    res, want = _small_qsft(prec, 0.0, 0.0, 20, 3)
    assert want == {}
    assert res["gwht"] == {} and res["locations"] == []
    assert res["avg_hamming_weight"] == 0 and res["max_hamming_weight"] == 0


@pytest.mark.parametrize("prec", PRECS)
def test_single_coefficient(cuda, prec):
    res, want = _small_qsft(prec, 1.0, 10.0, 1, 4)
    got = res["gwht"]
    assert set(got) == set(want) and len(want) == 1
    k = next(iter(want))
    assert abs(got[k] - want[k]) <= REL[prec] * abs(want[k])


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("q,n,S", [(4, 20, 1000), (20, 10, 37), (5, 100, 50), (3, 7, 1), (2, 128, 130)])
def test_eval_points_vs_oracle(cuda, prec, q, n, S):
    from qsft_gb300.engine import eval_points_device
    rs = np.random.RandomState(n + S)
    X = rs.randint(0, q, size=(3001, n))
    K = rs.randint(0, q, size=(n, S))
    A = rs.uniform(1, 10, S) * np.exp(1j * rs.uniform(0, 2 * np.pi, S))
    got = eval_points_device(X, K.T, A, q, precision=prec).cpu().numpy()
    want = O.eval_points(X, K, A, q)
    assert rel_err(got, want) < (1e-11 if prec == "fp64" else 2e-6 * np.sqrt(S))


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("name", golden_cases(full_only=True))
def test_sampling_and_gwht_vs_reference_bins(cuda, prec, name):
    """eval_cosets + gwht of every coset against the reference's own bins."""
    import qsft_gb300 as Q
    z = load_golden(name)
    q, n, S = int(z["q"]), int(z["n"]), int(z["S"])
    np.random.seed(int(z["seed"]))
    sig = Q.get_random_subsampled_signal(n=n, q=q, sparsity=S, a_min=1, a_max=10, noise_sd=float(z["noise_sd"]),
                                         query_args=case_query_args(z), precision=prec)
    got = sig._bins[int(z["b"])].cpu().numpy()
    assert got.shape == z["Us_clean"].shape
    assert rel_err(got, z["Us_clean"]) < REL[prec]


def _run_product(z, prec, noise="host"):
    import qsft_gb300 as Q
    q, n, b, S, C, R = (int(z[k]) for k in "q n b S C R".split())
    np.random.seed(int(z["seed"]))
    sig = Q.get_random_subsampled_signal(n=n, q=q, sparsity=S, a_min=1, a_max=10, noise_sd=float(z["noise_sd"]),
                                         query_args=case_query_args(z), precision=prec, noise=noise)
    res = Q.QSFT(num_subsample=C, num_repeat=R, b=transform_b(z), reconstruct_method_source=str(z["src"]),
                 reconstruct_method_channel=str(z["ch"])).transform(sig, report=True, sort=True)
    return sig, res


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("name", golden_cases())
def test_transform_vs_reference(cuda, prec, name):
    """QSFT.transform end to end against the reference run on the same seed."""
    z = load_golden(name)
    sig, res = _run_product(z, prec)
    got, want = res["gwht"], golden_dict(z)
    assert set(got) == set(want), f"support differs: +{len(set(got) - set(want))} -{len(set(want) - set(got))}"
    l2 = np.sqrt(sum(abs(got[k] - want[k]) ** 2 for k in want) / sum(abs(v) ** 2 for v in want.values()))
    assert l2 < (1e-10 if prec == "fp64" else 1e-5), l2
    nm = O.nmse(sig.signal_w, got)
    assert abs(nm - float(z["nmse"])) <= 0.01 * float(z["nmse"]) + 1e-12
    assert res["n_samples"] == int(z["n_samples"])
    assert np.array_equal(np.asarray(res["locations"]), np.asarray(z["locations"]))
    assert res["max_hamming_weight"] == int(z["max_hamming_weight"])


def test_rs_decode_vs_oracle(cuda):
    from qsft_gb300 import ReedSolomon
    from qsft_gb300.engine import rs_decode_batch
    rng = np.random.RandomState(1)
    for (n, t, q) in [(100, 8, 5), (20, 3, 3), (10, 2, 2), (30, 3, 7), (60, 5, 11)]:
        rs = ReedSolomon(n, t, q)
        ors = O.rs.ReedSolomonOracle(n, t, q)
        D = rs.get_delay_matrix()
        rows, want = [], []
        for i in range(200):
            if i % 2 == 0:   # valid weight <= t patterns
                k = np.zeros(n, int)
                w = rng.randint(0, t + 1)
                k[rng.choice(n, w, replace=False)] = rng.randint(1, q, size=w)
                syn = ((D @ k) % q)[1:]
            else:            # arbitrary syndromes (multiton bins)
                syn = rng.randint(0, q, size=2 * t * rs.s)
            rows.append(syn)
            want.append(ors.syndrome_decode(list(syn))[0][0])
        got = rs_decode_batch(rs, np.array(rows))
        assert np.array_equal(got, np.array(want)), (n, t, q)


def test_rs_decode_values_outside_gf_q(cuda):
    """Syndromes built from error values in GF(q^s) but not in GF(q) (weight <=
    t, on the last n positions): the decoder returns those values as integers
    >= q, as ReedSolomon.syndrome_decode does (qsft/ReedSolomon.py:46-48,
    -dec_codeword[:, -ns:] of galois field elements)."""
    from qsft_gb300 import ReedSolomon
    from qsft_gb300.engine import rs_decode_batch
    rng = np.random.RandomState(2)
    for (n, t, q) in [(20, 1, 5), (40, 2, 5), (30, 3, 3), (100, 8, 5)]:
        rs = ReedSolomon(n, t, q)
        ors = O.rs.ReedSolomonOracle(n, t, q)
        gf, s = ors.gf, ors.s
        rows, want = [], []
        for _ in range(100):
            e = np.zeros(n, int)
            w = rng.randint(1, t + 1)
            e[rng.choice(n, w, replace=False)] = rng.randint(q, q ** s, size=w)   # outside GF(q)
            syn = []
            for j in range(2 * t):
                acc = 0
                for i in np.nonzero(e)[0]:
                    acc = gf.add(acc, gf.mul(int(e[i]), ors.H(j, i)))
                syn += gf.vector(acc)
            rows.append(syn)
            want.append(e)
            assert np.array_equal(ors.syndrome_decode(syn)[0][0], e)        # the oracle, as the reference
        got = rs_decode_batch(rs, np.array(rows))
        assert np.array_equal(got, np.array(want)), (n, t, q)
        assert got.max() >= q


@pytest.mark.parametrize("prec", PRECS)
def test_coded_transform_keeps_keys_outside_gf_q(cuda, prec):
    """A coded transform in which noisy multiton bins decode to error values
    outside GF(q): the reference records such a k (entries >= q) as a key of
    its own and peels it like k mod q.  The GPU result equals the oracle's
    (which returns the decoded values as the reference does), keys >= q included."""
    import qsft_gb300 as Q
    q, n, b, S, t, C, R, snr, seed = 5, 20, 3, 20, 1, 3, 1, 20, 2
    qa = dict(query_method="complex", num_subsample=C, delays_method_source="coded", subsampling_method="qsft",
              delays_method_channel="nso", num_repeat=R, b=b, t=t)
    nsd = O.noise_sd_for_snr(S, snr)
    np.random.seed(seed)
    sig = Q.get_random_subsampled_signal(n=n, q=q, sparsity=S, a_min=1, a_max=10, noise_sd=nsd, query_args=dict(qa),
                                         max_weight=t, precision=prec)
    res = Q.QSFT(num_subsample=C, num_repeat=R, b=b, reconstruct_method_source="coded",
                 reconstruct_method_channel="nso", source_decoder=Q.get_reed_solomon_dec(n, t, q)).transform(sig)
    np.random.seed(seed)
    osig = O.OracleSignal(n, q, S, 1, 10, nsd, dict(qa), max_weight=t)
    calls = {"outside": 0}
    dec = O.rs.get_reed_solomon_dec(n, t, q)

    def counting(syn):
        out = dec(syn)
        calls["outside"] += int(out[0].max(initial=0) >= q)
        return out
    ores = O.OracleQSFT(num_subsample=C, num_repeat=R, b=b, reconstruct_method_source="coded",
                        reconstruct_method_channel="nso", source_decoder=counting).transform(osig)
    want = {tuple(int(x) for x in k): v for k, v in ores.items()}
    assert calls["outside"] > 0 and any(max(k) >= q for k in want)
    assert set(res) == set(want)
    l2 = np.sqrt(sum(abs(res[k] - want[k]) ** 2 for k in want) / sum(abs(v) ** 2 for v in want.values()))
    assert l2 < (1e-10 if prec == "fp64" else 1e-5)


@pytest.mark.parametrize("prec", PRECS)
def test_coded_transform_vs_oracle(cuda, prec):
    """RS-coded delays (parity vs the oracle: the reference needs galois)."""
    import qsft_gb300 as Q
    q, n, b, S, t, C, R = 5, 40, 3, 25, 4, 3, 2
    qa = dict(query_method="complex", num_subsample=C, delays_method_source="coded", subsampling_method="qsft",
              delays_method_channel="nso", num_repeat=R, b=b, t=t)
    nsd = O.noise_sd_for_snr(S, 20)
    np.random.seed(11)
    sig = Q.get_random_subsampled_signal(n=n, q=q, sparsity=S, a_min=1, a_max=10, noise_sd=nsd, query_args=dict(qa),
                                         max_weight=t, precision=prec)
    res = Q.QSFT(num_subsample=C, num_repeat=R, b=b, reconstruct_method_source="coded",
                 reconstruct_method_channel="nso", source_decoder=Q.get_reed_solomon_dec(n, t, q)).transform(sig)
    np.random.seed(11)
    osig = O.OracleSignal(n, q, S, 1, 10, nsd, dict(qa), max_weight=t)
    ores = O.OracleQSFT(num_subsample=C, num_repeat=R, b=b, reconstruct_method_source="coded",
                        reconstruct_method_channel="nso",
                        source_decoder=O.rs.get_reed_solomon_dec(n, t, q)).transform(osig)
    want = {tuple(int(x) for x in k): v for k, v in ores.items()}
    assert set(res) == set(want)
    l2 = np.sqrt(sum(abs(res[k] - want[k]) ** 2 for k in want) / sum(abs(v) ** 2 for v in want.values()))
    assert l2 < (1e-10 if prec == "fp64" else 1e-5)
    assert set(want) == set(osig.signal_w)


def test_device_noise_statistics(cuda):
    import torch
    from qsft_gb300.engine import Batch, JobSpec
    q, n, b, C, R, P = 4, 8, 6, 2, 2, 9
    nu = 0.37
    U = torch.zeros(C, R * P, q ** b, dtype=torch.complex64, device=cuda)
    sp = JobSpec(q, n, b, np.zeros((C, n, b)), np.zeros((C, R * P, n)), R, P, U=U, noise_nu=nu, noise_seed=1234)
    bt = Batch([sp], precision="fp32")
    bt.add_noise()
    x = bt.job_U(0).cpu().numpy().ravel()
    for part in (x.real, x.imag):
        assert abs(part.mean()) < 4 * nu / np.sqrt(part.size)
        assert abs(part.std() / nu - 1) < 0.01
        z = part / nu
        assert abs(np.mean(z ** 4) - 3.0) < 0.1                        # kurtosis of the normal
        assert abs(np.mean(np.abs(z) > 3.0) - 0.0026998) < 6e-4        # two-sided 3-sigma tail mass
        from scipy import stats
        assert stats.kstest(z, "norm").statistic < 0.006               # KS distance to N(0, 1)
    assert abs(np.corrcoef(x.real, x.imag)[0, 1]) < 0.01
    bt2 = Batch([sp], precision="fp32")
    bt2.add_noise()
    assert np.array_equal(bt2.job_U(0).cpu().numpy().ravel(), x), "same seed must give the same noise"


def test_device_noise_is_one_realisation_in_fp32_and_fp64(cuda):
    """The FP32 and FP64 plans draw the same device noise (the FP32 Box-Muller
    uses hardware approximations of log and sin/cos on the same angle), so the
    batched FP32 path and the plain FP64 path see the same noisy bins."""
    import torch
    from qsft_gb300.engine import Batch, JobSpec
    q, n, b, C, R, P = 5, 6, 5, 2, 2, 7
    out = {}
    for prec, dt in (("fp32", torch.complex64), ("fp64", torch.complex128)):
        U = torch.zeros(C, R * P, q ** b, dtype=dt, device=cuda)
        sp = JobSpec(q, n, b, np.zeros((C, n, b)), np.zeros((C, R * P, n)), R, P, U=U, noise_nu=1.0, noise_seed=99)
        bt = Batch([sp], precision=prec)
        bt.add_noise()
        out[prec] = bt.job_U(0).cpu().numpy().astype(np.complex128).ravel()
    # FP32 rounding of the uniforms and the approximations: ~1e-6 of a unit normal
    d = np.abs(out["fp32"] - out["fp64"])
    assert np.quantile(d, 0.999) < 2e-5 and np.max(d) < 1e-3
    assert np.mean(d) < 2e-6


@pytest.mark.parametrize("prec", PRECS)
def test_fused_gwht_noise_equals_separate_passes(cuda, prec):
    """qsft_gwht_noise (noise added in the transform's last pass: pairs of entries
    in the row kernel, one draw per entry in the tile, cluster and multi-pass
    kernels) == qsft_gwht then qsft_add_noise_philox."""
    import torch
    from qsft_gb300.engine import Batch, JobSpec
    rng = np.random.RandomState(8)
    specs = []
    # row kernel (q in {2, 4}), one-pass tile, cluster (q=5 b=6), two passes (q=5 b=7), q=20 in registers
    for (q, b, R, P, nu) in [(4, 6, 2, 9, 0.3), (2, 9, 1, 5, 0.2), (3, 5, 2, 4, 0.25), (4, 5, 1, 3, 0.0),
                             (5, 6, 1, 7, 0.2), (5, 7, 1, 8, 0.15), (20, 3, 1, 4, 0.1), (20, 4, 1, 5, 0.05)]:
        C = 2
        U = torch.from_numpy(rng.randn(C, R * P, q ** b) + 1j * rng.randn(C, R * P, q ** b))
        n = P - 1                                   # identity source: P - 1 >= n
        specs.append(JobSpec(q, n, b, np.zeros((C, n, b)), np.zeros((C, R * P, n)), R, P, U=U, noise_nu=nu,
                             noise_seed=77 + q))
    a = Batch(specs, precision=prec)
    a.gwht(); a.add_noise()
    b_ = Batch(specs, precision=prec)
    b_.gwht_noise()
    for j in range(len(specs)):
        x, y = a.job_U(j).cpu().numpy(), b_.job_U(j).cpu().numpy()
        assert np.allclose(x, y, rtol=0, atol=1e-6 if prec == "fp32" else 1e-13), j


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("q,b", [(4, 7), (2, 13), (2, 14), (2, 15), (4, 6), (2, 10), (3, 9), (5, 6), (5, 7), (20, 3),
                                 (20, 4), (4, 8), (16, 4)])
def test_every_gwht_schedule_vs_oracle(cuda, prec, q, b, monkeypatch):
    """Each GWHT schedule the library offers for the shape (the autotuner's
    candidates) gives the reference's gwht, and its fused device noise equals
    the transform followed by the separate noise pass."""
    import torch
    from qsft_gb300 import autotune
    from qsft_gb300.engine import Batch, JobSpec, gwht_device
    monkeypatch.setenv("QSFT_GWHT_AUTOTUNE", "0")      # the explicit selections below stand
    rs = np.random.RandomState(q * 31 + b)
    x = rs.randn(2, q ** b) + 1j * rs.randn(2, q ** b)
    want = np.stack([O.gwht(r, q, b) for r in x])
    P, R, C = 3, 1, 2
    U = torch.from_numpy(rs.randn(C, R * P, q ** b) + 1j * rs.randn(C, R * P, q ** b))
    spec = JobSpec(q, P - 1, b, np.zeros((C, P - 1, b)), np.zeros((C, R * P, P - 1)), R, P, U=U, noise_nu=0.3,
                   noise_seed=5 + q)
    cands = autotune.schedules(q, b, prec)
    assert cands
    fused = []
    try:
        for s in cands:
            autotune.select(q, b, prec, s)
            t = torch.from_numpy(x).to(cuda).to(torch.complex128 if prec == "fp64" else torch.complex64)
            got = gwht_device(t, q, b).cpu().numpy()
            assert rel_err(got, want) < REL[prec] * (3 if q == 20 else 1), s
            a = Batch([spec], precision=prec)
            a.gwht(); a.add_noise()
            b_ = Batch([spec], precision=prec)
            b_.gwht_noise()
            assert np.allclose(a.job_U(0).cpu().numpy(), b_.job_U(0).cpu().numpy(), rtol=0,
                               atol=1e-5 if prec == "fp32" else 1e-13), s
            fused.append(b_.job_U(0).cpu().numpy())
    finally:
        autotune.clear()
    for f in fused[1:]:                                 # one noise realisation whatever the schedule
        assert np.allclose(f, fused[0], rtol=0, atol=1e-5 if prec == "fp32" else 1e-12)


def test_autotuner_times_every_schedule(cuda):
    """The tuner times each valid schedule of the shape on the device and
    selects the fastest."""
    from qsft_gb300 import autotune
    try:
        rec = autotune.tune(4, 7, "fp32")
        names = [autotune._lib.GWHT_SCHEDULES[s] for s in autotune.schedules(4, 7, "fp32")]
        assert sorted(rec["times_ms"]) == sorted(names)
        assert all(0 < v < 100 for v in rec["times_ms"].values())
        assert rec["times_ms"][rec["name"]] == min(rec["times_ms"].values())
        assert autotune.selected(4, 7, "fp32") == rec["schedule"]
        assert rec["rows"] * 4 ** 7 * 8 >= autotune.TUNE_BYTES
    finally:
        autotune.clear()


@pytest.mark.parametrize("prec", PRECS)
def test_fp64_reprojection_vs_oracle(cuda, prec):
    """The optional re-projection (qsft_reproject) on a noisy transform equals
    the oracle's checker applied to the same raw bins and the same peeled
    estimates; and it does not make the estimates worse against the truth."""
    import torch
    from qsft_gb300.engine import Batch
    from qsft_gb300.serve import random_request
    np.random.seed(17)
    req = random_request(4, 14, 5, 120, C=3, R=2, snr_db=10.0)
    sp = req.spec()
    sp.noise_nu = 0.0
    nu = req.noise_sd / np.sqrt(2 * 4 ** 5)
    noise = np.random.RandomState(3).normal(0, nu, (3, 2 * 15, 4 ** 5, 2)).view(np.complex128)[..., 0]
    out = []
    for rp in (False, True):
        bt = Batch([sp], precision=prec, reproject=rp)
        bt.eval(); bt.gwht()
        bt.add_bins(0, torch.from_numpy(noise))
        raw = bt.job_U(0).cpu().numpy().astype(np.complex128)
        bt.peel()
        k, v, _, _ = bt.results()[0]
        out.append((raw, {tuple(int(x) for x in kk): complex(vv) for kk, vv in zip(k, v)}))
    (raw, base), (_, got) = out
    assert set(got) == set(base) and len(base) >= 100
    Ds = [np.vstack(d) for d in req.Ds]
    want = O.reproject([raw[c] for c in range(3)], req.Ms, Ds, 4, base)
    l2 = np.sqrt(sum(abs(got[k] - want[k]) ** 2 for k in want) / sum(abs(x) ** 2 for x in want.values()))
    assert l2 < (1e-10 if prec == "fp64" else 1e-5), l2
    truth = {tuple(int(x) for x in kk): complex(a) for kk, a in zip(req.locq.T, req.strengths)}
    assert O.nmse(truth, got) <= 1.02 * O.nmse(truth, base)


def test_batch_of_mixed_shapes_equals_single_runs(cuda):
    """Jobs of different (q, n, b, C, R, P, S) in one packed batch give the
    same results as each alone."""
    from qsft_gb300.engine import Batch, JobSpec
    rng = np.random.RandomState(5)
    specs = []
    for (q, n, b, S, R, ch) in [(4, 12, 5, 60, 2, "nso"), (3, 9, 4, 20, 1, "identity"), (20, 6, 2, 30, 3, "nso"),
                                (2, 16, 8, 40, 2, "nso")]:
        C = 3
        locq = rng.randint(0, q, size=(S, n))
        A = rng.uniform(1, 10, S) * np.exp(1j * rng.uniform(0, 2 * np.pi, S))
        M = rng.randint(0, q, size=(C, n, b))
        Dsrc = np.vstack((np.zeros(n), np.eye(n))).astype(int)
        if ch == "nso":
            offs = rng.randint(0, q, size=(R, n))
            D1 = np.vstack([(o - Dsrc) % q for o in offs])
        else:
            D1 = Dsrc
        D = np.stack([D1] * C)
        nu = 0.05 if ch == "nso" else 0.0
        cutoff = 1e-9 + 1.5 * 2 * nu ** 2      # qsft/qsft.py:125 with sigma^2 / q^b = 2 nu^2
        specs.append(JobSpec(q, n, b, M, D, R, n + 1, chan=ch, K=locq, A=A, cutoff=cutoff,
                             noise_nu=nu, noise_seed=99 + q))
    outs = []
    for sp in specs:
        bt = Batch([sp], precision="fp32")
        bt.eval(); bt.gwht(); bt.add_noise(); bt.peel()
        outs.append(bt.results()[0])
    bt = Batch(specs, precision="fp32")
    bt.eval(); bt.gwht_noise(); bt.peel()      # transform and noise fused in one pass
    mixed = bt.results()
    for (k1, v1, _, c1), (k2, v2, _, c2) in zip(outs, mixed):
        d1 = {tuple(k): v for k, v in zip(k1, v1)}
        d2 = {tuple(k): v for k, v in zip(k2, v2)}
        assert set(d1) == set(d2) and len(d1) > 0
        assert max(abs(d1[k] - d2[k]) for k in d1) < 1e-5
        assert c1.iter == c2.iter


def _random_spec(rng, q, n, b, S, C, R, chan="nso"):
    from qsft_gb300.engine import JobSpec
    locq = rng.randint(0, q, size=(S, n))
    A = rng.uniform(1, 10, S) * np.exp(1j * rng.uniform(0, 2 * np.pi, S))
    M = rng.randint(0, q, size=(C, n, b))
    Dsrc = np.vstack((np.zeros(n), np.eye(n))).astype(int)
    offs = rng.randint(0, q, size=(R, n))
    D1 = np.vstack([(o - Dsrc) % q for o in offs])
    return JobSpec(q, n, b, M, np.stack([D1] * C), R, n + 1, chan=chan, K=locq, A=A, cutoff=1e-3)


@pytest.mark.parametrize("shapes", [
    [(4, 20, 7, 1000, 3, 2)],                      # the benchmark shape, q=4 fast path, K=32
    [(2, 16, 9, 300, 3, 2)],                       # q=2 fast path
    [(20, 10, 3, 37, 3, 3)],                       # runtime q, rows not a multiple of 128
    [(3, 40, 5, 700, 2, 1)],                       # K=64
    [(5, 100, 3, 50, 3, 1)],                       # K=128
    [(20, 10, 3, 1500, 2, 1)],                     # support split over several chunks
    [(3, 12, 9, 200, 2, 1)],                       # runtime q with b > 8: four words of digits
    [(4, 12, 5, 60, 3, 2), (3, 9, 4, 20, 3, 1), (20, 6, 2, 30, 3, 3), (2, 16, 8, 40, 3, 2)],  # mixed batch
])
@pytest.mark.parametrize("method", ["gemm", "tc"])
def test_eval_tensor_cores_vs_cuda_cores_and_oracle(cuda, shapes, method):
    """tcgen05 coset evaluation (coset-factored GEMM, or dot products + lookup)
    == CUDA-core evaluation == oracle (FP32 tolerance)."""
    from qsft_gb300.engine import Batch
    rng = np.random.RandomState(len(shapes) * 7 + shapes[0][0])
    specs = [_random_spec(rng, *sh) for sh in shapes]
    bt = Batch(specs, precision="fp32")
    assert bt.gm_ok
    bt.U.fill_(float("nan"))     # every sample must be written
    bt.eval(method=method)
    tc = [bt.job_U(j).cpu().numpy().copy() for j in range(len(specs))]
    assert bt.device_status() == 0
    bt.eval(method="cuda")
    cc = [bt.job_U(j).cpu().numpy().copy() for j in range(len(specs))]
    for sp, a, c in zip(specs, tc, cc):
        scale = np.abs(c).max()
        assert np.all(np.isfinite(a))
        assert np.max(np.abs(a - c)) / scale < 2e-6 * np.sqrt(sp.S)
        # oracle on one coset row of each group
        for g in range(sp.C):
            X = O.coset_points(sp.M[g], sp.D[g][0], sp.q).T
            want = O.eval_points(X, sp.K.T, sp.A, sp.q)
            assert rel_err(a[g, 0], want) < 2e-6 * np.sqrt(sp.S)


def test_transform_batch_replays_new_inputs(cuda):
    """transform_batch captures one CUDA graph per layout; a second batch with
    the same layout but different inputs must give the results of a direct run."""
    from qsft_gb300.engine import Batch
    from qsft_gb300.serve import random_request, transform_batch
    np.random.seed(21)
    reqs_a = [random_request(4, 12, 5, 60, C=3, R=2, snr_db=20.0) for _ in range(3)]
    reqs_b = [random_request(4, 12, 5, 60, C=3, R=2, snr_db=20.0) for _ in range(3)]
    out_a = transform_batch(reqs_a)
    out_b = transform_batch(reqs_b)
    for reqs, out in ((reqs_a, out_a), (reqs_b, out_b)):
        bt = Batch([r.spec() for r in reqs], precision="fp32")
        bt.step()
        direct = bt.results(collected=True)
        for (k, v, _, _), res in zip(direct, out):
            d1 = {tuple(x): y for x, y in zip(k.tolist(), v)}
            d2 = {tuple(x): y for x, y in zip(res.keys.tolist(), res.values)}
            assert set(d1) == set(d2) and len(d1) > 0
            assert max(abs(d1[x] - d2[x]) for x in d1) < 1e-5
        truth = [set(map(tuple, r.locq.T.tolist())) for r in reqs]
        assert all(len(set(map(tuple, res.keys.tolist())) & t) >= 58 for res, t in zip(out, truth))


@pytest.mark.parametrize("prec", PRECS)
def test_config4_coded_full_size(cuda, prec):
    """q=5, n=100, b=5, C=3, RS-coded delays t=8, S=200 of Hamming weight <= 8,
    20 dB, at full size: the oracle on the same seed (same signal, query design,
    permutation and host noise) gives the same support and coefficients
    (relative L2 1e-5 FP32, 1e-10 FP64), and both recover the true support."""
    import os
    import qsft_gb300 as Q
    q, n, b, S, t = 5, 100, 5, 200, 8
    qa = dict(query_method="complex", num_subsample=3, delays_method_source="coded", subsampling_method="qsft",
              delays_method_channel="nso", num_repeat=1, b=b, t=t)
    nsd = O.noise_sd_for_snr(S, 20)
    np.random.seed(0)
    sig = Q.get_random_subsampled_signal(n=n, q=q, sparsity=S, a_min=1, a_max=10, noise_sd=nsd,
                                         query_args=dict(qa), max_weight=t, precision=prec)
    res = Q.QSFT(num_subsample=3, num_repeat=1, b=b, reconstruct_method_source="coded", reconstruct_method_channel="nso",
                 source_decoder=Q.get_reed_solomon_dec(n, t, q)).transform(sig, report=True)
    np.random.seed(0)
    osig = O.OracleSignal(n, q, S, 1, 10, nsd, dict(qa), max_weight=t, eval_threads=os.cpu_count() or 1)
    ores = O.OracleQSFT(num_subsample=3, num_repeat=1, b=b, reconstruct_method_source="coded",
                        reconstruct_method_channel="nso",
                        source_decoder=O.rs.get_reed_solomon_dec(n, t, q)).transform(osig)
    want = {tuple(int(x) for x in k): v for k, v in ores.items()}
    assert set(res["gwht"]) == set(want)
    l2 = np.sqrt(sum(abs(res["gwht"][k] - want[k]) ** 2 for k in want) / sum(abs(v) ** 2 for v in want.values()))
    assert l2 < (1e-10 if prec == "fp64" else 1e-5), l2
    assert set(res["gwht"]) == set(sig.signal_w)
    assert O.nmse(sig.signal_w, res["gwht"]) < 1e-4
    assert res["n_samples"] == 3 * sig.get_source_parity() * q ** b
    assert res["max_hamming_weight"] <= t


def test_folder_cache_round_trip(cuda, tmp_path):
    """folder=: Ms/Ds and the sub-transforms are saved on the first build and
    loaded on the second (qsft/input_signal_subsampled.py:92-155)."""
    import qsft_gb300 as Q
    qa = dict(query_method="complex", num_subsample=3, delays_method_source="identity", subsampling_method="qsft",
              delays_method_channel="nso", num_repeat=2, b=4)
    out = []
    for _ in range(2):
        np.random.seed(3)
        sig = Q.get_random_subsampled_signal(n=10, q=4, sparsity=30, a_min=1, a_max=10, noise_sd=0.5,
                                             query_args=dict(qa), folder=str(tmp_path))
        np.random.seed(99)
        out.append(Q.QSFT(num_subsample=3, num_repeat=2, b=4, reconstruct_method_source="identity",
                          reconstruct_method_channel="nso").transform(sig))
    assert (tmp_path / "Ms_and_Ds.pickle").is_file()
    assert set(out[0]) == set(out[1]) and len(out[0]) >= 28
    assert max(abs(out[0][k] - out[1][k]) for k in out[0]) < 1e-6


def _ref_save(obj, path):
    """The reference's cache writer (qsft/utils.py:189-192): zlib level 9 of a pickle."""
    import pickle
    import zlib
    path.parent.mkdir(parents=True, exist_ok=True)
    path.write_bytes(zlib.compress(pickle.dumps(obj, pickle.HIGHEST_PROTOCOL), 9))


def _ref_load(path):
    import pickle
    import zlib
    return pickle.loads(zlib.decompress(path.read_bytes()))


@pytest.mark.parametrize("prec", PRECS)
def test_folder_in_reference_format(cuda, tmp_path, prec):
    """A folder laid out as the reference fills it -- Ms_and_Ds.pickle,
    transforms/U{i}_{j}.pickle = (Us[i][j], transformTimes[i][j]) with
    Us[i][j] = {b: (P, q^b) bins} (qsft/input_signal_subsampled.py:92-155) --
    is loaded without sampling, and the transform gives the oracle's result on
    those bins; a folder filled here has the same files and contents."""
    import qsft_gb300 as Q
    q, n, b, S, C, R = 4, 10, 4, 30, 3, 2
    qa = dict(query_method="complex", num_subsample=C, delays_method_source="identity", subsampling_method="qsft",
              delays_method_channel="nso", num_repeat=R, b=b)
    np.random.seed(21)
    osig = O.OracleSignal(n, q, S, 1, 10, 0.5, dict(qa))
    ref_dir = tmp_path / "ref"
    _ref_save((osig.Ms, osig.Ds), ref_dir / "Ms_and_Ds.pickle")
    for i in range(C):
        for j in range(R):
            _ref_save(({b: osig.Us[i][j]}, {b: 0.01}), ref_dir / "transforms" / f"U{i}_{j}.pickle")

    class NoSampling(Q.SyntheticSubsampledSignal):
        def _sample_device(self):
            raise AssertionError("the cached transforms must be used")

    np.random.seed(21)
    _, locq, strengths = Q.generate_signal_w(n, q, S, 1, 10, full=False)
    sig = NoSampling(signal_w=None, locq=locq, strengths=strengths, noise_sd=0.5, n=n, q=q, query_args=dict(qa),
                     folder=str(ref_dir), precision=prec)
    np.random.seed(5)
    got = Q.QSFT(num_subsample=C, num_repeat=R, b=b, reconstruct_method_source="identity",
                 reconstruct_method_channel="nso").transform(sig)
    np.random.seed(5)
    want = O.OracleQSFT(num_subsample=C, num_repeat=R, b=b, reconstruct_method_source="identity",
                        reconstruct_method_channel="nso").transform(osig)
    want = {tuple(int(x) for x in k): v for k, v in want.items()}
    assert set(got) == set(want) and len(want) >= 25
    assert max(abs(got[k] - want[k]) / abs(want[k]) for k in want) < (1e-10 if prec == "fp64" else 1e-5)
    assert sig.transformTimes[0][0][b] == 0.01
    # written here: the reference's files, same layout and values
    out_dir = tmp_path / "ours"
    np.random.seed(21)
    mine = Q.get_random_subsampled_signal(n=n, q=q, sparsity=S, a_min=1, a_max=10, noise_sd=0.5, query_args=dict(qa),
                                          folder=str(out_dir), precision=prec)
    Ms, Ds = _ref_load(out_dir / "Ms_and_Ds.pickle")
    assert all(np.array_equal(x, y) for x, y in zip(Ms, osig.Ms))
    for i in range(C):
        for j in range(R):
            us, ts = _ref_load(out_dir / "transforms" / f"U{i}_{j}.pickle")
            assert set(us) == {b} and set(ts) == {b} and us[b].shape == (n + 1, q ** b)
            assert us[b].dtype == np.complex128
            assert rel_err(us[b], osig.Us[i][j]) < REL[prec]
            smp = _ref_load(out_dir / "samples" / f"M{i}_D{j}.pickle")
            assert smp.shape == (n + 1, q ** b)
    assert mine._bins[b].shape == (C, R, n + 1, q ** b)


def test_generic_plugin_subsample(cuda):
    """A user SubsampledSignal that only implements subsample(query_indices) on
    the host: sub-transforms and peeling on the GPU give the synthetic path's result."""
    import qsft_gb300 as Q
    from qsft_gb300.utils import dec_to_qary_vec

    class HostSignal(Q.SubsampledSignal):
        def __init__(self, locq, strengths, **kw):
            self.locq, self.strengths = locq, strengths
            self.noise_sd = kw["noise_sd"]     # read by transform's cutoff (qsft/qsft.py:125)
            super().__init__(**kw)

        def subsample(self, query_indices):
            X = dec_to_qary_vec(np.asarray(query_indices), self.q, self.n).T
            return np.exp(2j * np.pi * (X @ self.locq) / self.q) @ self.strengths

    qa = dict(query_method="complex", num_subsample=3, delays_method_source="identity", subsampling_method="qsft",
              delays_method_channel="identity", num_repeat=1, b=4)
    np.random.seed(12)
    syn = Q.get_random_subsampled_signal(n=9, q=4, sparsity=25, a_min=1, a_max=10, noise_sd=0.0, query_args=dict(qa))
    np.random.seed(12)
    _, locq, strengths = Q.generate_signal_w(9, 4, 25, 1, 10, full=False)
    host = HostSignal(locq, strengths, n=9, q=4, noise_sd=0.0, query_args=dict(qa))
    host.Ms, host.Ds = syn.Ms, syn.Ds          # same query design (drawn once)
    host._subsample_qsft()
    res = []
    for sig in (syn, host):
        np.random.seed(5)
        res.append(Q.QSFT(num_subsample=3, num_repeat=1, b=4, reconstruct_method_source="identity",
                          reconstruct_method_channel="identity").transform(sig))
    assert set(res[0]) == set(res[1]) == set(syn.signal_w)
    assert max(abs(res[0][k] - res[1][k]) for k in res[0]) < 1e-4


def test_test_nmse_matches_reference(cuda):
    """The GPU time-domain test NMSE == the reference's _test_qary on the same inputs."""
    from qsft_gb300.test_helper import test_nmse
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "test_qary_pins.npz"))
    for tag in ("q4_n10", "q3_n12", "q2_n20"):
        q, n = int(tag[1:tag.index("_")]), int(tag.split("_n")[1])
        beta = {tuple(int(x) for x in k): v for k, v in zip(z[f"{tag}_keys"], z[f"{tag}_vals"])}
        got = test_nmse(beta, z[f"{tag}_idx"], z[f"{tag}_samples"], q, n)
        assert abs(got - float(z[f"{tag}_nmse"])) <= 1e-9 * float(z[f"{tag}_nmse"])
    assert test_nmse({}, [0], [1.0], 4, 3) == 1


def test_test_helper_end_to_end(cuda, tmp_path):
    """TestHelper with a synthetic signal: train on coset samples (QSFT on the GPU),
    test on uniform noiseless samples; the NMSE equals the oracle's on the same
    recovered transform and is small at 20 dB."""
    import qsft_gb300 as Q
    from qsft_gb300.test_helper import TestHelper

    class Synthetic(TestHelper):
        def __init__(self, *a, **k):
            np.random.seed(4)
            sa = a[0]
            _, self.locq, self.strengths = Q.generate_signal_w(sa["n"], sa["q"], sa["sparsity"], 1, 10, full=False)
            super().__init__(*a, **k)

        def generate_signal(self, signal_args):
            args = dict(signal_args)
            return Q.SyntheticSubsampledSignal(signal_w=None, locq=self.locq, strengths=self.strengths,
                                               noise_sd=args.get("noise_sd", 0.0), n=args["n"], q=args["q"],
                                               query_args=args["query_args"], folder=args["folder"])

    S = 30
    sa = dict(n=12, q=4, sparsity=S, noise_sd=O.noise_sd_for_snr(S, 20))
    th = Synthetic(sa, ["qsft"], dict(num_subsample=3, num_repeat=2, b=5), dict(n_samples=3000), tmp_path)
    np.random.seed(9)
    beta = th.compute_model("qsft", dict(num_subsample=3, num_repeat=2, b=5, noise_sd=sa["noise_sd"]))
    nmse = th.test_model("qsft", beta=beta)
    ts = th.test_signal.signal_t
    want = O.test_qary_nmse(beta, list(ts.keys()), list(ts.values()), 4, 12)
    assert abs(nmse - want) <= 1e-9 * max(want, 1e-12)
    assert nmse < 1e-2 and len(beta) >= S - 2


def test_transform_stream_matches_transform_batch(cuda):
    """Pipelined TransformStream (ring of captured workspaces per layout, async
    read-back) returns what transform_batch returns, for interleaved layouts and
    more submissions in flight than the ring holds."""
    from qsft_gb300.serve import TransformStream, random_request, transform_batch
    np.random.seed(31)
    groups = [[random_request(4, 12, 5, 60, C=3, R=2, snr_db=20.0) for _ in range(3)] for _ in range(3)]
    groups += [[random_request(2, 14, 8, 40, C=3, R=2, snr_db=20.0) for _ in range(2)] for _ in range(2)]
    ts = TransformStream(depth=2)
    tickets = [ts.submit(g) for g in groups]          # 5 submissions, rings of 2: early collection
    got = [ts.result(t) for t in reversed(tickets)][::-1]
    for g, res in zip(groups, got):
        want = transform_batch(g)
        for a, b in zip(res, want):
            da, db = a.to_dict(), b.to_dict()
            assert set(da) == set(db) and len(da) > 0
            assert max(abs(da[k] - db[k]) for k in da) < 1e-6
            assert a.iterations == b.iterations
    with pytest.raises(KeyError):
        ts.result(tickets[0])
