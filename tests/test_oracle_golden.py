"""The oracle (a numpy restatement of the reference) against fixtures produced
by running the reference itself (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

import oracle as O
from conftest import case_query_args, golden_cases, golden_dict, load_golden, transform_b


@pytest.mark.parametrize("name", golden_cases(full_only=True))
def test_oracle_matches_reference(name):
    z = load_golden(name)
    q, n, b, S, C, R = (int(z[k]) for k in "q n b S C R".split())
    np.random.seed(int(z["seed"]))
    sig = O.OracleSignal(n, q, S, 1, 10, float(z["noise_sd"]), case_query_args(z))
    # RNG-ordered inputs are identical
    assert np.array_equal(sig.locq, z["locq"])
    assert np.array_equal(np.array(sig.Ms), z["Ms"])
    assert np.array_equal(np.array(sig.Ds[0]), z["Ds"])
    # bins before noise: bit-identical to the reference's
    Uc = np.array([[u for u in row] for row in sig.Us])
    assert np.array_equal(Uc, z["Us_clean"])
    trace = []
    res = O.OracleQSFT(num_subsample=C, num_repeat=R, reconstruct_method_source=str(z["src"]),
                       reconstruct_method_channel=str(z["ch"]), b=b).transform(sig, report=True, trace=trace)
    got = {tuple(int(x) for x in k): v for k, v in res["gwht"].items()}
    want = golden_dict(z)
    assert set(got) == set(want)
    assert max(abs(got[k] - want[k]) for k in want) < 1e-12
    # every singleton_detection call returned the same k, in the same order
    assert np.array_equal(np.concatenate(trace), z["detect_k"])
    assert res["n_samples"] == int(z["n_samples"])
    assert abs(O.nmse(sig.signal_w, res["gwht"]) - float(z["nmse"])) <= 1e-9 + 1e-6 * float(z["nmse"])


@pytest.mark.parametrize("name", golden_cases(full_only=True))
def test_oracle_query_and_eval_pins(name):
    z = load_golden(name)
    if z["query_dec_g0r0"].size == 0:
        pytest.skip("q^n too large for int64 decimals")
    q, n = int(z["q"]), int(z["n"])
    M, D0 = z["Ms"][0], z["Ds"][0]
    dec = np.array([[int(v) for v in O.qary_vec_to_dec(O.coset_points(M, d, q), q)] for d in D0])
    assert np.array_equal(dec, z["query_dec_g0r0"])
    X = O.dec_to_qary_vec(list(z["eval_idx"]), q, n).T
    f = O.eval_points(X, z["locq"], z["strengths"], q)
    assert np.allclose(f, z["eval_vals"], rtol=0, atol=1e-10)


def test_oracle_gwht_pins():
    z = load_golden("gwht_pins")
    for key in z:
        if not key.startswith("x_"):
            continue
        q, b = (int(t[1:]) for t in key[2:].split("_"))
        assert np.array_equal(O.gwht(z[key], q, b), z["y" + key[1:]])


@pytest.mark.parametrize("name", ["cfg2_q4n20b7_nso_10db", "cfg3_q20n10b3_nso_20db"])
def test_golden_large_configs_are_consistent(name):
    """The full-size fixtures: the reference recovered the support within the
    stated accuracy, and the stored inputs regenerate from the seed."""
    z = load_golden(name)
    q, n, b, S, C = (int(z[k]) for k in "q n b S C".split())
    np.random.seed(int(z["seed"]))
    w, locq, a = O.generate_signal_w(n, q, S, 1, 10)
    assert np.array_equal(locq, z["locq"])
    assert np.allclose(a, z["strengths"], rtol=0, atol=0)
    Ms = O.get_Ms(n, b, q, C, "complex")
    assert np.array_equal(np.array(Ms), z["Ms"])
    assert float(z["nmse"]) < 1e-4
    assert len(z["gwht_keys"]) >= S - 2


def test_rs_oracle_round_trips():
    rng = np.random.RandomState(0)
    for (n, t, q) in [(100, 8, 5), (20, 3, 3), (10, 2, 2), (30, 3, 7), (4, 1, 5), (60, 5, 11)]:
        rs = O.rs.ReedSolomonOracle(n, t, q)
        D = np.array(rs.get_delay_matrix())
        assert D.shape == (2 * t * rs.s + 1, n)
        for _ in range(25):
            w = rng.randint(0, t + 1)
            k = np.zeros(n, int)
            k[rng.choice(n, w, replace=False)] = rng.randint(1, q, size=w)
            dec, _ = rs.syndrome_decode(list(((D @ k) % q)[1:]))
            assert np.array_equal(dec[0], k)


def test_gf_tables_are_fields():
    for (p, m) in O.rs.CONWAY:
        g = O.rs.GF(p, m)
        assert g.poly == O.rs.CONWAY[(p, m)], "Conway polynomial not primitive"
        assert sorted(g.exp[:g.order - 1]) == list(range(1, g.order))


def test_oracle_all_bs_matches_reference():
    """all_bs: the signal is sampled at b=5 and transformed at b=4 from every
    4th sample (qsft/input_signal_subsampled.py:150-153, 264-266)."""
    z = load_golden("q4n10b5_allbs_b4_nso")
    np.random.seed(int(z["seed"]))
    sig = O.OracleSignal(int(z["n"]), int(z["q"]), int(z["S"]), 1, 10, float(z["noise_sd"]), case_query_args(z))
    res = O.OracleQSFT(num_subsample=int(z["C"]), num_repeat=int(z["R"]), reconstruct_method_source="identity",
                       reconstruct_method_channel="nso", b=transform_b(z)).transform(sig, report=True)
    got = {tuple(int(x) for x in k): v for k, v in res["gwht"].items()}
    want = golden_dict(z)
    assert set(got) == set(want)
    assert max(abs(got[k] - want[k]) for k in want) < 1e-12
    assert res["n_samples"] == int(z["n_samples"])


def test_oracle_test_qary_matches_reference():
    """TestHelper._test_qary (qsft/test_helper.py:235-260) restated, against the
    reference's own NMSE on the same recovered transform and test points."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "test_qary_pins.npz"))
    for tag in ("q4_n10", "q3_n12", "q2_n20"):
        q, n = int(tag[1:tag.index("_")]), int(tag.split("_n")[1])
        beta = {tuple(int(x) for x in k): v for k, v in zip(z[f"{tag}_keys"], z[f"{tag}_vals"])}
        got = O.test_qary_nmse(beta, z[f"{tag}_idx"], z[f"{tag}_samples"], q, n)
        assert abs(got - float(z[f"{tag}_nmse"])) <= 1e-12 * float(z[f"{tag}_nmse"])
    assert O.test_qary_nmse({}, [0], [1.0], 4, 3) == 1
