"""Host-side logic of the package against the oracle (no GPU): RNG-ordered
signal / query generation, the Reed-Solomon construction, codecs."""
import numpy as np
import pytest

import oracle as O
import qsft_gb300 as Q
from qsft_gb300 import synthetic_signal as SS
from qsft_gb300 import utils as U


@pytest.mark.parametrize("src,ch,R", [("identity", "identity", 1), ("identity", "nso", 2), ("coded", "nso", 2)])
def test_query_design_matches_oracle(src, ch, R):
    qa = dict(query_method="complex", num_subsample=3, b=3, delays_method_source=src,
              delays_method_channel=ch, num_repeat=R, t=3)
    np.random.seed(7)
    Ms, Ds = Q.get_Ms_and_Ds(20, 5, **qa)
    np.random.seed(7)
    oMs, oDs = O.get_Ms_and_Ds(20, 5, **qa)
    assert all(np.array_equal(a, b) for a, b in zip(Ms, oMs))
    assert all(np.array_equal(np.array(a), np.array(b)) for a, b in zip(Ds, oDs))


def test_simple_query_method():
    Ms = Q.get_Ms(12, 4, 3, num_to_get=3, method="simple")
    assert np.array_equal(Ms[2][:4], np.eye(4)) and np.array_equal(Ms[0][8:], np.eye(4))
    with pytest.raises(ValueError):
        Q.get_Ms(12, 4, 3, num_to_get=4, method="simple")


@pytest.mark.parametrize("mw", [None, 4])
def test_generate_signal_matches_oracle(mw):
    np.random.seed(3)
    w, locq, a = SS.generate_signal_w(30, 5, 40, 1, 10, full=False, max_weight=mw)
    np.random.seed(3)
    ow, olocq, oa = O.generate_signal_w(30, 5, 40, 1, 10, max_weight=mw)
    assert np.array_equal(locq, olocq) and np.array_equal(a, oa)


@pytest.mark.parametrize("n,t,q", [(100, 8, 5), (20, 3, 3), (10, 2, 2), (30, 3, 7), (4, 1, 5), (60, 5, 11)])
def test_rs_construction_matches_oracle(n, t, q):
    rs = Q.ReedSolomon(n, t, q)
    ors = O.rs.ReedSolomonOracle(n, t, q)
    assert rs.s == ors.s
    assert np.array_equal(rs.get_delay_matrix(), np.array(ors.get_delay_matrix()))
    f = rs.field
    og = ors.gf
    assert list(f.exp[:f.order - 1]) == og.exp[:og.order - 1]
    # Zech logarithms: alpha^z = 1 + alpha^k
    for k in range(f.order - 1):
        z = f.zech[k]
        s = og.add(1, og.exp[k])
        assert (z < 0 and s == 0) or og.exp[z] == s


def test_rs_rejects_non_field():
    with pytest.raises(ValueError):
        Q.get_reed_solomon_dec(20, 2, 15)   # 15 is in the reference's "prime" list
    with pytest.raises(NotImplementedError):
        Q.get_reed_solomon_dec(20, 2, 4)


def test_codecs():
    q, n = 7, 9
    idx = np.random.RandomState(0).randint(0, q ** n, size=100)
    X = U.dec_to_qary_vec(idx, q, n)
    assert np.array_equal(X, O.dec_to_qary_vec(list(idx), q, n))
    assert list(U.qary_vec_to_dec(X, q)) == list(idx)
    big = [3 ** 60 - 1, 12345678901234567890123]
    assert np.array_equal(U.dec_to_qary_vec(np.array(big, dtype=object), 3, 60), O.dec_to_qary_vec(big, 3, 60))
    assert np.array_equal(U.qary_ints(3, 4), O.qary_ints(3, 4))


def test_jobspec_rejects_what_the_kernels_cannot_take():
    import pytest
    from qsft_gb300.engine import JobSpec
    M, D = np.zeros((1, 4, 2)), np.zeros((1, 5, 4))
    with pytest.raises(ValueError):
        JobSpec(1, 4, 2, M, D, 1, 5)                        # q < 2
    with pytest.raises(ValueError):
        JobSpec(33, 4, 2, M, D, 1, 5)                       # q above 32
    with pytest.raises(ValueError):
        JobSpec(2, 4, 23, np.zeros((1, 4, 23)), D, 1, 5)    # q^b above 2^22
    with pytest.raises(ValueError):
        JobSpec(4, 4, 2, M - 1, D, 1, 5)                    # negative digit
    with pytest.raises(ValueError):
        JobSpec(4, 4, 2, M, D, 1, 5, src="coded")           # coded source without its code


def test_request_spec_is_built_once_and_stays_equal():
    """spec() stacks and checks a request's arrays at the first call; later calls
    build a JobSpec from them with the current scalars, equal to a fresh one."""
    from qsft_gb300.engine import JobSpec
    from qsft_gb300.serve import random_request
    np.random.seed(2)
    r = random_request(4, 12, 5, 40, C=3, R=2, snr_db=10.0)
    first, again = r.spec(), r.spec()
    fresh = JobSpec(r.q, r.n, r.b, np.stack(r.Ms), np.stack([np.vstack(d) for d in r.Ds]), 2, r.n + 1,
                    chan="nso", cutoff=r.cutoff, K=r.locq.T, A=r.strengths,
                    noise_nu=r.noise_sd / np.sqrt(2 * r.q ** r.b), noise_seed=r.noise_seed)
    for sp in (first, again):
        for k in ("q", "n", "b", "C", "R", "P", "S", "B", "chan", "src", "cutoff", "max_iter", "noise_nu",
                  "noise_seed"):
            assert getattr(sp, k) == getattr(fresh, k), k
        for k in ("M", "D", "K", "A"):
            assert np.array_equal(getattr(sp, k), getattr(fresh, k)), k
    assert again.M is first.M          # the stacked arrays are shared, not rebuilt
    r.noise_seed = 12345               # scalars are read at every call
    assert r.spec().noise_seed == 12345
