"""Generate the golden fixtures in this folder by running the reference q-SFT.

This script is the only committed code that executes the reference
(basics-lab/qsft).  It is run once, by hand, on a machine that has a checkout
of the reference, given by ``--ref PATH`` or the ``QSFT_REFERENCE`` environment
variable; the fixtures it writes (``*.npz``) are committed and travel with the
repository, the reference itself does not.

The reference needs packages this image lacks.  The shims below replace them
with stand-ins that are never reached on the q-SFT path:

* numpy 2 removed ``np.complex`` / ``np.int`` (used at
  qsft/input_signal_subsampled.py:136, synt_exp/synt_src/synthetic_signal.py:34,129);
* ``group_lasso``, ``matplotlib`` are import-time only (qsft/utils.py:6,16);
* ``galois`` is imported by qsft/ReedSolomon.py:1-2 but only used by the
  RS-coded source path, which therefore cannot be pinned here;
* ``multiprocess.Pool`` (synthetic_signal.py:6) becomes a thread pool with
  ``imap`` -- evaluation order and results are unchanged.

Usage:  python tests/golden/make_golden.py --ref PATH [case ...]
"""
import copy
import os
import sys
import time
import types
from multiprocessing.pool import ThreadPool

import numpy as np

REF = os.environ.get("QSFT_REFERENCE")   # the reference checkout (or --ref PATH)
HERE = os.path.dirname(os.path.abspath(__file__))


def _install_shims():
    np.complex = complex
    np.int = int
    gl = types.ModuleType("group_lasso")
    gl.GroupLasso = None
    sys.modules["group_lasso"] = gl
    glf = types.ModuleType("group_lasso._fista")
    glf.ConvergenceWarning = Warning
    sys.modules["group_lasso._fista"] = glf
    mpl = types.ModuleType("matplotlib")
    mpl.pyplot = types.ModuleType("matplotlib.pyplot")
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = mpl.pyplot

    class _Pool:
        def __init__(self, *a, **k):
            self._p = ThreadPool(os.cpu_count())

        def __enter__(self):
            return self

        def __exit__(self, *a):
            self._p.close()
            self._p.join()

        def imap(self, f, it):
            return self._p.imap(f, it)

    mp = types.ModuleType("multiprocess")
    mp.Pool = _Pool
    sys.modules["multiprocess"] = mp
    gal = types.ModuleType("galois")
    gal.ReedSolomon = object
    sys.modules["galois"] = gal
    for m in ["galois._codes", "galois._codes._reed_solomon"]:
        sys.modules[m] = types.ModuleType(m)
    sys.modules["galois._codes._reed_solomon"].decode_jit = None
    if not REF or not os.path.isdir(os.path.join(REF, "qsft")):
        raise SystemExit("give the reference checkout with --ref PATH or QSFT_REFERENCE=PATH")
    sys.path.insert(0, REF)


def noise_sd_for(S, snr_db, a_min=1.0, a_max=10.0):
    """Per-sample time-domain SNR: sigma^2 = S * E|a|^2 / 10^(SNR/10), |a|~U[a_min,a_max]
    (the convention of synt_exp/run-tests-complexity-vs-size.py:72)."""
    if snr_db is None:
        return 0.0
    ea2 = (a_max ** 3 - a_min ** 3) / (3.0 * (a_max - a_min))
    return float(np.sqrt(S * ea2 / (10.0 ** (snr_db / 10.0))))


# name -> parameters.  full=True stores every intermediate (small cases only).
CASES = {
    "cfg1_q4n10b4_identity": dict(q=4, n=10, b=4, S=50, C=3, R=1, src="identity", ch="identity", snr=None, seed=0, full=True),
    "q4n12b5_nso_10db": dict(q=4, n=12, b=5, S=100, C=3, R=2, src="identity", ch="nso", snr=10, seed=1, full=True),
    "q20n6b2_nso_20db": dict(q=20, n=6, b=2, S=40, C=3, R=3, src="identity", ch="nso", snr=20, seed=2, full=True),
    "q3n8b4_identity": dict(q=3, n=8, b=4, S=10, C=3, R=1, src="identity", ch="identity", snr=None, seed=3, full=True),
    "q2n16b8_nso_20db": dict(q=2, n=16, b=8, S=50, C=3, R=2, src="identity", ch="nso", snr=20, seed=4, full=True),
    "q5n10b3_nso_clean": dict(q=5, n=10, b=3, S=30, C=3, R=1, src="identity", ch="nso", snr=None, seed=5, full=True),
    "q4n10b4_simple_nso": dict(q=4, n=10, b=4, S=40, C=2, R=2, src="identity", ch="nso", snr=20, seed=6, full=True,
                               query_method="simple"),
    "q4n10b5_allbs_b4_nso": dict(q=4, n=10, b=5, S=30, C=3, R=2, src="identity", ch="nso", snr=20, seed=8, full=False,
                                 all_bs=[4, 5], transform_b=4),
    "cfg2_q4n20b7_nso_10db": dict(q=4, n=20, b=7, S=1000, C=3, R=2, src="identity", ch="nso", snr=10, seed=0, full=False),
    "cfg3_q20n10b3_nso_20db": dict(q=20, n=10, b=3, S=500, C=3, R=3, src="identity", ch="nso", snr=20, seed=0, full=False),
}


def run_case(name, p):
    import qsft.qsft as qmod
    from qsft.qsft import QSFT
    from synt_exp.synt_src.synthetic_signal import get_random_subsampled_signal

    q, n, b, S, C, R = p["q"], p["n"], p["b"], p["S"], p["C"], p["R"]
    nsd = noise_sd_for(S, p["snr"])
    qa = dict(query_method=p.get("query_method", "complex"), num_subsample=C,
              delays_method_source=p["src"], subsampling_method="qsft",
              delays_method_channel=p["ch"], num_repeat=R, b=b)
    if "all_bs" in p:
        qa["all_bs"] = list(p["all_bs"])
    tb = p.get("transform_b", b)
    np.random.seed(p["seed"])
    t0 = time.time()
    sig = get_random_subsampled_signal(n=n, q=q, sparsity=S, a_min=1, a_max=10, noise_sd=nsd, query_args=qa)
    t1 = time.time()

    # record what transform() sees: the permutation draws and the noisy bins
    rng_state = np.random.get_state()
    np.random.set_state(rng_state)
    perm_c = np.random.choice(C, C, replace=False)
    perm_r = np.random.choice(R, R, replace=False)
    np.random.set_state(rng_state)

    captured = {}
    orig_get_mdu = sig.get_MDU

    def rec_get_mdu(*a, **k):
        out = orig_get_mdu(*a, **k)
        captured["Us_noisy"] = np.array([[np.asarray(u) for u in row] for row in out[2]])
        return out

    sig.get_MDU = rec_get_mdu

    calls = []
    orig_sd = qmod.singleton_detection

    def rec_sd(col, **kw):
        k = orig_sd(col, **kw)
        calls.append(np.asarray(k, dtype=np.int64).copy())
        return k

    qmod.singleton_detection = rec_sd
    try:
        res = QSFT(num_subsample=C, num_repeat=R, reconstruct_method_source=p["src"],
                   reconstruct_method_channel=p["ch"], b=tb).transform(sig, report=True, sort=True)
    finally:
        qmod.singleton_detection = orig_sd
    t2 = time.time()

    g = res["gwht"]
    keys = np.array([list(map(int, k)) for k in g.keys()], dtype=np.int64).reshape(-1, n)
    vals = np.array(list(g.values()), dtype=np.complex128)
    tw = sig.signal_w
    nmse = sum(abs(tw.get(k, 0) - g.get(k, 0)) ** 2 for k in set(tw) | set(g)) / sum(abs(v) ** 2 for v in tw.values())

    out = dict(
        q=q, n=n, b=b, S=S, C=C, R=R, seed=p["seed"], noise_sd=nsd, transform_b=tb,
        all_bs=np.array(qa.get("all_bs", [b]), dtype=np.int64),
        src=p["src"], ch=p["ch"], query_method=qa["query_method"],
        locq=np.asarray(sig.locq, dtype=np.int64),
        strengths=np.asarray(list(tw.values()), dtype=np.complex128),
        Ms=np.array(sig.Ms, dtype=np.int64),
        Ds=np.array(sig.Ds[0], dtype=np.int64),
        perm_c=perm_c, perm_r=perm_r,
        gwht_keys=keys, gwht_vals=vals,
        n_samples=int(res["n_samples"]),
        locations=np.asarray(res["locations"], dtype=np.int64).reshape(-1, n),
        avg_hamming_weight=float(res["avg_hamming_weight"]),
        max_hamming_weight=int(res["max_hamming_weight"]),
        nmse=float(nmse),
        ref_seconds_signal=t1 - t0, ref_seconds_transform=t2 - t1,
    )
    if p["full"]:
        Us_clean = np.array([[np.asarray(sig.Us[i][j][b]) for j in range(R)] for i in range(C)])
        out["Us_clean"] = Us_clean
        out["Us_noisy"] = captured["Us_noisy"]
        lens = np.array([len(c) for c in calls], dtype=np.int64)
        out["detect_k"] = np.concatenate(calls) if calls else np.zeros(0, np.int64)
        out["detect_len"] = lens
        # query generation pin: decimals of group 0, repeat 0
        qi = sig._get_qsft_query_indices(sig.Ms[0], sig.Ds[0][0])
        out["query_dec_g0r0"] = np.array([[int(v) for v in row] for row in qi], dtype=np.int64) if q ** n < 2 ** 62 else np.zeros(0)
        # evaluation pin: samples at the first 97 indices of that coset
        if q ** n < 2 ** 62:
            idx = np.array(qi[0][:97], dtype=object)
            out["eval_idx"] = np.array([int(v) for v in idx], dtype=np.int64)
            out["eval_vals"] = np.asarray(sig.subsample(idx), dtype=np.complex128)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: signal {t1 - t0:.2f}s transform {t2 - t1:.2f}s found {len(g)} nmse {nmse:.3e}", flush=True)


def gwht_pins():
    from qsft.utils import gwht
    rs = np.random.RandomState(123)
    out = {}
    for (q, b) in [(2, 5), (3, 4), (4, 3), (5, 3), (20, 2), (4, 7)]:
        x = rs.randn(q ** b) + 1j * rs.randn(q ** b)
        out[f"x_q{q}_b{b}"] = x
        out[f"y_q{q}_b{b}"] = gwht(x, q, b)
    np.savez_compressed(os.path.join(HERE, "gwht_pins.npz"), **out)
    print("gwht_pins written")


def test_qary_pins():
    """TestHelper._test_qary (qsft/test_helper.py:235-260) on a recovered
    transform with a few wrong and missing coefficients, at uniform test points
    of the true signal: the reference method is called on a stand-in `self`
    that carries only the attributes it reads (q, n, test_signal.signal_t)."""
    from qsft.test_helper import TestHelper
    rs = np.random.RandomState(321)
    out = {}
    for (q, n, S, N) in [(4, 10, 30, 2000), (3, 12, 20, 1500), (2, 20, 25, 3000)]:
        locq = rs.randint(q, size=(S, n))
        a = rs.uniform(1, 10, S) * np.exp(2j * np.pi * rs.uniform(size=S))
        idx = rs.randint(0, q ** n, size=N)
        X = np.array([[(int(x) // q ** (n - 1 - i)) % q for i in range(n)] for x in idx])
        samples = np.exp(2j * np.pi * ((X @ locq.T) % q) / q) @ a
        beta = {tuple(k): v * (1 + 0.01 * rs.randn()) for k, v in zip(map(tuple, locq[:-3]), a[:-3])}
        stand_in = types.SimpleNamespace(q=q, n=n, test_signal=types.SimpleNamespace(
            signal_t=dict(zip([int(x) for x in idx], samples))))
        nmse = TestHelper._test_qary(stand_in, beta)
        tag = f"q{q}_n{n}"
        out[f"{tag}_keys"] = np.array(list(beta.keys()), dtype=np.int64)
        out[f"{tag}_vals"] = np.array(list(beta.values()), dtype=np.complex128)
        # the test points as the reference holds them: a dict, so repeated indices collapse
        st = stand_in.test_signal.signal_t
        out[f"{tag}_idx"] = np.array(list(st.keys()), dtype=np.int64)
        out[f"{tag}_samples"] = np.array(list(st.values()), dtype=np.complex128)
        out[f"{tag}_nmse"] = np.float64(nmse)
    np.savez_compressed(os.path.join(HERE, "test_qary_pins.npz"), **out)
    print("test_qary_pins written", {k: float(v) for k, v in out.items() if k.endswith("_nmse")})


if __name__ == "__main__":
    args = sys.argv[1:]
    if "--ref" in args:
        i = args.index("--ref")
        REF = args[i + 1]
        del args[i:i + 2]
    _install_shims()
    names = args or list(CASES) + ["gwht", "test_qary"]
    for nm in names:
        if nm == "gwht":
            gwht_pins()
        elif nm == "test_qary":
            test_qary_pins()
        else:
            run_case(nm, CASES[nm])
