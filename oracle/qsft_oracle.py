"""numpy restatement of the reference q-SFT hot path -- oracle (test infrastructure only).

Each function names the reference file:line it restates (paths within
basics-lab/qsft).  Host RNG draws use the legacy ``np.random`` stream in the
reference's order so that a seeded run reproduces the reference's signal,
query matrices, permutations and noise exactly.
"""
import itertools
from concurrent.futures import ThreadPoolExecutor

import numpy as np

try:  # the reference's GWHT is scipy.fft.fftn (qsft/utils.py:31-36)
    import scipy.fft as _fft
except Exception:  # pragma: no cover - numpy's pocketfft is the same algorithm
    import numpy.fft as _fft

__all__ = [
    "qary_ints", "qary_vec_to_dec", "dec_to_qary_vec", "sort_qary_vecs", "calc_hamming_weight",
    "random_signal_strength_model", "generate_signal_w", "get_Ms", "get_D", "get_Ms_and_Ds",
    "coset_points", "eval_points", "gwht", "subsample_qsft", "get_MDU_perm", "bin_noise",
    "singleton_detection", "peel", "OracleSignal", "OracleQSFT", "noise_sd_for_snr", "nmse", "closed_form_bins",
    "test_qary_nmse", "reproject",
]


# ---------------------------------------------------------------- codecs (qsft/utils.py)
def qary_ints(m, q):
    """All length-m q-ary vectors as columns, itertools.product order (qsft/utils.py:107-108)."""
    return np.array(list(itertools.product(np.arange(q), repeat=m)), dtype=np.int64).reshape(-1, m).T


def qary_vec_to_dec(x, q):
    """MSB-first q-ary -> decimal with Python big ints (qsft/utils.py:74-76)."""
    x = np.asarray(x)
    n = x.shape[0]
    return np.array([q ** (n - (i + 1)) for i in range(n)], dtype=object) @ np.array(x, dtype=object)


def dec_to_qary_vec(x, q, n):
    """Decimal -> MSB-first q-ary digits, n x len(x) (qsft/utils.py:79-84)."""
    x = np.array(x, dtype=object)
    out = []
    for i in range(n):
        d = np.array([a // (q ** (n - (i + 1))) for a in x], dtype=object)
        out.append(d)
        x = x - (q ** (n - (i + 1))) * d
    return np.array(out, dtype=np.int64)


def sort_qary_vecs(v):
    """Lexicographic sort of q-ary row vectors (qsft/utils.py:180-183)."""
    v = np.array(v)
    return v[np.lexsort(v.T[::-1, :])]


def calc_hamming_weight(v):  # qsft/utils.py:185-187
    return np.sum(np.array(v) != 0, axis=1)


# ---------------------------------------------------------------- synthetic signal
def random_signal_strength_model(S, a, b):  # qsft/utils.py:161-164
    mag = np.random.uniform(a, b, S)
    ph = np.random.uniform(0, 2 * np.pi, S)
    return mag * np.exp(1j * ph)


def generate_signal_w(n, q, S, a_min, a_max, max_weight=None):
    """Sparse support + coefficients (synt_exp/synt_src/synthetic_signal.py:10-38, full=False)."""
    max_weight = n if max_weight is None else max_weight
    if max_weight == n:
        locq = sort_qary_vecs(np.random.randint(q, size=(n, S)).T).T
    else:
        vals = np.random.randint(q - 1, size=(max_weight, S)) + 1
        pos = np.random.choice(a=n, size=(S, max_weight))
        locq = np.zeros((n, S), dtype=int)
        for i in range(S):
            locq[pos[i, :], i] = vals[:, i]
        locq = sort_qary_vecs(locq.T).T
    strengths = random_signal_strength_model(S, a_min, a_max)
    signal_w = dict(zip(list(map(tuple, locq.T)), strengths))
    return signal_w, locq, strengths


def noise_sd_for_snr(S, snr_db, a_min=1.0, a_max=10.0):
    """sigma for a per-sample SNR (synt_exp/run-tests-complexity-vs-size.py:72 convention,
    with E|a|^2 of |a|~U[a_min,a_max])."""
    if snr_db is None or not np.isfinite(snr_db):
        return 0.0
    ea2 = (a_max ** 3 - a_min ** 3) / (3.0 * (a_max - a_min)) if a_max > a_min else a_min ** 2
    return float(np.sqrt(S * ea2 / (10.0 ** (snr_db / 10.0))))


# ---------------------------------------------------------------- query design (qsft/query.py)
def get_Ms(n, b, q, num_to_get=None, method="simple"):
    """qsft/query.py:13-70."""
    if num_to_get is None:
        num_to_get = max(n // b, 3)
    if method == "simple":
        if num_to_get > n // b:
            raise ValueError("When query_method is 'simple', the number of M matrices to return cannot be larger than n // b")
        Ms = []
        for i in range(num_to_get - 1, -1, -1):
            M = np.zeros((n, b), dtype=np.int32)
            M[(b * i):(b * (i + 1)), :] = np.eye(b)
            Ms.append(M)
        return Ms
    return [np.random.randint(q, size=(n, b)) for _ in range(num_to_get)]


def get_D(n, q, **kw):
    """Source layer then channel layer (qsft/query.py:73-143)."""
    src = kw.get("delays_method_source", "random")
    if src == "identity":
        D = np.vstack((np.zeros(n), np.eye(n))).astype(int)            # :73-76
    elif src == "random":
        D = np.random.choice(q, (kw.get("num_delays"), n))               # :79-85
    elif src == "coded":
        from .rs import ReedSolomonOracle                                 # :88-92
        D = np.array(ReedSolomonOracle(n, kw.get("t"), q).get_delay_matrix(), dtype=int)
    else:
        raise ValueError(src)
    ch = kw.get("delays_method_channel", "identity")
    if ch == "nso":                                                       # :95-106
        offs = np.random.choice(q, (kw.get("num_repeat"), n))
        return [(row - D) % q for row in offs]
    if ch == "identity":                                                  # :112-114
        return [D % q]
    raise NotImplementedError(ch)


def get_Ms_and_Ds(n, q, **kw):
    """qsft/query.py:182-203: C matrices M, one delay list shared by all groups."""
    Ms = get_Ms(n, kw.get("b"), q, method=kw.get("query_method"), num_to_get=kw.get("num_subsample"))
    D = get_D(n, q=q, **kw)
    return Ms, [D for _ in Ms]


# ---------------------------------------------------------------- sampling + GWHT
def coset_points(M, d, q):
    """Coset {M l + d : l in Z_q^b} as an n x q^b digit matrix
    (qsft/input_signal_subsampled.py:198-201, before the decimal conversion)."""
    L = qary_ints(M.shape[1], q)
    return ((M @ L) % q + np.asarray(d).reshape(-1, 1)) % q


def eval_points(X, locq, strengths, q, threads=1, batch=10000):
    """f(x) = sum_s a_s exp(2 pi i <x,k_s>/q) for the rows of X (N x n)
    (synt_exp/synt_src/synthetic_signal.py:100-102, batched like :108-118)."""
    X = np.asarray(X)
    freq = 2j * np.pi * np.asarray(locq) / q
    a = np.asarray(strengths)

    def one(lo):
        return np.exp(X[lo:lo + batch] @ freq) @ a

    starts = list(range(0, X.shape[0], batch))
    if threads <= 1 or len(starts) == 1:
        parts = [one(s) for s in starts]
    else:
        with ThreadPoolExecutor(threads) as ex:
            parts = list(ex.map(one, starts))
    return np.concatenate(parts) if parts else np.zeros(0, np.complex128)


def gwht(x, q, b):
    """fftn over the [q]*b tensor / q^b (qsft/utils.py:31-36)."""
    return np.reshape(_fft.fftn(np.reshape(x, [q] * b)) / (q ** b), [q ** b])


def subsample_qsft(Ms, Ds, q, eval_fn, all_bs=None):
    """Us[c][r] = P x B bins for every (group, repeat) (qsft/input_signal_subsampled.py:107-155).
    With all_bs, returns {b: Us} where the sub-transform for b takes every
    q^(b_max-b)-th sample (_compute_subtransform, :264-266)."""
    per_b = {}
    for M, Dlist in zip(Ms, Ds):
        bmax = M.shape[1]
        bs = all_bs or [bmax]
        rows = {bb: [] for bb in bs}
        for D in Dlist:
            pts = [coset_points(M, d, q) for d in D]
            samples = eval_fn(np.concatenate([p.T for p in pts], axis=0)).reshape(len(D), q ** bmax)
            for bb in bs:
                rows[bb].append(np.array([gwht(s[::q ** (bmax - bb)], q, bb) for s in samples]))
        for bb in bs:
            per_b.setdefault(bb, []).append(rows[bb])
    return per_b if all_bs else per_b[Ms[0].shape[1]]


def get_MDU_perm(C_have, R_have, C, R):
    """The two permutation draws of qsft/input_signal_subsampled.py:246-247."""
    return (np.random.choice(C_have, C, replace=False), np.random.choice(R_have, R, replace=False))


def bin_noise(noise_sd, q, b, shape):
    """Complex AWGN added to the bins (synt_exp/synt_src/synthetic_signal.py:126-129)."""
    nu = noise_sd / np.sqrt(2 * q ** b)
    return np.random.normal(0, nu, size=tuple(shape) + (2,)).view(np.complex128).reshape(shape)


# ---------------------------------------------------------------- detection (qsft/reconstruct.py)
def _detect_noiseless(U, q):  # :12-31, vectorised over columns
    ang = np.angle(U)
    a = q * (ang[1:] - ang[0]) / (2 * np.pi)
    return a.round().astype(int) % q


def _detect_nso1(U, q, p1):  # :100-113, vectorised over columns
    q_roots = 2 * np.pi / q * np.arange(q + 1)
    U0 = U[0::p1]
    out = np.zeros((p1 - 1, U.shape[1]), dtype=int)
    for i in range(1, p1):
        ang = np.angle(np.mean(U0 * np.conjugate(U[i::p1]), axis=0)) % (2 * np.pi)
        out[i - 1] = np.abs(q_roots[:, None] - ang[None, :]).argmin(axis=0) % q
    return out


def singleton_detection(U, q, chan, src, p1, decoder=None):
    """Column-wise k for the columns of U (qsft/reconstruct.py:132-168, nso_subtype 'nso1')."""
    if chan == "identity":
        K = _detect_noiseless(U, q)
    elif chan == "nso":
        K = _detect_nso1(U, q, p1)
    else:
        raise NotImplementedError(chan)
    if src == "coded":  # :34-51
        K = np.stack([np.array(decoder(list(K[:, c]))[0][0, :], dtype=np.int64) for c in range(K.shape[1])], axis=1) \
            if K.shape[1] else np.zeros((0, 0), dtype=np.int64)
    return K


def _col_sqnorm(V):
    """||col||^2 as np.linalg.norm(col)**2 computes it, per column."""
    return np.sqrt(np.sum(V.real * V.real, axis=0) + np.sum(V.imag * V.imag, axis=0)) ** 2


def peel(Us, Ms, Ds, q, n, b, cutoff, chan, src, p1, decoder=None, max_iter=15, trace=None):
    """The peeling decoder of QSFT.transform (qsft/qsft.py:98-255).

    Us: list of C arrays (R*P) x B (modified in place).  Returns (gwht dict, result list, iterations)."""
    omega = np.exp(2j * np.pi / q)
    peeling_max = q ** n
    result = []
    num_peeling = 0
    iter_step = 0
    cont = True
    digits = qary_ints(b, q)  # column j = MSB-first digits of j (dec_to_qary_vec, qsft/qsft.py:178)
    while cont and num_peeling < peeling_max and iter_step < max_iter:      # :151
        iter_step += 1
        singletons = {}
        multitons = []
        for i, (U, M, D) in enumerate(zip(Us, Ms, Ds)):                     # :162-193
            RP = U.shape[0]
            energy = _col_sqnorm(U)
            cand = np.nonzero(energy > cutoff * RP)[0]
            if len(cand) == 0:
                continue
            cols = U[:, cand]
            K = singleton_detection(cols, q, chan, src, p1, decoder)
            if trace is not None:
                for c in range(len(cand)):
                    trace.append(K[:, c].copy())
            sig = omega ** (D @ K)                                          # :174
            rho = np.sum(np.conjugate(sig) * cols, axis=0) / D.shape[0]     # :175
            res = _col_sqnorm(cols - rho[None, :] * sig)                    # :176,183
            match = np.all((M.T @ K) % q == digits[:, cand], axis=0)        # :178-179
            for c, j in enumerate(cand):
                if (not match[c]) or res[c] > cutoff * RP:
                    multitons.append((i, int(j)))
                else:
                    singletons[(i, int(j))] = (K[:, c], rho[c])
        if len(multitons) == 0 or len(singletons) == 0:                     # :204-205
            cont = False
        balls = set()
        ball_values = {}
        for (i, j) in singletons:                                           # :209-217
            k, rho = singletons[(i, j)]
            ball = tuple(k)
            balls.add(ball)
            ball_values[ball] = rho
            result.append((k, ball_values[ball]))
        for ball in balls:                                                  # :223-241
            num_peeling += 1
            k = np.array(ball)[..., np.newaxis]
            for l, M in enumerate(Ms):
                jl = int(qary_vec_to_dec(M.T.dot(k) % q, q)[0])
                sig = omega ** (Ds[l] @ k)
                Us[l][:, jl] -= (ball_values[ball] * sig.reshape(-1, 1))[:, 0]
    gw, cnt = {}, {}
    for k, v in result:                                                     # :247-255
        key = tuple(k)
        if key in cnt:
            gw[key] = (gw[key] * cnt[key] + v) / (cnt[key] + 1)
            cnt[key] += 1
        else:
            gw[key] = v
            cnt[key] = 1
    return gw, result, iter_step


# ---------------------------------------------------------------- API mirrors
class OracleSignal:
    """A seeded synthetic subsampled signal: get_random_subsampled_signal + SyntheticSubsampledSignal
    (synt_exp/synt_src/synthetic_signal.py:70-130) without the decimal round trip."""

    def __init__(self, n, q, S, a_min, a_max, noise_sd, query_args, max_weight=None, eval_threads=1,
                 skip_sampling=False):
        self.n, self.q, self.noise_sd = n, q, noise_sd
        self.signal_w, self.locq, self.strengths = generate_signal_w(n, q, S, a_min, a_max, max_weight)
        qa = dict(query_args)
        qa.setdefault("num_repeat", 1)
        self.query_args = qa
        self.b = qa["b"]
        self.num_subsample = qa["num_subsample"]
        self.num_repeat = qa["num_repeat"]
        self.Ms, self.Ds = get_Ms_and_Ds(n, q, **qa)
        self.all_bs = qa.get("all_bs", [self.b])
        if not skip_sampling:
            self.Us_b = subsample_qsft(self.Ms, self.Ds, q,
                                       lambda X: eval_points(X, self.locq, self.strengths, q, threads=eval_threads),
                                       all_bs=self.all_bs)
            self.Us = self.Us_b[self.b]

    def get_source_parity(self):  # qsft/input_signal_subsampled.py:268-269
        return self.Ds[0][0].shape[0]

    def get_MDU(self, C, R, b):
        """qsft/input_signal_subsampled.py:225-262 + synthetic noise (synthetic_signal.py:120-130)."""
        if not (C <= self.num_subsample and R <= self.num_repeat and b <= self.b):
            raise ValueError("There are not enough Ms or Ds.")
        ci, ri = get_MDU_perm(self.num_subsample, self.num_repeat, C, R)
        Ms = [self.Ms[i][:, :b] for i in ci]
        Ds = [[self.Ds[i][j] for j in ri] for i in ci]
        src = self.Us if b == self.b else self.Us_b[b]
        Us = [[src[i][j] for j in ri] for i in ci]
        out = []
        for row in Us:
            out.append([u + bin_noise(self.noise_sd, self.q, b, u.shape) for u in row])
        return Ms, Ds, out


class OracleQSFT:
    """QSFT(**kw).transform(signal) (qsft/qsft.py:47-281) over OracleSignal."""

    def __init__(self, **kw):
        self.src = kw.get("reconstruct_method_source")
        self.chan = kw.get("reconstruct_method_channel")
        self.C = kw.get("num_subsample")
        self.R = kw.get("num_repeat")
        self.b = kw.get("b")
        self.decoder = kw.get("source_decoder")

    def transform(self, signal, report=False, trace=None, **kw):
        q, n, b = signal.q, signal.n, self.b
        Ms, Ds, Us = signal.get_MDU(self.C, self.R, b)
        Us = [np.vstack(u) for u in Us]
        Ds = [np.vstack(d) for d in Ds]
        cutoff = kw.get("cutoff", 1e-9 + 1.5 * signal.noise_sd ** 2 / q ** b)   # qsft/qsft.py:124-126
        gw, result, iters = peel(Us, Ms, Ds, q, n, b, cutoff, self.chan, self.src,
                                 signal.get_source_parity(), self.decoder, trace=trace)
        if not report:
            return gw
        loc = list({tuple(k) for k, _ in result})
        if loc and kw.get("sort", False):
            loc = sort_qary_vecs(loc)
        hw = calc_hamming_weight(loc) if len(loc) else np.zeros(1)
        return {"gwht": gw, "n_samples": int(np.prod(np.shape(np.array(Us)))), "locations": loc,
                "avg_hamming_weight": float(np.mean(hw)) if len(loc) else 0,
                "max_hamming_weight": int(np.max(hw)) if len(loc) else 0, "iterations": iters}


def nmse(true_w, est_w):
    """Coefficient-domain NMSE over the union of keys (synt_exp/quick_example.py:71-80)."""
    keys = set(true_w) | set(est_w)
    num = sum(abs(true_w.get(k, 0) - est_w.get(k, 0)) ** 2 for k in keys)
    return float(num / sum(abs(v) ** 2 for v in true_w.values()))


def closed_form_bins(Ms, Ds, locq, strengths, q):
    """Exact noiseless bins of a synthetic signal: U_c[r*P+p][j] = sum over s with
    M_c^T k_s = j (mod q) of a_s omega^<d_{r,p}, k_s> -- the identity that eval +
    GWHT must reproduce (f's spectrum aliased by M_c, phased by the delays).
    Ms: C of (n x b); Ds: C of (R*P x n) stacked delays; returns C x (R*P) x q^b."""
    locq = np.asarray(locq)
    a = np.asarray(strengths)
    out = []
    for M, D in zip(Ms, Ds):
        b = M.shape[1]
        j = (np.asarray(M).T @ locq) % q                       # b x S digits, MSB first
        jdec = np.zeros(locq.shape[1], dtype=np.int64)
        for t in range(b):
            jdec = jdec * q + j[t]
        ph = (np.asarray(D) @ locq) % q                        # (R*P) x S
        vals = a[None, :] * np.exp(2j * np.pi * ph / q)
        U = np.zeros((np.asarray(D).shape[0], q ** b), dtype=np.complex128)
        for r in range(U.shape[0]):
            np.add.at(U[r], jdec, vals[r])
        out.append(U)
    return np.array(out)


def test_qary_nmse(beta, query_indices, samples, q, n):
    """TestHelper._test_qary (qsft/test_helper.py:235-260): NMSE of the sparse
    transform `beta` against `samples` at decimal `query_indices`; 1 when beta
    is empty."""
    if len(beta) == 0:
        return 1
    keys = np.array([list(k) for k in beta.keys()], dtype=np.int64).reshape(-1, n)
    vals = np.array(list(beta.values()), dtype=np.complex128)
    X = np.array([[(int(x) // q ** (n - 1 - i)) % q for i in range(n)] for x in query_indices], dtype=np.int64)
    y_hat = np.exp(2j * np.pi * ((X @ keys.T) % q) / q) @ vals
    samples = np.asarray(samples, dtype=np.complex128)
    return float(np.linalg.norm(y_hat - samples) ** 2 / np.linalg.norm(samples) ** 2)


def reproject(Us_raw, Ms, Ds, q, gw):
    """Checker of the optional FP64 re-projection (no counterpart in the
    reference, which keeps the running mean of qsft/qsft.py:247-255): subtract
    every (k, a) of `gw` from the raw bins of every group, then re-estimate each
    a as the mean over the groups of a + <omega^(D_l k), residual column>/len.
    Us_raw: C arrays (R*P) x B (copied); Ds: C arrays (R*P) x n."""
    omega = np.exp(2j * np.pi / q)
    R = [np.array(U, dtype=np.complex128, copy=True) for U in Us_raw]
    keys = list(gw)
    K = np.array(keys, dtype=np.int64).reshape(len(keys), -1)
    a = np.array([gw[k] for k in keys], dtype=np.complex128)
    bins = []
    for M, D, U in zip(Ms, Ds, R):
        b = M.shape[1]
        j = np.zeros(len(keys), dtype=np.int64)
        for t in range(b):
            j = j * q + (K @ M[:, t]) % q
        sig = omega ** ((np.asarray(D) @ K.T) % q)          # (R*P) x keys
        np.add.at(U.T, j, -(sig * a).T)
        bins.append((j, sig))
    new = np.zeros_like(a)
    for (j, sig), U in zip(bins, R):
        new += a + np.sum(np.conjugate(sig) * U[:, j], axis=0) / U.shape[0]
    new /= len(R)
    return dict(zip(keys, new))
