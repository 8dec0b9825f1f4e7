"""Utility functions of the reference's qsft/utils.py that the hot path uses.

Index codecs stay on the host (they are Python big-int conversions the GPU
path never needs: query points travel as q-ary digit rows).  ``gwht`` runs on
the GPU.
"""
import itertools
import pickle
import zlib

import numpy as np
import torch


def qary_ints(m, q, dtype=int):
    """All length-m q-ary vectors as columns, itertools.product order (qsft/utils.py:107-108)."""
    return np.array(list(itertools.product(np.arange(q), repeat=m)), dtype=dtype).reshape(-1, m).T


def qary_digits(idx, q, m):
    """MSB-first digits of integers idx < q^m as an (m, len) int array (vectorised dec_to_qary_vec)."""
    idx = np.asarray(idx, dtype=np.int64)
    out = np.empty((m, idx.size), dtype=np.int64)
    for i in range(m - 1, -1, -1):
        out[i] = idx % q
        idx = idx // q
    return out


def qary_vec_to_dec(x, q):
    """MSB-first q-ary -> decimal, Python big ints (qsft/utils.py:74-76)."""
    x = np.asarray(x)
    n = x.shape[0]
    return np.array([q ** (n - (i + 1)) for i in range(n)], dtype=object) @ np.array(x, dtype=object)


def dec_to_qary_vec(x, q, n):
    """Decimal (int or Python big int) -> MSB-first digits, n x len(x) (qsft/utils.py:79-84)."""
    x = np.asarray(x)
    if x.dtype != object and q ** n < 2 ** 63:
        return qary_digits(x.astype(np.int64), q, n)
    x = np.array(x, dtype=object)
    out = []
    for i in range(n):
        d = np.array([a // (q ** (n - (i + 1))) for a in x], dtype=object)
        out.append(d)
        x = x - (q ** (n - (i + 1))) * d
    return np.array(out, dtype=int)


def sort_qary_vecs(qary_vecs):  # qsft/utils.py:180-183
    qary_vecs = np.array(qary_vecs)
    return qary_vecs[np.lexsort(qary_vecs.T[::-1, :])]


def calc_hamming_weight(qary_vecs):  # qsft/utils.py:185-187
    return np.sum(np.array(qary_vecs) != 0, axis=1)


def random_signal_strength_model(sparsity, a, b):  # qsft/utils.py:161-164
    magnitude = np.random.uniform(a, b, sparsity)
    phase = np.random.uniform(0, 2 * np.pi, sparsity)
    return magnitude * np.exp(1j * phase)


def angle_q(x, q):  # qsft/utils.py:104-105
    return (((np.angle(x) % (2 * np.pi) // (np.pi / q)) + 1) // 2) % q


def gwht(x, q, n, precision="fp64"):
    """GWHT with forward scaling, fftn(reshape(x,[q]*n)) / q^n (qsft/utils.py:31-36), on the GPU.

    Accepts a numpy array (returned as numpy) or a CUDA tensor (transformed in place and returned)."""
    from .engine import gwht_device
    if isinstance(x, torch.Tensor):
        return gwht_device(x, q, n)
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    t = torch.as_tensor(np.ascontiguousarray(np.asarray(x, dtype=np.complex128).reshape(-1))).to(
        device=torch.device("cuda", torch.cuda.current_device()), dtype=cdt)
    gwht_device(t, q, n)
    return t.cpu().numpy().astype(np.complex128)


def save_data(data, filename):  # qsft/utils.py:189-192
    with open(filename, "wb") as f:
        f.write(zlib.compress(pickle.dumps(data, pickle.HIGHEST_PROTOCOL), 9))


def load_data(filename):  # qsft/utils.py:194-197
    with open(filename, "rb") as f:
        return pickle.loads(zlib.decompress(f.read()))
