"""Query design: subsampling matrices M and delay matrices D (qsft/query.py).

Host code with the reference's legacy ``np.random`` draws in the reference's
order, so a seeded run builds the same M and D as the reference.
"""
import time

import numpy as np

from .reed_solomon import ReedSolomon


def get_Ms_simple(n, b, q, num_to_get=None):  # qsft/query.py:13-23
    Ms = []
    for i in range(num_to_get - 1, -1, -1):
        M = np.zeros((n, b), dtype=np.int32)
        M[(b * i):(b * (i + 1)), :] = np.eye(b)
        Ms.append(M)
    return Ms


def get_Ms_complex(n, b, q, num_to_get=None):  # qsft/query.py:26-35
    return [np.random.randint(q, size=(n, b)) for _ in range(num_to_get)]


def get_Ms(n, b, q, num_to_get=None, method="simple"):  # qsft/query.py:38-70
    if num_to_get is None:
        num_to_get = max(n // b, 3)
    if method == "simple" and num_to_get > n // b:
        raise ValueError("When query_method is 'simple', the number of M matrices to return cannot be larger than n // b")
    return {"simple": get_Ms_simple, "complex": get_Ms_complex}.get(method)(n, b, q, num_to_get)


def get_D_identity(n, **kwargs):  # qsft/query.py:73-76
    return np.vstack((np.zeros(n), np.eye(n))).astype(int)


def get_D_random(n, **kwargs):  # qsft/query.py:79-85
    return np.random.choice(kwargs.get("q"), (kwargs.get("num_delays"), n))


def get_D_source_coded(n, **kwargs):  # qsft/query.py:88-92
    return np.array(ReedSolomon(n, kwargs.get("t"), kwargs.get("q")).get_delay_matrix(), dtype=int)


def get_D_nso(n, D_source, **kwargs):  # qsft/query.py:95-106
    q = kwargs.get("q")
    offsets = get_D_random(n, q=q, num_delays=kwargs.get("num_repeat"))
    return [(row - D_source) % q for row in offsets]


def get_D_channel_coded(n, D, **kwargs):  # qsft/query.py:109-110
    raise NotImplementedError("One day this might be implemented")


def get_D_channel_identity(n, D, **kwargs):  # qsft/query.py:112-114
    return [D % kwargs.get("q")]


def get_D(n, **kwargs):  # qsft/query.py:116-143
    D = {"random": get_D_random, "identity": get_D_identity, "coded": get_D_source_coded}.get(
        kwargs.get("delays_method_source", "random"))(n, **kwargs)
    return {"nso": get_D_nso, "coded": get_D_channel_coded, "identity": get_D_channel_identity}.get(
        kwargs.get("delays_method_channel", "identity"))(n, D, **kwargs)


def get_Ms_and_Ds(n, q, **kwargs):  # qsft/query.py:182-203
    timing_verbose = kwargs.get("timing_verbose", False)
    t0 = time.time()
    Ms = get_Ms(n, kwargs.get("b"), q, method=kwargs.get("query_method"), num_to_get=kwargs.get("num_subsample"))
    if timing_verbose:
        print(f"M Generation:{time.time() - t0}")
    t0 = time.time()
    D = get_D(n, q=q, **kwargs)
    if timing_verbose:
        print(f"D Generation:{time.time() - t0}")
    return Ms, [D for _ in Ms]


def get_reed_solomon_dec(n, t_max, q):  # qsft/query.py:231-243
    """A Reed-Solomon syndrome decoder for a t_max-error-correcting code (decodes on the GPU)."""
    primeset = [2, 3, 5, 7, 11, 13, 15, 17, 19, 23, 29]
    if q in primeset:
        return ReedSolomon(n, t_max, q)
    raise NotImplementedError("q is not a prime number under 30!")
