"""Reed-Solomon source code for coded delays (host construction, GPU decoding).

Mirrors qsft/ReedSolomon.py (which subclasses ``galois.ReedSolomon``):

* ``ReedSolomon(n, t, q)`` -- s = ceil(log n / log q), bumped when
  n > q^s - 1 (qsft/ReedSolomon.py:18-24); a primitive narrow-sense (first root
  alpha^1) RS code of length q^s - 1 over GF(q^s).  GF(q^s) is built on the
  Conway polynomial with primitive element x (galois' defaults for a prime
  power field; smallest primitive root when s = 1).
* ``get_delay_matrix()`` -- (2ts+1) x n delays whose rows s*j+1..s*(j+1) are
  the GF(q) coefficient vectors (highest degree first) of the parity-check
  entries alpha^((1+j)(n-1-i)) (qsft/ReedSolomon.py:50-65).
* ``syndrome_decode(syndrome)`` -- decodes on the GPU (``qsft_rs_decode``:
  Berlekamp-Massey, Chien search, Forney) and returns (k as a 1 x n array,
  number of nonzero error values), like qsft/ReedSolomon.py:26-48.

``gf_tables()`` returns the exp | log | Zech-log tables the CUDA detector uses.
"""
import math

import numpy as np

# Conway polynomials a_0..a_m (monic), the field galois builds by default
CONWAY = {
    (2, 1): [1, 1], (2, 2): [1, 1, 1], (2, 3): [1, 1, 0, 1], (2, 4): [1, 1, 0, 0, 1],
    (2, 5): [1, 0, 1, 0, 0, 1], (2, 6): [1, 1, 0, 1, 1, 0, 1], (2, 7): [1, 1, 0, 0, 0, 0, 0, 1],
    (2, 8): [1, 0, 1, 1, 1, 0, 0, 0, 1],
    (3, 1): [1, 1], (3, 2): [2, 2, 1], (3, 3): [1, 2, 0, 1], (3, 4): [2, 0, 0, 2, 1],
    (3, 5): [1, 2, 0, 0, 0, 1],
    (5, 1): [3, 1], (5, 2): [2, 4, 1], (5, 3): [3, 3, 0, 1], (5, 4): [2, 4, 4, 0, 1],
    (7, 1): [4, 1], (7, 2): [3, 6, 1], (7, 3): [4, 0, 6, 1],
    (11, 1): [9, 1], (11, 2): [2, 7, 1], (11, 3): [9, 2, 0, 1],
    (13, 1): [11, 1], (13, 2): [2, 12, 1], (13, 3): [11, 2, 0, 1],
    (17, 1): [14, 1], (17, 2): [3, 16, 1], (19, 1): [17, 1], (19, 2): [2, 18, 1],
    (23, 1): [18, 1], (23, 2): [5, 21, 1], (29, 1): [27, 1], (29, 2): [2, 24, 1],
}


class GaloisField:
    """GF(p^m); element e = sum_i c_i p^i with c_i the coefficient of x^i."""

    def __init__(self, p, m):
        if p < 2 or any(p % d == 0 for d in range(2, int(p ** 0.5) + 1)):
            raise ValueError(f"GF({p}^{m}) is not a field: {p} is not prime")
        self.p, self.m, self.order = p, m, p ** m
        poly = CONWAY.get((p, m))
        if poly is None or not self._primitive(poly):
            poly = next(pl for pl in self._candidates() if self._primitive(pl))
        self.poly = poly
        n1 = self.order - 1
        exp = np.zeros(2 * n1, dtype=np.int32)
        log = np.full(self.order, -1, dtype=np.int32)
        e = 1
        for i in range(n1):
            exp[i] = e
            log[e] = i
            e = self._times_alpha(e)
        exp[n1:] = exp[:n1]
        self.exp, self.log = exp, log
        one_plus = np.array([self._add_digits(1, int(exp[k])) for k in range(n1)], dtype=np.int64)
        self.zech = np.where(one_plus == 0, -1, log[one_plus]).astype(np.int32)

    def _digits(self, e):
        return [(e // self.p ** i) % self.p for i in range(self.m)]

    def _value(self, d):
        return int(sum(int(c) * self.p ** i for i, c in enumerate(d)))

    def _add_digits(self, a, b):
        return self._value([(x + y) % self.p for x, y in zip(self._digits(a), self._digits(b))])

    def _times_alpha(self, e, poly=None):
        poly = poly or self.poly
        p, m = self.p, self.m
        if m == 1:
            return (e * ((p - poly[0]) % p)) % p
        d = [0] + self._digits(e)
        top = d[m]
        return self._value([(d[i] - top * poly[i]) % p for i in range(m)])

    def _candidates(self):
        p, m = self.p, self.m
        for v in range(p ** m):
            yield [(v // p ** i) % p for i in range(m)] + [1]

    def _primitive(self, poly):
        if len(poly) != self.m + 1 or poly[-1] != 1 or poly[0] % self.p == 0:
            return False
        e, k = 1, 0
        while True:
            e = self._times_alpha(e, poly)
            k += 1
            if e == 1:
                return k == self.order - 1
            if k > self.order:
                return False

    def vector(self, e):
        """Coefficients, highest degree first (galois ``FieldArray.vector``)."""
        return list(reversed(self._digits(e)))

    def tables(self):
        return np.concatenate([self.exp, self.log, self.zech]).astype(np.int32)


class ReedSolomon:
    """Host description of the coded-delay RS code; decoding runs on the GPU."""

    def __init__(self, n, t, q):
        s = math.ceil(math.log(n) / math.log(q))   # qsft/ReedSolomon.py:20
        if n > q ** s - 1:                          # qsft/ReedSolomon.py:21-22
            s += 1
        if t < 1 or t > 16:
            raise ValueError("t must be in 1..16")
        self.n, self.t, self.q, self.s, self.ns = q ** s - 1, t, q, s, n
        self.field = GaloisField(q, s)
        if self.field.order > 4096:
            raise ValueError("GF(q^s) larger than 4096 elements is not supported")

    def get_parity_length(self):  # qsft/ReedSolomon.py:67-74
        return 2 * self.t * self.s

    def get_delay_matrix(self):  # qsft/ReedSolomon.py:50-65
        s, ns, t, f = self.s, self.ns, self.t, self.field
        D = np.zeros((2 * t * s + 1, ns), dtype=np.int64)
        for i in range(ns):
            for j in range(2 * t):
                e = int(f.exp[((1 + j) * (ns - 1 - i)) % (f.order - 1)])
                D[s * j + 1:s * (j + 1) + 1, i] = f.vector(e)
        return D

    def gf_tables(self):
        return self.field.tables()

    def syndrome_decode(self, syndrome):
        """Decode one syndrome (2ts q-ary symbols) on the GPU."""
        from .engine import rs_decode_batch
        k = rs_decode_batch(self, np.asarray(syndrome, dtype=np.int64).reshape(1, -1))
        return k.astype(np.int64), int(np.count_nonzero(k))

    __call__ = syndrome_decode
