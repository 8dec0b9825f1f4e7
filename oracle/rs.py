"""Reed-Solomon source code over GF(q^s) -- oracle (test infrastructure only).

Restates what qsft/ReedSolomon.py builds on top of ``galois==0.1.1``:

* ``ReedSolomon.__init__`` (qsft/ReedSolomon.py:18-24): s = ceil(log n / log q),
  bumped by one when n > q^s - 1; a primitive narrow-sense (c = 1) RS code of
  length nt = q^s - 1 and dimension nt - 2t over GF(q^s).
* ``get_delay_matrix`` (qsft/ReedSolomon.py:50-65): the (2ts+1) x n source delay
  matrix; row 0 is zero and rows s*j+1 .. s*(j+1) hold the GF(q)-coefficient
  vectors (highest degree first) of H[j, nt-n+i] = alpha^((c+j)(n-1-i)).
* ``syndrome_decode`` (qsft/ReedSolomon.py:26-48): group the 2ts received
  q-ary symbols into 2t GF(q^s) syndromes, decode the all-zero received word
  against them and return -codeword[-n:], i.e. the error values on the last
  n positions (= k for a weight <= t index).

galois itself is absent, so its field choices are restated: the field is
GF(p^m) built on the Conway polynomial and its primitive element is x (the
root of a Conway polynomial is primitive); for m = 1 it is the smallest
primitive root mod p.  Decoding uses Berlekamp-Massey, Chien search and Forney's
formula (published algorithms); a decoder failure (deg Lambda > t or fewer
roots than its degree) returns the received word unchanged, i.e. k = 0.
"""
import math

# Conway polynomials, coefficients a_0 .. a_m (monic).  Checked for
# primitivity at field construction.
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


class GF:
    """GF(p^m) with elements as integers sum_i c_i p^i (c_i = coefficient of x^i)."""

    def __init__(self, p, m):
        self.p, self.m = p, m
        self.order = p ** m
        poly = CONWAY.get((p, m))
        if poly is None or not self._is_primitive(poly):
            poly = self._first_primitive()
        self.poly = poly
        alpha = (p - poly[0]) % p if m == 1 else p  # root of x + a0, or x
        self.alpha = alpha
        n1 = self.order - 1
        self.exp = [0] * (2 * n1)
        self.log = [0] * self.order
        e = 1
        for i in range(n1):
            self.exp[i] = e
            self.log[e] = i
            e = self._mul_alpha(e, poly)
        for i in range(n1, 2 * n1):
            self.exp[i] = self.exp[i - n1]

    # -- raw polynomial arithmetic used to build the tables --
    def _digits(self, e):
        d = []
        for _ in range(self.m):
            d.append(e % self.p)
            e //= self.p
        return d

    def _from_digits(self, d):
        v = 0
        for i in reversed(range(self.m)):
            v = v * self.p + d[i] % self.p
        return v

    def _mul_alpha(self, e, poly):
        p, m = self.p, self.m
        if m == 1:
            return (e * ((p - poly[0]) % p)) % p
        d = [0] + self._digits(e)          # multiply by x
        top = d[m]
        for i in range(m):
            d[i] = (d[i] - top * poly[i]) % p
        return self._from_digits(d[:m])

    def _order_of_x(self, poly):
        e, k = 1, 0
        while True:
            e = self._mul_alpha(e, poly)
            k += 1
            if e == 1 or k > self.order:
                return k

    def _is_primitive(self, poly):
        if len(poly) != self.m + 1 or poly[-1] != 1 or poly[0] % self.p == 0:
            return False
        return self._order_of_x(poly) == self.order - 1

    def _first_primitive(self):
        p, m = self.p, self.m
        for v in range(p ** m):
            poly = [(v // p ** i) % p for i in range(m)] + [1]
            if poly[0] != 0 and self._is_primitive(poly):
                return poly
        raise ValueError("no primitive polynomial")

    # -- field operations --
    def add(self, a, b):
        p, r, w = self.p, 0, 1
        while a or b:
            r += ((a % p + b % p) % p) * w
            a //= p
            b //= p
            w *= p
        return r

    def neg(self, a):
        p, r, w = self.p, 0, 1
        while a:
            r += ((-(a % p)) % p) * w
            a //= p
            w *= p
        return r

    def sub(self, a, b):
        return self.add(a, self.neg(b))

    def mul(self, a, b):
        if a == 0 or b == 0:
            return 0
        return self.exp[self.log[a] + self.log[b]]

    def inv(self, a):
        return self.exp[(self.order - 1 - self.log[a]) % (self.order - 1)]

    def pow_alpha(self, k):
        return self.exp[k % (self.order - 1)]

    def vector(self, a):
        """GF(p) coefficients, highest degree first (galois ``.vector()``)."""
        return list(reversed(self._digits(a)))

    def from_vector(self, v):
        return self._from_digits(list(reversed([int(x) % self.p for x in v])))


class ReedSolomonOracle:
    """Restatement of qsft/ReedSolomon.py (see module docstring)."""

    def __init__(self, n, t, q):
        s = math.ceil(math.log(n) / math.log(q))  # qsft/ReedSolomon.py:20
        if n > q ** s - 1:                         # qsft/ReedSolomon.py:21-22
            s += 1
        self.s, self.ns, self.t, self.q = s, n, t, q
        self.gf = GF(q, s)
        self.nt = q ** s - 1
        self.c = 1

    def H(self, j, i):
        """Parity-check entry for syndrome j and source position i (last ns columns)."""
        return self.gf.pow_alpha((self.c + j) * (self.ns - 1 - i))

    def get_parity_length(self):  # qsft/ReedSolomon.py:67-74
        return 2 * self.t * self.s

    def get_delay_matrix(self):  # qsft/ReedSolomon.py:50-65
        s, ns, t = self.s, self.ns, self.t
        D = [[0] * ns for _ in range(2 * t * s + 1)]
        for i in range(ns):
            for j in range(2 * t):
                vec = self.gf.vector(self.H(j, i))
                for mm in range(s):
                    D[s * j + 1 + mm][i] = vec[mm]
        return D

    def syndromes_of(self, k):
        """GF(q^s) syndromes S_j = sum_i k_i H[j,i] (what D_src @ k encodes)."""
        gf = self.gf
        out = []
        for j in range(2 * self.t):
            acc = 0
            for i, ki in enumerate(k):
                if ki % self.q:
                    acc = gf.add(acc, gf.mul(ki % self.q, self.H(j, i)))
            out.append(acc)
        return out

    def decode_syndromes(self, S):
        """Berlekamp-Massey + Chien + Forney.  Returns the length-nt error vector
        (index 0 = highest degree) or None on failure."""
        gf, t, nt = self.gf, self.t, self.nt
        if all(v == 0 for v in S):
            return [0] * nt
        # Berlekamp-Massey (Massey 1969): connection polynomial Lambda, ascending
        lam = [1]
        prev = [1]
        L, mshift, bcoef = 0, 1, 1
        for r in range(2 * t):
            d = S[r]
            for i in range(1, L + 1):
                if i < len(lam):
                    d = gf.add(d, gf.mul(lam[i], S[r - i]))
            if d == 0:
                mshift += 1
                continue
            coef = gf.mul(d, gf.inv(bcoef))
            tmp = lam[:]
            need = len(prev) + mshift
            if len(lam) < need:
                lam = lam + [0] * (need - len(lam))
            for i, pv in enumerate(prev):
                lam[i + mshift] = gf.sub(lam[i + mshift], gf.mul(coef, pv))
            if 2 * L <= r:
                L = r + 1 - L
                prev = tmp
                bcoef = d
                mshift = 1
            else:
                mshift += 1
        while len(lam) > 1 and lam[-1] == 0:
            lam.pop()
        deg = len(lam) - 1
        if deg > t or deg != L:
            return None
        # Chien search over degrees d of the codeword polynomial: X = alpha^d
        roots = []
        for dgr in range(nt):
            xinv = gf.pow_alpha(-dgr)
            acc, pw = 0, 1
            for coef in lam:
                acc = gf.add(acc, gf.mul(coef, pw))
                pw = gf.mul(pw, xinv)
            if acc == 0:
                roots.append(dgr)
        if len(roots) != deg:
            return None
        # Forney: Omega = S(x) Lambda(x) mod x^{2t};  e = -X^{1-c} Omega(X^-1) / Lambda'(X^-1)
        om = [0] * (2 * t)
        for i in range(2 * t):
            acc = 0
            for j in range(0, min(i, deg) + 1):
                acc = gf.add(acc, gf.mul(lam[j], S[i - j]))
            om[i] = acc
        dlam = []  # formal derivative
        for i in range(1, deg + 1):
            c = lam[i]
            v = 0
            for _ in range(i % self.gf.p):
                v = gf.add(v, c)
            dlam.append(v)
        err = [0] * nt
        for dgr in roots:
            X = gf.pow_alpha(dgr)
            xinv = gf.pow_alpha(-dgr)
            num, pw = 0, 1
            for coef in om:
                num = gf.add(num, gf.mul(coef, pw))
                pw = gf.mul(pw, xinv)
            den, pw = 0, 1
            for coef in dlam:
                den = gf.add(den, gf.mul(coef, pw))
                pw = gf.mul(pw, xinv)
            if den == 0:
                return None
            val = gf.neg(gf.mul(num, gf.inv(den)))
            val = gf.mul(val, gf.pow_alpha((1 - self.c) * dgr))
            _ = X
            err[nt - 1 - dgr] = val
        return err

    def syndrome_decode(self, syndrome):
        """Mirror of ReedSolomon.syndrome_decode (qsft/ReedSolomon.py:26-48):
        returns (array of shape (1, ns), n_errors) like the reference."""
        import numpy as np
        s = self.s
        S = [self.gf.from_vector(syndrome[s * j:s * (j + 1)]) for j in range(2 * self.t)]
        err = self.decode_syndromes(S)
        if err is None:
            return np.zeros((1, self.ns), dtype=np.int64), -1
        tail = err[-self.ns:]
        return np.array([tail], dtype=np.int64), sum(1 for v in err if v)


def get_reed_solomon_dec(n, t_max, q):
    """Mirror of qsft/query.py:231-243 (including its prime list)."""
    primeset = [2, 3, 5, 7, 11, 13, 15, 17, 19, 23, 29]
    if q in primeset:
        return ReedSolomonOracle(n, t_max, q).syndrome_decode
    raise NotImplementedError("q is not a prime number under 30!")
