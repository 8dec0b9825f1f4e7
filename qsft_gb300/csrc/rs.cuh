// GF(q^s) arithmetic on exp / log / Zech-logarithm tables and the
// Reed-Solomon syndrome decoder used by singleton detection.
#pragma once
#include "common.cuh"

namespace qsft {

struct GFt {
  const int32_t* exp;   // [2*ord1]
  const int32_t* log;   // [ord1+1], log[0] = -1
  const int32_t* zech;  // [ord1], log(1 + alpha^k) or -1 when 1 + alpha^k = 0
  int ord1, neg1, p;
};
__device__ __forceinline__ int gf_add(const GFt& g, int a, int b) {
  if (a == 0) return b;
  if (b == 0) return a;
  const int la = g.log[a], lb = g.log[b];
  int d = lb - la;
  if (d < 0) d += g.ord1;
  const int z = g.zech[d];
  if (z < 0) return 0;
  return g.exp[la + z];
}
__device__ __forceinline__ int gf_mul(const GFt& g, int a, int b) {
  if (a == 0 || b == 0) return 0;
  return g.exp[g.log[a] + g.log[b]];
}
__device__ __forceinline__ int gf_inv(const GFt& g, int a) { return g.exp[(g.ord1 - g.log[a]) % g.ord1]; }
__device__ __forceinline__ int gf_neg(const GFt& g, int a) { return a == 0 ? 0 : g.exp[g.log[a] + g.neg1]; }
__device__ __forceinline__ int gf_sub(const GFt& g, int a, int b) { return gf_add(g, a, gf_neg(g, b)); }
__device__ __forceinline__ int gf_pow_alpha(const GFt& g, int k) {
  k %= g.ord1;
  if (k < 0) k += g.ord1;
  return g.exp[k];
}

// Syndrome decoding of a primitive narrow-sense RS[q^s-1, q^s-1-2t] code
// (qsft/ReedSolomon.py:26-48): Berlekamp-Massey, Chien search, Forney.
// syms: 2ts q-ary symbols (MSB-first digits of the 2t syndromes).  On success
// the error value v on each of the last n positions is written as
// k[i] = v mod q and khi[i] = v / q, v being the integer form of the GF(q^s)
// element (sum of its coefficients c_m q^m).  The reference returns v itself
// (np.array of the decoded field elements, qsft/reconstruct.py:34-51), so a
// value outside GF(q) gives a k entry >= q: it behaves as v mod q in every
// later computation (signatures and bin indices are taken mod q) but is a key
// of its own; khi keeps that key.  v < q^s and q^(s-1) <= n, so khi < 128.
// A decoding failure leaves k = khi = 0 (the all-zero received word).
static __device__ void rs_decode(const GFt& g, int q, int s, int t, int n, const uint8_t* syms, uint8_t* k,
                                 uint8_t* khi) {
  constexpr int CAP = 2 * QSFT_MAX_RS_T + 2;
  for (int i = 0; i < n; ++i) k[i] = khi[i] = 0;
  int S[2 * QSFT_MAX_RS_T];
  bool any = false;
  for (int j = 0; j < 2 * t; ++j) {
    int v = 0;
    for (int m = 0; m < s; ++m) v = v * q + syms[s * j + m];
    S[j] = v;
    any |= v != 0;
  }
  if (!any) return;
  int lam[CAP], prev[CAP], tmp[CAP];
  int lam_len = 1, prev_len = 1, L = 0, mshift = 1, bc = 1;
  lam[0] = 1;
  prev[0] = 1;
  for (int r = 0; r < 2 * t; ++r) {
    int d = S[r];
    for (int i = 1; i <= L && i < lam_len; ++i) d = gf_add(g, d, gf_mul(g, lam[i], S[r - i]));
    if (d == 0) {
      ++mshift;
      continue;
    }
    const int coef = gf_mul(g, d, gf_inv(g, bc));
    for (int i = 0; i < lam_len; ++i) tmp[i] = lam[i];
    const int tmp_len = lam_len;
    const int need = prev_len + mshift;
    if (need > CAP) return;
    for (int i = lam_len; i < need; ++i) lam[i] = 0;
    if (need > lam_len) lam_len = need;
    for (int i = 0; i < prev_len; ++i) lam[i + mshift] = gf_sub(g, lam[i + mshift], gf_mul(g, coef, prev[i]));
    if (2 * L <= r) {
      L = r + 1 - L;
      for (int i = 0; i < tmp_len; ++i) prev[i] = tmp[i];
      prev_len = tmp_len;
      bc = d;
      mshift = 1;
    } else {
      ++mshift;
    }
  }
  while (lam_len > 1 && lam[lam_len - 1] == 0) --lam_len;
  const int deg = lam_len - 1;
  if (deg > t || deg != L) return;
  int roots[QSFT_MAX_RS_T];
  int nroots = 0;
  for (int dg = 0; dg < g.ord1; ++dg) {
    const int xinv = gf_pow_alpha(g, -dg);
    int acc = lam[deg];
    for (int i = deg - 1; i >= 0; --i) acc = gf_add(g, gf_mul(g, acc, xinv), lam[i]);
    if (acc == 0) {
      if (nroots >= deg) return;
      roots[nroots++] = dg;
    }
  }
  if (nroots != deg) return;
  int om[2 * QSFT_MAX_RS_T];
  for (int i = 0; i < 2 * t; ++i) {
    int acc = 0;
    for (int j = 0; j <= i && j <= deg; ++j) acc = gf_add(g, acc, gf_mul(g, lam[j], S[i - j]));
    om[i] = acc;
  }
  const int nt = g.ord1;
  int16_t kk[QSFT_MAX_N];
  for (int i = 0; i < n; ++i) kk[i] = 0;
  for (int r = 0; r < nroots; ++r) {
    const int dg = roots[r];
    const int xinv = gf_pow_alpha(g, -dg);
    int num = 0, pw = 1;
    for (int i = 0; i < 2 * t; ++i) {
      num = gf_add(g, num, gf_mul(g, om[i], pw));
      pw = gf_mul(g, pw, xinv);
    }
    int den = 0;
    pw = 1;
    for (int i = 1; i <= deg; ++i) {
      const int ip = i % g.p;
      if (ip) den = gf_add(g, den, gf_mul(g, gf_mul(g, lam[i], ip), pw));
      pw = gf_mul(g, pw, xinv);
    }
    if (den == 0) return;
    const int val = gf_neg(g, gf_mul(g, num, gf_inv(g, den)));  // c = 1: X^(1-c) = 1
    const int pos = nt - 1 - dg;
    if (pos >= nt - n) kk[pos - (nt - n)] = (int16_t)val;
  }
  for (int i = 0; i < n; ++i) {
    k[i] = (uint8_t)(kk[i] % q);
    khi[i] = (uint8_t)(kk[i] / q);
  }
}

// Table layout at `tb` (built by the host): exp[2*(q^s-1)] | log[q^s] | zech[q^s-1].
__device__ __forceinline__ GFt make_gf(const int32_t* tb, int q, int s) {
  int order = 1;
  for (int i = 0; i < s; ++i) order *= q;
  GFt g;
  g.ord1 = order - 1;
  g.exp = tb;
  g.log = tb + 2 * g.ord1;
  g.zech = g.log + order;
  g.p = q;
  g.neg1 = (q == 2) ? 0 : g.ord1 / 2;
  return g;
}

}  // namespace qsft
