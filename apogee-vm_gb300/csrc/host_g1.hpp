// Host-side BN254 G1 arithmetic for MSMs over a handful of points, where the
// work is one serial chain: a weighted sum of a few commitments (the stacked
// opening's cm* = sum_j w_j cm_j, crates/pcs/src/lib.rs:568-581). On the
// device such a sum is a windowed Horner of about 255 dependent doublings in
// one thread, each a chain of Montgomery products of about a microsecond's
// latency; one host core does a product in about 18 ns.
//
// Fq in Montgomery form over four 64-bit limbs (R = 2^256); points in Jacobian
// coordinates on y^2 = x^3 + 3 with the published formulas dbl-2009-l,
// add-2007-bl and madd-2007-bl (Explicit-Formulas Database); the sum is
// Straus's method with 4-bit windows, affine multiples and one shared
// doubling chain.
#pragma once
#include <cstdint>
#include <cstring>
#include <vector>

#include "host_fr.hpp"

namespace apg {
namespace host {
namespace g1 {

// The base field's modulus (little-endian 64-bit limbs); R, R^2 and -q^-1 are
// derived from it once.
static constexpr uint64_t kQ[4] = {0x3c208c16d87cfd47ull, 0x97816a916871ca8dull, 0xb85045b68181585dull,
                                   0x30644e72e131a029ull};

struct Q {
  uint64_t w[4];
};

struct QConsts {
  uint64_t inv;  // -q^-1 mod 2^64
  Q one, r2;     // R mod q, R^2 mod q
  QConsts() {
    uint64_t x = 1;  // q^-1 mod 2^64 by Newton's iteration
    for (int i = 0; i < 6; ++i) x *= 2 - kQ[0] * x;
    inv = 0 - x;
    uint64_t t[4] = {1, 0, 0, 0};
    for (int i = 0; i < 512; ++i) {
      dbl_mod(t);
      if (i == 255) memcpy(one.w, t, 32);
    }
    memcpy(r2.w, t, 32);
  }
  static bool geq_q(const uint64_t a[4]) {
    for (int i = 3; i >= 0; --i)
      if (a[i] != kQ[i]) return a[i] > kQ[i];
    return true;
  }
  static void sub_q(uint64_t a[4]) {
    uint64_t br = 0;
    for (int i = 0; i < 4; ++i) {
      const u128 d = (u128)a[i] - kQ[i] - br;
      a[i] = (uint64_t)d;
      br = (uint64_t)(d >> 127);
    }
  }
  // a <- 2a mod q for a < q (q < 2^254, so 2a never leaves 256 bits).
  static void dbl_mod(uint64_t a[4]) {
    uint64_t c = 0;
    for (int i = 0; i < 4; ++i) {
      const uint64_t n = (a[i] << 1) | c;
      c = a[i] >> 63;
      a[i] = n;
    }
    if (geq_q(a)) sub_q(a);
  }
};

inline const QConsts& qc() {
  static const QConsts k;
  return k;
}

inline Q qzero() { return Q{{0, 0, 0, 0}}; }
inline bool qis_zero(const Q& a) { return (a.w[0] | a.w[1] | a.w[2] | a.w[3]) == 0; }
inline bool qeq(const Q& a, const Q& b) { return memcmp(a.w, b.w, 32) == 0; }

inline Q qadd(const Q& a, const Q& b) {
  Q r;
  uint64_t c = 0;
  for (int i = 0; i < 4; ++i) {
    const u128 s = (u128)a.w[i] + b.w[i] + c;
    r.w[i] = (uint64_t)s;
    c = (uint64_t)(s >> 64);
  }
  if (QConsts::geq_q(r.w)) QConsts::sub_q(r.w);
  return r;
}

inline Q qsub(const Q& a, const Q& b) {
  Q r;
  uint64_t br = 0;
  for (int i = 0; i < 4; ++i) {
    const u128 d = (u128)a.w[i] - b.w[i] - br;
    r.w[i] = (uint64_t)d;
    br = (uint64_t)(d >> 127);
  }
  if (br) {
    uint64_t c = 0;
    for (int i = 0; i < 4; ++i) {
      const u128 s = (u128)r.w[i] + kQ[i] + c;
      r.w[i] = (uint64_t)s;
      c = (uint64_t)(s >> 64);
    }
  }
  return r;
}

// Montgomery product, the full 512-bit product first, then the reduction a
// limb at a time (the same shape as host_fr.hpp's fmul_r), reduced to [0, q).
inline Q qmul(const Q& A, const Q& B) {
  const uint64_t *a = A.w, *b = B.w;
  const uint64_t inv = qc().inv;
  u128 col[9];
  for (int k = 0; k < 9; ++k) col[k] = 0;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      const u128 pr = (u128)a[i] * b[j];
      col[i + j] += (uint64_t)pr;
      col[i + j + 1] += (uint64_t)(pr >> 64);
    }
  for (int i = 0; i < 4; ++i) {
    const uint64_t lo = (uint64_t)col[i];
    const uint64_t m = lo * inv;
    col[i + 1] += (uint64_t)(col[i] >> 64) + (uint64_t)(lo != 0);
    const u128 q0 = (u128)m * kQ[0], q1 = (u128)m * kQ[1], q2 = (u128)m * kQ[2], q3 = (u128)m * kQ[3];
    col[i + 1] += (u128)(uint64_t)(q0 >> 64) + (uint64_t)q1;
    col[i + 2] += (u128)(uint64_t)(q1 >> 64) + (uint64_t)q2;
    col[i + 3] += (u128)(uint64_t)(q2 >> 64) + (uint64_t)q3;
    col[i + 4] += (uint64_t)(q3 >> 64);
  }
  Q r;
  u128 c = 0;
  for (int k = 0; k < 4; ++k) {
    c += col[4 + k];
    r.w[k] = (uint64_t)c;
    c >>= 64;
  }
  if (QConsts::geq_q(r.w)) QConsts::sub_q(r.w);
  return r;
}

inline Q qsqr(const Q& a) { return qmul(a, a); }

// Canonical limbs (below q) <-> Montgomery form.
inline Q q_from_canonical(const uint64_t c[4]) { return qmul(Q{{c[0], c[1], c[2], c[3]}}, qc().r2); }
inline void q_to_canonical(const Q& a, uint64_t out[4]) { memcpy(out, qmul(a, Q{{1, 0, 0, 0}}).w, 32); }

// 1/a by Fermat (a^(q-2)); a != 0.
inline Q qinv(const Q& a) {
  uint64_t e[4] = {kQ[0] - 2, kQ[1], kQ[2], kQ[3]};
  Q acc = qc().one, base = a;
  for (int i = 0; i < 4; ++i)
    for (int bit = 0; bit < 64; ++bit) {
      if ((e[i] >> bit) & 1) acc = qmul(acc, base);
      base = qsqr(base);
    }
  return acc;
}

// Jacobian (X, Y, Z) = (X/Z^2, Y/Z^3); Z = 0 is the point at infinity.
struct Jac {
  Q x, y, z;
};

inline Jac jinf() { return Jac{qc().one, qc().one, qzero()}; }
inline bool jis_inf(const Jac& p) { return qis_zero(p.z); }

// dbl-2009-l (a = 0).
inline Jac jdbl(const Jac& p) {
  if (jis_inf(p) || qis_zero(p.y)) return jinf();
  const Q A = qsqr(p.x), B = qsqr(p.y), C = qsqr(B);
  Q D = qsub(qsub(qsqr(qadd(p.x, B)), A), C);
  D = qadd(D, D);
  const Q E = qadd(qadd(A, A), A), F = qsqr(E);
  Jac r;
  r.x = qsub(F, qadd(D, D));
  Q c8 = qadd(C, C);
  c8 = qadd(c8, c8);
  c8 = qadd(c8, c8);
  r.y = qsub(qmul(E, qsub(D, r.x)), c8);
  const Q yz = qmul(p.y, p.z);
  r.z = qadd(yz, yz);
  return r;
}

// add-2007-bl, with the cases it excludes (an infinity, P = Q, P = -Q).
inline Jac jadd(const Jac& p, const Jac& q) {
  if (jis_inf(p)) return q;
  if (jis_inf(q)) return p;
  const Q z1z1 = qsqr(p.z), z2z2 = qsqr(q.z);
  const Q u1 = qmul(p.x, z2z2), u2 = qmul(q.x, z1z1);
  const Q s1 = qmul(qmul(p.y, q.z), z2z2), s2 = qmul(qmul(q.y, p.z), z1z1);
  const Q h = qsub(u2, u1);
  Q rr = qsub(s2, s1);
  if (qis_zero(h)) return qis_zero(rr) ? jdbl(p) : jinf();
  const Q h2 = qadd(h, h), I = qsqr(h2), J = qmul(h, I);
  rr = qadd(rr, rr);
  const Q V = qmul(u1, I);
  Jac r;
  r.x = qsub(qsub(qsqr(rr), J), qadd(V, V));
  const Q s1j = qmul(s1, J);
  r.y = qsub(qmul(rr, qsub(V, r.x)), qadd(s1j, s1j));
  r.z = qmul(qsub(qsub(qsqr(qadd(p.z, q.z)), z1z1), z2z2), h);
  return r;
}

// An affine point (inf: the point at infinity).
struct Aff {
  Q x, y;
  bool inf;
};

// madd-2007-bl (Jacobian plus affine), with the cases it excludes.
inline Jac jadd_aff(const Jac& p, const Aff& q) {
  if (q.inf) return p;
  if (jis_inf(p)) return Jac{q.x, q.y, qc().one};
  const Q z1z1 = qsqr(p.z);
  const Q u2 = qmul(q.x, z1z1), s2 = qmul(qmul(q.y, p.z), z1z1);
  const Q h = qsub(u2, p.x);
  Q rr = qsub(s2, p.y);
  if (qis_zero(h)) return qis_zero(rr) ? jdbl(p) : jinf();
  const Q hh = qsqr(h);
  Q i4 = qadd(hh, hh);
  i4 = qadd(i4, i4);
  const Q J = qmul(h, i4);
  rr = qadd(rr, rr);
  const Q V = qmul(p.x, i4);
  Jac r;
  r.x = qsub(qsub(qsqr(rr), J), qadd(V, V));
  const Q yj = qmul(p.y, J);
  r.y = qsub(qmul(rr, qsub(V, r.x)), qadd(yj, yj));
  r.z = qsub(qsub(qsqr(qadd(p.z, h)), z1z1), hh);
  return r;
}

// Jacobian points to affine with one inversion (Montgomery's batch trick).
inline std::vector<Aff> to_affine(const std::vector<Jac>& pts) {
  const size_t n = pts.size();
  std::vector<Aff> out(n);
  std::vector<Q> pre(n + 1);
  pre[0] = qc().one;
  for (size_t i = 0; i < n; ++i) pre[i + 1] = jis_inf(pts[i]) ? pre[i] : qmul(pre[i], pts[i].z);
  Q inv = qinv(pre[n]);
  for (size_t i = n; i-- > 0;) {
    if (jis_inf(pts[i])) {
      out[i].inf = true;
      continue;
    }
    const Q zi = qmul(inv, pre[i]), zi2 = qsqr(zi);
    inv = qmul(inv, pts[i].z);
    out[i] = Aff{qmul(pts[i].x, zi2), qmul(pts[i].y, qmul(zi2, zi)), false};
  }
  return out;
}

// A canonical 64-byte encoding (x || y, little-endian; all zero = infinity)
// as a Jacobian point. The caller has validated it (coordinates below q, on
// the curve).
// A canonical 64-byte encoding (x then y, little-endian) of a point on
// y^2 = x^3 + 3, or all zero (the point at infinity). G1 has cofactor 1, so a
// point on the curve is in the order-r subgroup.
inline bool valid_encoding(const uint8_t b[64]) {
  bool inf = true;
  for (int i = 0; i < 64; ++i) inf &= b[i] == 0;
  if (inf) return true;
  uint64_t x[4], y[4];
  memcpy(x, b, 32);
  memcpy(y, b + 32, 32);
  if (QConsts::geq_q(x) || QConsts::geq_q(y)) return false;
  const uint64_t three[4] = {3, 0, 0, 0};
  const Q X = q_from_canonical(x), Y = q_from_canonical(y);
  return qeq(qmul(Y, Y), qadd(qmul(qmul(X, X), X), q_from_canonical(three)));
}

inline Jac jfrom_bytes(const uint8_t b[64]) {
  bool inf = true;
  for (int i = 0; i < 64; ++i) inf &= b[i] == 0;
  if (inf) return jinf();
  uint64_t x[4], y[4];
  memcpy(x, b, 32);
  memcpy(y, b + 32, 32);
  return Jac{q_from_canonical(x), q_from_canonical(y), qc().one};
}

inline void jto_bytes(const Jac& p, uint8_t out[64]) {
  if (jis_inf(p)) {
    memset(out, 0, 64);
    return;
  }
  const Q zi = qinv(p.z), zi2 = qsqr(zi), zi3 = qmul(zi2, zi);
  uint64_t x[4], y[4];
  q_to_canonical(qmul(p.x, zi2), x);
  q_to_canonical(qmul(p.y, zi3), y);
  memcpy(out, x, 32);
  memcpy(out + 32, y, 32);
}

// sum_j scalars[j] * points[j]: points as canonical 64-byte encodings,
// scalars as host Fr (Montgomery). Straus with 4-bit windows: each point's
// multiples 1..15 (made affine together with one inversion), then 64 windows
// from the top, four doublings and one mixed addition a nonzero nibble each,
// so one chain of 252 doublings serves every point.
inline void msm_small(const uint8_t* points, const F* scalars, size_t n, uint8_t out[64]) {
  std::vector<Jac> tab(16 * n);
  std::vector<uint64_t> k(4 * n);
  for (size_t j = 0; j < n; ++j) {
    tab[16 * j] = jinf();
    tab[16 * j + 1] = jfrom_bytes(points + 64 * j);
    for (int d = 2; d < 16; ++d)
      tab[16 * j + d] = (d & 1) ? jadd(tab[16 * j + d - 1], tab[16 * j + 1]) : jdbl(tab[16 * j + d / 2]);
    to_canonical(scalars[j], &k[4 * j]);
  }
  const std::vector<Aff> aff = to_affine(tab);
  Jac acc = jinf();
  for (int w = 63; w >= 0; --w) {
    if (!jis_inf(acc))
      for (int s = 0; s < 4; ++s) acc = jdbl(acc);
    for (size_t j = 0; j < n; ++j) {
      const int d = (int)((k[4 * j + w / 16] >> (4 * (w % 16))) & 15u);
      if (d) acc = jadd_aff(acc, aff[16 * j + d]);
    }
  }
  jto_bytes(acc, out);
}

}  // namespace g1
}  // namespace host
}  // namespace apg
