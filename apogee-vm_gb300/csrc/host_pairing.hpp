// The optimal ate pairing on BN254 on the host, for the verifier's last step:
//
//   e(P, Q) = f_{6x+2, Q}(P) ^ ((q^12 - 1) / r),   x = 4965661367192848881,
//
// the Miller loop over the binary expansion of 6x + 2 closed by the two
// Frobenius lines (pi(Q), then -pi^2(Q)), then the exact final exponent
// (factored, each factor by square-and-multiply). The tower is Fq2 = Fq[u]/(u^2 + 1),
// Fq6 = Fq2[v]/(v^3 - xi), Fq12 = Fq6[w]/(w^2 - v) with xi = 9 + u; G2 is the
// D-type sextic twist E'/Fq2: y^2 = x^3 + 3/xi, mapped into E(Fq12) by
// (x, y) -> (x w^2, y w^3).
//
// The lines are evaluated in affine coordinates: the line through T and R on
// E' with slope lambda, at P = (xP, yP) in E(Fq), is
//
//   yP - lambda xP w + (lambda xT - yT) v w,
//
// and vertical lines, whose values lie in Fq6, are dropped (the final
// exponent's factor q^6 - 1 sends every element of Fq6 to 1). This is
// verification-side code: a pairing check runs a few times a proof, so
// nothing here is tuned (generic Fq12 products, a plain exponentiation).
#pragma once
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <vector>

#include "host_g1.hpp"

namespace apg {
namespace host {
namespace pairing {

using g1::Q;
using g1::qadd;
using g1::qsub;
using g1::qmul;
using g1::qzero;
using g1::qis_zero;
using g1::qeq;
using g1::qinv;
using g1::qc;
using g1::kQ;

inline Q qneg(const Q& a) { return qsub(qzero(), a); }
inline Q qsmall(uint64_t v) {
  const uint64_t c[4] = {v, 0, 0, 0};
  return g1::q_from_canonical(c);
}

// ---- exponents as little-endian 64-bit limbs ----------------------------------

typedef std::vector<uint64_t> Big;

inline void big_trim(Big& a) {
  while (!a.empty() && a.back() == 0) a.pop_back();
}

inline Big big_mul(const Big& a, const Big& b) {
  Big out(a.size() + b.size(), 0);
  for (size_t i = 0; i < a.size(); ++i) {
    u128 c = 0;
    for (size_t j = 0; j < b.size(); ++j) {
      c += (u128)a[i] * b[j] + out[i + j];
      out[i + j] = (uint64_t)c;
      c >>= 64;
    }
    out[i + b.size()] += (uint64_t)c;
  }
  big_trim(out);
  return out;
}

inline Big big_add(const Big& a, const Big& b) {
  Big out(std::max(a.size(), b.size()) + 1, 0);
  uint64_t c = 0;
  for (size_t i = 0; i + 1 < out.size(); ++i) {
    const u128 s = (u128)(i < a.size() ? a[i] : 0) + (i < b.size() ? b[i] : 0) + c;
    out[i] = (uint64_t)s;
    c = (uint64_t)(s >> 64);
  }
  out.back() = c;
  big_trim(out);
  return out;
}

inline int big_cmp(const Big& a, const Big& b) {
  if (a.size() != b.size()) return a.size() < b.size() ? -1 : 1;
  for (size_t i = a.size(); i-- > 0;)
    if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
  return 0;
}

// a - b for a >= b.
inline Big big_sub(const Big& a, const Big& b) {
  Big out(a);
  uint64_t br = 0;
  for (size_t i = 0; i < out.size(); ++i) {
    const u128 d = (u128)out[i] - (i < b.size() ? b[i] : 0) - br;
    out[i] = (uint64_t)d;
    br = (uint64_t)(d >> 127);
  }
  big_trim(out);
  return out;
}

inline size_t big_bits(const Big& a) {
  if (a.empty()) return 0;
  size_t n = 64 * (a.size() - 1);
  for (uint64_t t = a.back(); t; t >>= 1) ++n;
  return n;
}

inline bool big_bit(const Big& a, size_t i) { return i / 64 < a.size() && ((a[i / 64] >> (i % 64)) & 1); }

// Floor quotient by binary long division.
inline Big big_div(const Big& a, const Big& d) {
  Big q(a.size(), 0), rem;
  for (size_t i = big_bits(a); i-- > 0;) {
    uint64_t carry = big_bit(a, i) ? 1 : 0;  // rem = 2 rem + bit i of a
    for (auto& limb : rem) {
      const uint64_t n = (limb << 1) | carry;
      carry = limb >> 63;
      limb = n;
    }
    if (carry) rem.push_back(carry);
    if (big_cmp(rem, d) >= 0) {
      rem = big_sub(rem, d);
      q[i / 64] |= 1ull << (i % 64);
    }
  }
  big_trim(q);
  return q;
}

inline Big big_from4(const uint64_t w[4]) {
  Big b(w, w + 4);
  big_trim(b);
  return b;
}

// ---- Fq2 = Fq[u]/(u^2 + 1) ------------------------------------------------------

struct F2 {
  Q c0, c1;
};

inline F2 f2zero() { return F2{qzero(), qzero()}; }
inline F2 f2one() { return F2{qc().one, qzero()}; }
inline F2 f2add(const F2& a, const F2& b) { return F2{qadd(a.c0, b.c0), qadd(a.c1, b.c1)}; }
inline F2 f2sub(const F2& a, const F2& b) { return F2{qsub(a.c0, b.c0), qsub(a.c1, b.c1)}; }
inline F2 f2neg(const F2& a) { return F2{qneg(a.c0), qneg(a.c1)}; }
inline F2 f2conj(const F2& a) { return F2{a.c0, qneg(a.c1)}; }
inline bool f2is_zero(const F2& a) { return qis_zero(a.c0) && qis_zero(a.c1); }
inline bool f2eq(const F2& a, const F2& b) { return qeq(a.c0, b.c0) && qeq(a.c1, b.c1); }
inline F2 f2mul(const F2& a, const F2& b) {
  return F2{qsub(qmul(a.c0, b.c0), qmul(a.c1, b.c1)), qadd(qmul(a.c0, b.c1), qmul(a.c1, b.c0))};
}
inline F2 f2sqr(const F2& a) { return f2mul(a, a); }
inline F2 f2mul_q(const F2& a, const Q& k) { return F2{qmul(a.c0, k), qmul(a.c1, k)}; }
// 1/(a0 + a1 u) = (a0 - a1 u)/(a0^2 + a1^2); a != 0.
inline F2 f2inv(const F2& a) {
  const Q t = qinv(qadd(qmul(a.c0, a.c0), qmul(a.c1, a.c1)));
  return F2{qmul(a.c0, t), qneg(qmul(a.c1, t))};
}
// a * xi, xi = 9 + u: (9 a0 - a1) + (9 a1 + a0) u.
inline F2 f2mul_xi(const F2& a) {
  auto nine = [](const Q& x) {
    const Q x2 = qadd(x, x), x4 = qadd(x2, x2), x8 = qadd(x4, x4);
    return qadd(x8, x);
  };
  return F2{qsub(nine(a.c0), a.c1), qadd(nine(a.c1), a.c0)};
}
inline F2 f2pow(F2 base, const Big& e) {
  F2 acc = f2one();
  for (size_t i = big_bits(e); i-- > 0;) {
    acc = f2sqr(acc);
    if (big_bit(e, i)) acc = f2mul(acc, base);
  }
  return acc;
}

// ---- Fq6 = Fq2[v]/(v^3 - xi) ------------------------------------------------------

struct F6 {
  F2 c0, c1, c2;
};

inline F6 f6zero() { return F6{f2zero(), f2zero(), f2zero()}; }
inline F6 f6one() { return F6{f2one(), f2zero(), f2zero()}; }
inline F6 f6add(const F6& a, const F6& b) { return F6{f2add(a.c0, b.c0), f2add(a.c1, b.c1), f2add(a.c2, b.c2)}; }
inline F6 f6sub(const F6& a, const F6& b) { return F6{f2sub(a.c0, b.c0), f2sub(a.c1, b.c1), f2sub(a.c2, b.c2)}; }
inline F6 f6neg(const F6& a) { return F6{f2neg(a.c0), f2neg(a.c1), f2neg(a.c2)}; }
inline bool f6eq(const F6& a, const F6& b) { return f2eq(a.c0, b.c0) && f2eq(a.c1, b.c1) && f2eq(a.c2, b.c2); }
// Schoolbook, v^3 = xi folding the three high products.
inline F6 f6mul(const F6& a, const F6& b) {
  return F6{f2add(f2mul(a.c0, b.c0), f2mul_xi(f2add(f2mul(a.c1, b.c2), f2mul(a.c2, b.c1)))),
            f2add(f2add(f2mul(a.c0, b.c1), f2mul(a.c1, b.c0)), f2mul_xi(f2mul(a.c2, b.c2))),
            f2add(f2add(f2mul(a.c0, b.c2), f2mul(a.c1, b.c1)), f2mul(a.c2, b.c0))};
}
// a * v = c2 xi + c0 v + c1 v^2.
inline F6 f6mul_v(const F6& a) { return F6{f2mul_xi(a.c2), a.c0, a.c1}; }
// 1/a through the norm to Fq2: with t0 = c0^2 - xi c1 c2, t1 = xi c2^2 - c0 c1,
// t2 = c1^2 - c0 c2, a (t0 + t1 v + t2 v^2) = c0 t0 + xi (c2 t1 + c1 t2).
inline F6 f6inv(const F6& a) {
  const F2 t0 = f2sub(f2sqr(a.c0), f2mul_xi(f2mul(a.c1, a.c2)));
  const F2 t1 = f2sub(f2mul_xi(f2sqr(a.c2)), f2mul(a.c0, a.c1));
  const F2 t2 = f2sub(f2sqr(a.c1), f2mul(a.c0, a.c2));
  const F2 d = f2add(f2mul(a.c0, t0), f2mul_xi(f2add(f2mul(a.c2, t1), f2mul(a.c1, t2))));
  const F2 di = f2inv(d);
  return F6{f2mul(t0, di), f2mul(t1, di), f2mul(t2, di)};
}

// ---- Fq12 = Fq6[w]/(w^2 - v) ------------------------------------------------------

struct F12 {
  F6 c0, c1;
};

inline F12 f12one() { return F12{f6one(), f6zero()}; }
inline bool f12eq(const F12& a, const F12& b) { return f6eq(a.c0, b.c0) && f6eq(a.c1, b.c1); }
inline F12 f12mul(const F12& a, const F12& b) {
  return F12{f6add(f6mul(a.c0, b.c0), f6mul_v(f6mul(a.c1, b.c1))),
             f6add(f6mul(a.c0, b.c1), f6mul(a.c1, b.c0))};
}
inline F12 f12sqr(const F12& a) { return f12mul(a, a); }
// 1/(c0 + c1 w) = (c0 - c1 w)/(c0^2 - v c1^2).
inline F12 f12inv(const F12& a) {
  const F6 di = f6inv(f6sub(f6mul(a.c0, a.c0), f6mul_v(f6mul(a.c1, a.c1))));
  return F12{f6mul(a.c0, di), f6neg(f6mul(a.c1, di))};
}
inline F12 f12pow(const F12& base, const Big& e) {
  F12 acc = f12one();
  for (size_t i = big_bits(e); i-- > 0;) {
    acc = f12sqr(acc);
    if (big_bit(e, i)) acc = f12mul(acc, base);
  }
  return acc;
}

// ---- constants derived once ---------------------------------------------------------

struct Consts {
  Big q, r, final_exp;  // (q^12 - 1)/r
  Big q2, hard;         // q^2 and (q^4 - q^2 + 1)/r
  F2 b2;                // 3/xi, the twist's constant
  F2 frob_x, frob_y;    // xi^((q-1)/3), xi^((q-1)/2): pi(x, y) = (conj(x) frob_x, conj(y) frob_y)
  Big loop;             // 6x + 2
  Consts() {
    q = big_from4(kQ);
    r = big_from4(host::kP);
    Big q12{1};
    for (int i = 0; i < 12; ++i) q12 = big_mul(q12, q);
    final_exp = big_div(big_sub(q12, Big{1}), r);
    q2 = big_mul(q, q);
    hard = big_div(big_sub(big_add(big_mul(q2, q2), Big{1}), q2), r);
    const F2 xi = f2mul_xi(f2one());
    b2 = f2mul(F2{qsmall(3), qzero()}, f2inv(xi));
    const Big qm1 = big_sub(q, Big{1});
    frob_x = f2pow(xi, big_div(qm1, Big{3}));
    frob_y = f2pow(xi, big_div(qm1, Big{2}));
    const u128 L = (u128)6 * 4965661367192848881ull + 2;
    loop = Big{(uint64_t)L, (uint64_t)(L >> 64)};
    big_trim(loop);
  }
};

inline const Consts& pc() {
  static const Consts k;
  return k;
}

// ---- G2 on the twist, affine ---------------------------------------------------------

struct G2 {
  F2 x, y;
  bool inf;
};

inline G2 g2inf() { return G2{f2zero(), f2zero(), true}; }
inline bool g2on_curve(const G2& p) {
  return p.inf || f2eq(f2sqr(p.y), f2add(f2mul(f2sqr(p.x), p.x), pc().b2));
}
inline G2 g2neg(const G2& p) { return p.inf ? p : G2{p.x, f2neg(p.y), false}; }
inline bool g2eq(const G2& a, const G2& b) {
  if (a.inf || b.inf) return a.inf == b.inf;
  return f2eq(a.x, b.x) && f2eq(a.y, b.y);
}

// The slope of the chord (or tangent) through a and b, false for a vertical
// line (b = -a, or a 2-torsion tangent).
inline bool g2slope(const G2& a, const G2& b, F2& lambda) {
  if (f2eq(a.x, b.x)) {
    if (!f2eq(a.y, b.y) || f2is_zero(a.y)) return false;
    const F2 x2 = f2sqr(a.x);
    lambda = f2mul(f2add(f2add(x2, x2), x2), f2inv(f2add(a.y, a.y)));
    return true;
  }
  lambda = f2mul(f2sub(b.y, a.y), f2inv(f2sub(b.x, a.x)));
  return true;
}

inline G2 g2add_with(const G2& a, const G2& b, const F2& lambda) {
  const F2 x = f2sub(f2sub(f2sqr(lambda), a.x), b.x);
  return G2{x, f2sub(f2mul(lambda, f2sub(a.x, x)), a.y), false};
}

inline G2 g2add(const G2& a, const G2& b) {
  if (a.inf) return b;
  if (b.inf) return a;
  F2 lambda;
  if (!g2slope(a, b, lambda)) return g2inf();
  return g2add_with(a, b, lambda);
}

inline G2 g2mul(const G2& p, const Big& k) {
  G2 acc = g2inf();
  for (size_t i = big_bits(k); i-- > 0;) {
    acc = g2add(acc, acc);
    if (big_bit(k, i)) acc = g2add(acc, p);
  }
  return acc;
}

inline bool g2in_subgroup(const G2& p) { return g2mul(p, pc().r).inf; }

inline G2 g2frob(const G2& p) {
  if (p.inf) return p;
  return G2{f2mul(f2conj(p.x), pc().frob_x), f2mul(f2conj(p.y), pc().frob_y), false};
}

// Canonical 128-byte encodings: x.c0 || x.c1 || y.c0 || y.c1, each a
// little-endian Fq below q; all zero is the point at infinity. Returns false
// for a coordinate at or above q, a point off the twist, or one outside the
// order-r subgroup (G2's cofactor is not 1).
inline bool g2from_bytes(const uint8_t b[128], G2& out) {
  bool zero = true;
  for (int i = 0; i < 128; ++i) zero &= b[i] == 0;
  if (zero) {
    out = g2inf();
    return true;
  }
  Q c[4];
  for (int i = 0; i < 4; ++i) {
    uint64_t w[4];
    memcpy(w, b + 32 * i, 32);
    if (g1::QConsts::geq_q(w)) return false;
    c[i] = g1::q_from_canonical(w);
  }
  out = G2{F2{c[0], c[1]}, F2{c[2], c[3]}, false};
  return g2on_curve(out) && g2in_subgroup(out);
}

inline void q_bytes(const Q& a, uint8_t* out) {
  uint64_t w[4];
  g1::q_to_canonical(a, w);
  memcpy(out, w, 32);
}

inline void g2to_bytes(const G2& p, uint8_t out[128]) {
  if (p.inf) {
    memset(out, 0, 128);
    return;
  }
  q_bytes(p.x.c0, out);
  q_bytes(p.x.c1, out + 32);
  q_bytes(p.y.c0, out + 64);
  q_bytes(p.y.c1, out + 96);
}

// c0 || c1 with each Fq6 as c0 || c1 || c2 and each Fq2 as c0 || c1: 384 bytes.
inline void f12to_bytes(const F12& a, uint8_t out[384]) {
  const F6* h[2] = {&a.c0, &a.c1};
  for (int i = 0; i < 2; ++i) {
    const F2* t[3] = {&h[i]->c0, &h[i]->c1, &h[i]->c2};
    for (int j = 0; j < 3; ++j) {
      q_bytes(t[j]->c0, out + 192 * i + 64 * j);
      q_bytes(t[j]->c1, out + 192 * i + 64 * j + 32);
    }
  }
}

// ---- the Miller loop and the pairing ----------------------------------------------------

// The line through T with slope lambda, at P: yP - lambda xP w + (lambda xT - yT) v w.
inline F12 line_at(const G2& t, const F2& lambda, const Q& xp, const Q& yp) {
  F12 l;
  l.c0 = F6{F2{yp, qzero()}, f2zero(), f2zero()};
  l.c1 = F6{f2neg(f2mul_q(lambda, xp)), f2sub(f2mul(lambda, t.x), t.y), f2zero()};
  return l;
}

// One step: f *= l_{T,R}(P), T += R (vertical lines contribute nothing).
inline void miller_step(F12& f, G2& t, const G2& r, const Q& xp, const Q& yp) {
  if (t.inf) {
    t = r;
    return;
  }
  if (r.inf) return;
  F2 lambda;
  if (!g2slope(t, r, lambda)) {
    t = g2inf();
    return;
  }
  f = f12mul(f, line_at(t, lambda, xp, yp));
  t = g2add_with(t, r, lambda);
}

// f_{6x+2,Q}(P) times the two Frobenius lines; P in affine Montgomery form.
inline F12 miller_loop(const Q& xp, const Q& yp, bool p_inf, const G2& q) {
  if (p_inf || q.inf) return f12one();
  const Big& L = pc().loop;
  F12 f = f12one();
  G2 t = q;
  for (size_t i = big_bits(L) - 1; i-- > 0;) {
    f = f12sqr(f);
    miller_step(f, t, t, xp, yp);
    if (big_bit(L, i)) miller_step(f, t, q, xp, yp);
  }
  const G2 q1 = g2frob(q), q2 = g2neg(g2frob(q1));
  miller_step(f, t, q1, xp, yp);
  miller_step(f, t, q2, xp, yp);
  return f;
}

// f^((q^12 - 1)/r) as ((f^(q^6 - 1))^(q^2 + 1))^((q^4 - q^2 + 1)/r), the same
// integer factored (r divides q^4 - q^2 + 1), with f^(q^6) = c0 - c1 w: the
// q^6-power map fixes Fq6 and sends w to -w, v being a non-square in Fq6.
inline F12 final_exponentiation(const F12& f) {
  const F12 f1 = f12mul(F12{f.c0, f6neg(f.c1)}, f12inv(f));
  const F12 f2 = f12mul(f12pow(f1, pc().q2), f1);
  return f12pow(f2, pc().hard);
}

// P from a canonical 64-byte G1 encoding (validated by the caller).
inline void g1_affine(const uint8_t b[64], Q& x, Q& y, bool& inf) {
  inf = true;
  for (int i = 0; i < 64; ++i) inf &= b[i] == 0;
  if (inf) return;
  uint64_t xw[4], yw[4];
  memcpy(xw, b, 32);
  memcpy(yw, b + 32, 32);
  x = g1::q_from_canonical(xw);
  y = g1::q_from_canonical(yw);
}

// prod_i e(P_i, Q_i) == 1, one final exponentiation for the product.
inline bool pairing_check(const std::vector<const uint8_t*>& ps, const std::vector<G2>& qs) {
  F12 f = f12one();
  for (size_t i = 0; i < ps.size(); ++i) {
    Q x, y;
    bool inf;
    g1_affine(ps[i], x, y, inf);
    f = f12mul(f, miller_loop(x, y, inf, qs[i]));
  }
  return f12eq(final_exponentiation(f), f12one());
}

}  // namespace pairing
}  // namespace host
}  // namespace apg
