// BN254 G1 (y^2 = x^3 + 3 over Fq) for the MSM: affine bases and XYZZ
// accumulators.
//
// XYZZ coordinates (X, Y, ZZ, ZZZ) stand for (X/ZZ, Y/ZZZ) with ZZ^3 = ZZZ^2;
// ZZ = 0 is the point at infinity. The formulas are the published ones for
// a = 0 short Weierstrass curves: madd-2008-s (8M + 2S, the bucket hot path),
// add-2008-s (12M + 2S), dbl-2008-s-1 and mdbl-2008-s-1. The reference keeps
// Jacobian coordinates (crates/curve/src/g1.rs:155-277); an MSM's value does
// not depend on the coordinates, and every result leaves the device as the
// canonical affine encoding (g1.rs:92-100), so parity is compared there.
//
// Device affine points carry Montgomery coordinates; (0, 0), which is not on
// the curve, encodes infinity.
#pragma once
#include "field.cuh"

namespace apg {

struct Affine {
  Fq x, y;
};

// The curve formulas call out-of-line Fq products: a point addition inlines
// ten of them, and ten inlined copies of a multiply overflow the instruction
// cache of a bucket-accumulation loop. The paired forms compute two
// independent products in one call (half the calls); each formula is written
// as pairs of products that do not depend on each other. In one thread the
// two products of a pair do not overlap, even written in lockstep (measured
// on GB300: 1164 cycles a product, 2412 a pair, 2434 a lockstep pair): a
// lone warp's product is bound by its own instruction issue, so the serial
// tails (bucket reduction, edge folds) cost about 17,000 cycles an XYZZ
// addition whatever the pairing.
struct Fq2 {
  Fq a, b;
};
static __device__ __noinline__ Fq cmul(const Fq a, const Fq b) { return fe_mul(a, b); }
static __device__ __noinline__ Fq csqr(const Fq a) { return fe_sqr(a); }
static __device__ __noinline__ Fq2 cmul2(const Fq a, const Fq b, const Fq c, const Fq d) {
  Fq2 r;
  r.a = fe_mul(a, b);
  r.b = fe_mul(c, d);
  return r;
}
static __device__ __noinline__ Fq2 csqr2(const Fq a, const Fq b) {
  Fq2 r;
  r.a = fe_sqr(a);
  r.b = fe_sqr(b);
  return r;
}

struct Xyzz {
  Fq x, y, zz, zzz;
};

__device__ __forceinline__ bool aff_is_inf(const Affine& p) { return fe_is_zero(p.x) && fe_is_zero(p.y); }

__device__ __forceinline__ Xyzz xyzz_inf() {
  Xyzz r;
  r.x = fe_zero<FqConsts>();
  r.y = fe_zero<FqConsts>();
  r.zz = fe_zero<FqConsts>();
  r.zzz = fe_zero<FqConsts>();
  return r;
}

__device__ __forceinline__ bool xyzz_is_inf(const Xyzz& p) { return fe_is_zero(p.zz); }

__device__ __forceinline__ Xyzz xyzz_from_affine(const Affine& a) {
  if (aff_is_inf(a)) return xyzz_inf();
  Xyzz r;
  r.x = a.x;
  r.y = a.y;
  r.zz = fe_one<FqConsts>();
  r.zzz = fe_one<FqConsts>();
  return r;
}

// mdbl-2008-s-1: 2 * (x, y) for an affine finite point.
__device__ __forceinline__ Xyzz xyzz_dbl_affine(const Affine& a) {
  Fq u = fe_dbl(a.y);
  Fq v = csqr(u);
  Fq w = cmul(u, v);
  Fq s = cmul(a.x, v);
  Fq x2 = csqr(a.x);
  Fq m = fe_add(fe_dbl(x2), x2);
  Xyzz r;
  r.x = fe_sub(fe_sub(csqr(m), s), s);
  r.y = fe_sub(cmul(m, fe_sub(s, r.x)), cmul(w, a.y));
  r.zz = v;
  r.zzz = w;
  return r;
}

// dbl-2008-s-1.
__device__ __forceinline__ Xyzz xyzz_dbl(const Xyzz& p) {
  if (xyzz_is_inf(p)) return p;
  Fq u = fe_dbl(p.y);
  Fq v = csqr(u);
  Fq w = cmul(u, v);
  Fq s = cmul(p.x, v);
  Fq x2 = csqr(p.x);
  Fq m = fe_add(fe_dbl(x2), x2);
  Xyzz r;
  r.x = fe_sub(fe_sub(csqr(m), s), s);
  r.y = fe_sub(cmul(m, fe_sub(s, r.x)), cmul(w, p.y));
  r.zz = cmul(v, p.zz);
  r.zzz = cmul(w, p.zzz);
  return r;
}

// madd-2008-s: acc + (x2, y2), the affine point assumed finite. The 8M + 2S
// go as four product pairs and one square pair.
__device__ __forceinline__ Xyzz xyzz_add_affine(const Xyzz& p, const Affine& a) {
  if (xyzz_is_inf(p)) return xyzz_from_affine(a);
  const Fq2 us = cmul2(a.x, p.zz, a.y, p.zzz);  // U2, S2
  const Fq pp_ = fe_sub(us.a, p.x);
  const Fq r = fe_sub(us.b, p.y);
  if (fe_is_zero(pp_)) {
    if (fe_is_zero(r)) return xyzz_dbl_affine(a);
    return xyzz_inf();
  }
  const Fq2 sq = csqr2(pp_, r);                    // PP, R^2
  const Fq2 pq = cmul2(pp_, sq.a, p.x, sq.a);      // PPP, Q
  const Fq2 zz = cmul2(p.zz, sq.a, p.zzz, pq.a);  // ZZ3, ZZZ3
  Xyzz o;
  o.x = fe_sub(fe_sub(fe_sub(sq.b, pq.a), pq.b), pq.b);
  const Fq2 yy = cmul2(r, fe_sub(pq.b, o.x), p.y, pq.a);
  o.y = fe_sub(yy.a, yy.b);
  o.zz = zz.a;
  o.zzz = zz.b;
  return o;
}

// add-2008-s (12M + 2S as six product pairs and one square pair).
__device__ __forceinline__ Xyzz xyzz_add(const Xyzz& p, const Xyzz& q) {
  if (xyzz_is_inf(p)) return q;
  if (xyzz_is_inf(q)) return p;
  const Fq2 u = cmul2(p.x, q.zz, q.x, p.zz);    // U1, U2
  const Fq2 s = cmul2(p.y, q.zzz, q.y, p.zzz);  // S1, S2
  const Fq pp_ = fe_sub(u.b, u.a);
  const Fq r = fe_sub(s.b, s.a);
  if (fe_is_zero(pp_)) {
    if (fe_is_zero(r)) return xyzz_dbl(p);
    return xyzz_inf();
  }
  const Fq2 sq = csqr2(pp_, r);                        // PP, R^2
  const Fq2 pq = cmul2(pp_, sq.a, u.a, sq.a);          // PPP, Q
  const Fq2 zp = cmul2(p.zz, q.zz, p.zzz, q.zzz);      // ZZ1 ZZ2, ZZZ1 ZZZ2
  const Fq2 zz = cmul2(zp.a, sq.a, zp.b, pq.a);        // ZZ3, ZZZ3
  Xyzz o;
  o.x = fe_sub(fe_sub(fe_sub(sq.b, pq.a), pq.b), pq.b);
  const Fq2 yy = cmul2(r, fe_sub(pq.b, o.x), s.a, pq.a);
  o.y = fe_sub(yy.a, yy.b);
  o.zz = zz.a;
  o.zzz = zz.b;
  return o;
}

__device__ __forceinline__ Xyzz xyzz_neg(const Xyzz& p) {
  Xyzz r = p;
  r.y = fe_neg(p.y);
  return r;
}

// XYZZ -> affine (Montgomery); infinity -> (0, 0). One inversion.
__device__ __forceinline__ Affine xyzz_to_affine(const Xyzz& p, uint32_t* flags = nullptr) {
  Affine a;
  if (xyzz_is_inf(p)) {
    a.x = fe_zero<FqConsts>();
    a.y = fe_zero<FqConsts>();
    return a;
  }
  Fq t = fe_inverse(cmul(p.zz, p.zzz), flags);
  a.x = cmul(p.x, cmul(t, p.zzz));
  a.y = cmul(p.y, cmul(t, p.zz));
  return a;
}

__device__ __forceinline__ Affine ld_affine(const Affine* p) {
  Affine a;
  a.x = ld_fe(&p->x);
  a.y = ld_fe(&p->y);
  return a;
}

__device__ __forceinline__ Xyzz ld_xyzz(const Xyzz* p) {
  Xyzz a;
  a.x = ld_fe(&p->x);
  a.y = ld_fe(&p->y);
  a.zz = ld_fe(&p->zz);
  a.zzz = ld_fe(&p->zzz);
  return a;
}

__device__ __forceinline__ void st_xyzz(Xyzz* p, const Xyzz& a) {
  st_fe(&p->x, a.x);
  st_fe(&p->y, a.y);
  st_fe(&p->zz, a.zz);
  st_fe(&p->zzz, a.zzz);
}

}  // namespace apg
