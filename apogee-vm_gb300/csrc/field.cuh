// BN254 Fr / Fq arithmetic for sm_103a: 8 x 32-bit little-endian limbs in
// Montgomery form with R = 2^256, byte-identical to the reference's in-memory
// 4 x 64-bit representation (crates/field/src/lib.rs:30-36, 321), so a
// caller's `&[Fr]` crosses the C ABI with no conversion.
//
// The multiply is CIOS on the integer multiply pipe: per limb of b, one row of
// 32x32->64 products (mul.wide) accumulates a*b_i and one accumulates m*p,
// 136 wide products a multiply, then one conditional subtraction. With
// a, b < m < 2^254 the accumulator stays below 2m < 2^255 between limbs and
// below 2^288 inside one, so nine 32-bit words always hold it. (Measured on
// GB300: 47 G products/s against 38 G/s for the same CIOS written as
// mad.lo/mad.hi carry chains, which issue two multiplies per partial product.)
#pragma once
#include <cstdint>

namespace apg {

struct FrConsts {
  static constexpr uint32_t P0 = 0xf0000001u, P1 = 0x43e1f593u, P2 = 0x79b97091u, P3 = 0x2833e848u,
                            P4 = 0x8181585du, P5 = 0xb85045b6u, P6 = 0xe131a029u, P7 = 0x30644e72u;
  static constexpr uint32_t INV = 0xefffffffu;  // -p^-1 mod 2^32
  __host__ __device__ static constexpr uint32_t R(int i) {
    return (const uint32_t[8]){0x4ffffffbu, 0xac96341cu, 0x9f60cd29u, 0x36fc7695u,
                               0x7879462eu, 0x666ea36fu, 0x9a07df2fu, 0x0e0a77c1u}[i];
  }
  __host__ __device__ static constexpr uint32_t R2(int i) {
    return (const uint32_t[8]){0xae216da7u, 0x1bb8e645u, 0xe35c59e3u, 0x53fe3ab1u,
                               0x53bb8085u, 0x8c49833du, 0x7f4e44a5u, 0x0216d0b1u}[i];
  }
};

struct FqConsts {
  static constexpr uint32_t P0 = 0xd87cfd47u, P1 = 0x3c208c16u, P2 = 0x6871ca8du, P3 = 0x97816a91u,
                            P4 = 0x8181585du, P5 = 0xb85045b6u, P6 = 0xe131a029u, P7 = 0x30644e72u;
  static constexpr uint32_t INV = 0xe4866389u;  // -q^-1 mod 2^32
  __host__ __device__ static constexpr uint32_t R(int i) {
    return (const uint32_t[8]){0xc58f0d9du, 0xd35d438du, 0xf5c70b3du, 0x0a78eb28u,
                               0x7879462cu, 0x666ea36fu, 0x9a07df2fu, 0x0e0a77c1u}[i];
  }
  __host__ __device__ static constexpr uint32_t R2(int i) {
    return (const uint32_t[8]){0x538afa89u, 0xf32cfc5bu, 0xd44501fbu, 0xb5e71911u,
                               0x0a417ff6u, 0x47ab1effu, 0xcab8351fu, 0x06d89f71u}[i];
  }
};

template <class C>
struct Fe {
  uint32_t v[8];
};

typedef Fe<FrConsts> Fr;
typedef Fe<FqConsts> Fq;

template <class C>
__host__ __device__ __forceinline__ Fe<C> fe_zero() {
  Fe<C> r;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.v[i] = 0;
  return r;
}

template <class C>
__host__ __device__ __forceinline__ Fe<C> fe_one() {
  Fe<C> r;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.v[i] = C::R(i);
  return r;
}

template <class C>
__device__ __forceinline__ bool fe_is_zero(const Fe<C>& a) {
  return (a.v[0] | a.v[1] | a.v[2] | a.v[3] | a.v[4] | a.v[5] | a.v[6] | a.v[7]) == 0;
}

template <class C>
__device__ __forceinline__ bool fe_eq(const Fe<C>& a, const Fe<C>& b) {
  uint32_t d = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) d |= a.v[i] ^ b.v[i];
  return d == 0;
}

// r = a - m if a >= m (a < 2m): subtract, keep the difference unless it borrowed.
template <class C>
__device__ __forceinline__ void fe_reduce_once(uint32_t r[8]) {
  uint32_t s0, s1, s2, s3, s4, s5, s6, s7, br;
  asm("sub.cc.u32  %0, %9, %17;\n\t"
      "subc.cc.u32 %1, %10, %18;\n\t"
      "subc.cc.u32 %2, %11, %19;\n\t"
      "subc.cc.u32 %3, %12, %20;\n\t"
      "subc.cc.u32 %4, %13, %21;\n\t"
      "subc.cc.u32 %5, %14, %22;\n\t"
      "subc.cc.u32 %6, %15, %23;\n\t"
      "subc.cc.u32 %7, %16, %24;\n\t"
      "subc.u32    %8, 0, 0;"
      : "=r"(s0), "=r"(s1), "=r"(s2), "=r"(s3), "=r"(s4), "=r"(s5), "=r"(s6), "=r"(s7), "=r"(br)
      : "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
        "n"(C::P0), "n"(C::P1), "n"(C::P2), "n"(C::P3), "n"(C::P4), "n"(C::P5), "n"(C::P6), "n"(C::P7));
  const bool keep = br != 0;
  r[0] = keep ? r[0] : s0;
  r[1] = keep ? r[1] : s1;
  r[2] = keep ? r[2] : s2;
  r[3] = keep ? r[3] : s3;
  r[4] = keep ? r[4] : s4;
  r[5] = keep ? r[5] : s5;
  r[6] = keep ? r[6] : s6;
  r[7] = keep ? r[7] : s7;
}

template <class C>
__device__ __forceinline__ Fe<C> fe_add(const Fe<C>& a, const Fe<C>& b) {
  Fe<C> r;
  asm("add.cc.u32  %0, %8, %16;\n\t"
      "addc.cc.u32 %1, %9, %17;\n\t"
      "addc.cc.u32 %2, %10, %18;\n\t"
      "addc.cc.u32 %3, %11, %19;\n\t"
      "addc.cc.u32 %4, %12, %20;\n\t"
      "addc.cc.u32 %5, %13, %21;\n\t"
      "addc.cc.u32 %6, %14, %22;\n\t"
      "addc.u32    %7, %15, %23;"
      : "=r"(r.v[0]), "=r"(r.v[1]), "=r"(r.v[2]), "=r"(r.v[3]), "=r"(r.v[4]), "=r"(r.v[5]), "=r"(r.v[6]),
        "=r"(r.v[7])
      : "r"(a.v[0]), "r"(a.v[1]), "r"(a.v[2]), "r"(a.v[3]), "r"(a.v[4]), "r"(a.v[5]), "r"(a.v[6]), "r"(a.v[7]),
        "r"(b.v[0]), "r"(b.v[1]), "r"(b.v[2]), "r"(b.v[3]), "r"(b.v[4]), "r"(b.v[5]), "r"(b.v[6]), "r"(b.v[7]));
  fe_reduce_once<C>(r.v);
  return r;
}

template <class C>
__device__ __forceinline__ Fe<C> fe_sub(const Fe<C>& a, const Fe<C>& b) {
  Fe<C> r;
  uint32_t br;
  asm("sub.cc.u32  %0, %9, %17;\n\t"
      "subc.cc.u32 %1, %10, %18;\n\t"
      "subc.cc.u32 %2, %11, %19;\n\t"
      "subc.cc.u32 %3, %12, %20;\n\t"
      "subc.cc.u32 %4, %13, %21;\n\t"
      "subc.cc.u32 %5, %14, %22;\n\t"
      "subc.cc.u32 %6, %15, %23;\n\t"
      "subc.cc.u32 %7, %16, %24;\n\t"
      "subc.u32    %8, 0, 0;"
      : "=r"(r.v[0]), "=r"(r.v[1]), "=r"(r.v[2]), "=r"(r.v[3]), "=r"(r.v[4]), "=r"(r.v[5]), "=r"(r.v[6]),
        "=r"(r.v[7]), "=r"(br)
      : "r"(a.v[0]), "r"(a.v[1]), "r"(a.v[2]), "r"(a.v[3]), "r"(a.v[4]), "r"(a.v[5]), "r"(a.v[6]), "r"(a.v[7]),
        "r"(b.v[0]), "r"(b.v[1]), "r"(b.v[2]), "r"(b.v[3]), "r"(b.v[4]), "r"(b.v[5]), "r"(b.v[6]), "r"(b.v[7]));
  // On borrow add the modulus back (masked add: br is 0 or all ones).
  asm("add.cc.u32  %0, %0, %8;\n\t"
      "addc.cc.u32 %1, %1, %9;\n\t"
      "addc.cc.u32 %2, %2, %10;\n\t"
      "addc.cc.u32 %3, %3, %11;\n\t"
      "addc.cc.u32 %4, %4, %12;\n\t"
      "addc.cc.u32 %5, %5, %13;\n\t"
      "addc.cc.u32 %6, %6, %14;\n\t"
      "addc.u32    %7, %7, %15;"
      : "+r"(r.v[0]), "+r"(r.v[1]), "+r"(r.v[2]), "+r"(r.v[3]), "+r"(r.v[4]), "+r"(r.v[5]), "+r"(r.v[6]),
        "+r"(r.v[7])
      : "r"(br & C::P0), "r"(br & C::P1), "r"(br & C::P2), "r"(br & C::P3), "r"(br & C::P4), "r"(br & C::P5),
        "r"(br & C::P6), "r"(br & C::P7));
  return r;
}

template <class C>
__device__ __forceinline__ Fe<C> fe_neg(const Fe<C>& a) {
  return fe_is_zero(a) ? a : fe_sub(fe_zero<C>(), a);
}

template <class C>
__device__ __forceinline__ Fe<C> fe_dbl(const Fe<C>& a) {
  return fe_add(a, a);
}

// One CIOS row per limb of b with 32x32->64 products (mul.wide): t += a*b_i,
// m = t0 * inv, t = (t + m*p) >> 32. Each 64-bit step adds one product, one
// word of t and the previous carry, which cannot overflow:
// (2^32-1)^2 + 2(2^32-1) = 2^64 - 1.
template <class C>
__device__ __forceinline__ Fe<C> fe_mul(const Fe<C>& a, const Fe<C>& b) {
  const uint32_t p[8] = {C::P0, C::P1, C::P2, C::P3, C::P4, C::P5, C::P6, C::P7};
  uint32_t t[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) t[k] = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    uint64_t c = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint64_t uv = (uint64_t)a.v[j] * b.v[i] + t[j] + c;
      t[j] = (uint32_t)uv;
      c = uv >> 32;
    }
    t[8] += (uint32_t)c;  // t < 2^287 here: no carry out of word 8
    const uint32_t m = t[0] * C::INV;
    uint64_t uv = (uint64_t)m * p[0] + t[0];  // low word cancels
    c = uv >> 32;
#pragma unroll
    for (int j = 1; j < 8; ++j) {
      uv = (uint64_t)m * p[j] + t[j] + c;
      t[j - 1] = (uint32_t)uv;
      c = uv >> 32;
    }
    uv = (uint64_t)t[8] + c;  // t < 2^288 before the shift, < 2^256 after
    t[7] = (uint32_t)uv;
    t[8] = 0;
  }
  Fe<C> r;
#pragma unroll
  for (int k = 0; k < 8; ++k) r.v[k] = t[k];
  fe_reduce_once<C>(r.v);
  return r;
}

// a^2 with the cross products computed once: rows of a_i * a_j (i < j) with
// 64-bit carries into a 512-bit T, T doubled, the squares a_i^2 added, then
// the eight Montgomery reduction rows. 36 wide products for the square
// against 64 in a multiply (measured on GB300: 61 G squares/s against 49 G
// products/s). T < a^2 < 2^508, so the doubling and the additions never
// carry out of 16 words, and the reduced value is below 2m.
template <class C>
__device__ __forceinline__ Fe<C> fe_sqr(const Fe<C>& a) {
  const uint32_t p[8] = {C::P0, C::P1, C::P2, C::P3, C::P4, C::P5, C::P6, C::P7};
  uint32_t T[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) T[k] = 0;
#pragma unroll
  for (int i = 0; i < 7; ++i) {
    uint64_t c = 0;
#pragma unroll
    for (int j = i + 1; j < 8; ++j) {
      const uint64_t uv = (uint64_t)a.v[i] * a.v[j] + T[i + j] + c;
      T[i + j] = (uint32_t)uv;
      c = uv >> 32;
    }
    T[i + 8] = (uint32_t)c;
  }
  T[15] = T[14] >> 31;
#pragma unroll
  for (int k = 14; k > 0; --k) T[k] = (T[k] << 1) | (T[k - 1] >> 31);
  T[0] <<= 1;
  uint64_t c = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const uint64_t sq = (uint64_t)a.v[i] * a.v[i];
    const uint64_t lo = (uint64_t)T[2 * i] + (uint32_t)sq + c;
    T[2 * i] = (uint32_t)lo;
    const uint64_t hi = (uint64_t)T[2 * i + 1] + (uint32_t)(sq >> 32) + (lo >> 32);
    T[2 * i + 1] = (uint32_t)hi;
    c = hi >> 32;
  }
  uint32_t carry_hi = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const uint32_t m = T[i] * C::INV;
    uint64_t cc = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint64_t uv = (uint64_t)m * p[j] + T[i + j] + cc;
      T[i + j] = (uint32_t)uv;
      cc = uv >> 32;
    }
    const uint64_t s = (uint64_t)T[i + 8] + cc + carry_hi;
    T[i + 8] = (uint32_t)s;
    carry_hi = (uint32_t)(s >> 32);
  }
  Fe<C> r;
#pragma unroll
  for (int k = 0; k < 8; ++k) r.v[k] = T[8 + k];
  fe_reduce_once<C>(r.v);
  return r;
}

// Montgomery form -> canonical limbs (multiply by 1), and back (multiply by R^2).
template <class C>
__device__ __forceinline__ Fe<C> fe_from_mont(const Fe<C>& a) {
  // a * R^-1: the reduction rows of the multiply alone (a * 1 has no product
  // rows), eight m*p rows of 64-bit steps.
  const uint32_t p[8] = {C::P0, C::P1, C::P2, C::P3, C::P4, C::P5, C::P6, C::P7};
  uint32_t t[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) t[k] = a.v[k];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const uint32_t m = t[0] * C::INV;
    uint64_t uv = (uint64_t)m * p[0] + t[0];
    uint64_t c = uv >> 32;
#pragma unroll
    for (int j = 1; j < 8; ++j) {
      uv = (uint64_t)m * p[j] + t[j] + c;
      t[j - 1] = (uint32_t)uv;
      c = uv >> 32;
    }
    t[7] = (uint32_t)c;  // (t + m*p) / 2^32 < 2^256
  }
  Fe<C> r;
#pragma unroll
  for (int k = 0; k < 8; ++k) r.v[k] = t[k];
  fe_reduce_once<C>(r.v);
  return r;
}

template <class C>
__device__ __forceinline__ Fe<C> fe_to_mont(const Fe<C>& a) {
  Fe<C> r2;
#pragma unroll
  for (int i = 0; i < 8; ++i) r2.v[i] = C::R2(i);
  return fe_mul(a, r2);
}

template <class C>
__device__ __forceinline__ Fe<C> fe_from_u64(uint64_t x) {
  Fe<C> a = fe_zero<C>();
  a.v[0] = (uint32_t)x;
  a.v[1] = (uint32_t)(x >> 32);
  return fe_to_mont(a);
}

// Canonical value < m? (used to validate inputs arriving in canonical form)
template <class C>
__device__ __forceinline__ bool fe_lt_mod(const uint32_t a[8]) {
  const uint32_t p[8] = {C::P0, C::P1, C::P2, C::P3, C::P4, C::P5, C::P6, C::P7};
#pragma unroll
  for (int i = 7; i >= 0; --i) {
    if (a[i] != p[i]) return a[i] < p[i];
  }
  return false;
}

// 1/a by Bernstein and Yang's divsteps ("Fast constant-time gcd computation
// and modular inversion", 2019), in the half-delta form, on the Montgomery
// value A = aR. State: eta = 2 delta (starts at 1), f = m (odd), g = A, and
// d, e with f = d A and g = e A (mod m), starting at d = 0, e = 1. One divstep:
// if delta > 0 and g is odd, (delta, f, g) <- (1 - delta, g, (g - f) / 2);
// otherwise (1 + delta, f, (g + (g mod 2) f) / 2). g reaches 0 with f = +-1,
// and then 1/A = +-d. Thirty divsteps depend only on the low 32 bits of f and
// g, so they run on those bits alone and yield an integer matrix T with
// 2^30 (f', g') = T (f, g) (entries at most 2^30); T is then applied once to
// the full f, g and (mod m) to d, e. Big values are nine signed 30-bit limbs
// (value = sum l_i 2^(30 i), limbs 0..7 in [0, 2^30), limb 8 signed), so a
// limb of T (f, g) is one 64-bit sum of 32x32 products. For d, e the multiple
// k m that clears the low 30 bits (k = -(T (d, e))_0 m^-1 mod 2^30, taken in
// [-2^29, 2^29)) is added before the division: each batch grows |d|, |e| by
// less than m / 2, so they stay below 2^269 for the batches a 254-bit modulus
// needs (the half-delta form needs at most 590 divsteps for 256-bit inputs:
// 20 batches; measured at most 18 over 400,000 random inputs of both fields),
// and one reduction at the end brings d into [0, m). Variable time (the
// inputs are public values). Written as __host__ __device__ plain C++ so the
// same code is checked on the host.
struct Signed30 {
  int32_t l[9];
};

__host__ __device__ __forceinline__ Signed30 s30_from_words(const uint32_t w[8]) {
  Signed30 s;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const int bit = 30 * i, wi = bit >> 5, sh = bit & 31;
    uint64_t v = wi < 8 ? (uint64_t)(w[wi] >> sh) : 0;
    if (wi + 1 < 8 && sh) v |= (uint64_t)w[wi + 1] << (32 - sh);
    s.l[i] = (int32_t)(v & 0x3fffffffu);
  }
  return s;
}

// (f, g) <- (u f + v g, q f + r g) / 2^30 (exact: the low 30 bits cancel).
__host__ __device__ __forceinline__ void s30_update_fg(Signed30& f, Signed30& g, int32_t u, int32_t v, int32_t q,
                                                       int32_t r) {
  int64_t cf = ((int64_t)u * f.l[0] + (int64_t)v * g.l[0]) >> 30;
  int64_t cg = ((int64_t)q * f.l[0] + (int64_t)r * g.l[0]) >> 30;
#pragma unroll
  for (int i = 1; i < 9; ++i) {
    cf += (int64_t)u * f.l[i] + (int64_t)v * g.l[i];
    cg += (int64_t)q * f.l[i] + (int64_t)r * g.l[i];
    f.l[i - 1] = (int32_t)(cf & 0x3fffffff);
    g.l[i - 1] = (int32_t)(cg & 0x3fffffff);
    cf >>= 30;
    cg >>= 30;
  }
  f.l[8] = (int32_t)cf;
  g.l[8] = (int32_t)cg;
}

// (d, e) <- (u d + v e + k_d m, q d + r e + k_e m) / 2^30, each k chosen to
// clear the low 30 bits, so the results are d / 2^30-style values mod m.
__host__ __device__ __forceinline__ void s30_update_de(Signed30& d, Signed30& e, int32_t u, int32_t v, int32_t q,
                                                       int32_t r, const Signed30& m, uint32_t minv30) {
  const int64_t d0 = (int64_t)u * d.l[0] + (int64_t)v * e.l[0];
  const int64_t e0 = (int64_t)q * d.l[0] + (int64_t)r * e.l[0];
  int32_t kd = (int32_t)(((uint32_t)(0u - (uint32_t)d0) * minv30) & 0x3fffffffu);
  int32_t ke = (int32_t)(((uint32_t)(0u - (uint32_t)e0) * minv30) & 0x3fffffffu);
  kd -= (kd >> 29) << 30;  // into [-2^29, 2^29)
  ke -= (ke >> 29) << 30;
  int64_t cd = (d0 + (int64_t)kd * m.l[0]) >> 30;
  int64_t ce = (e0 + (int64_t)ke * m.l[0]) >> 30;
#pragma unroll
  for (int i = 1; i < 9; ++i) {
    cd += (int64_t)u * d.l[i] + (int64_t)v * e.l[i] + (int64_t)kd * m.l[i];
    ce += (int64_t)q * d.l[i] + (int64_t)r * e.l[i] + (int64_t)ke * m.l[i];
    d.l[i - 1] = (int32_t)(cd & 0x3fffffff);
    e.l[i - 1] = (int32_t)(ce & 0x3fffffff);
    cd >>= 30;
    ce >>= 30;
  }
  d.l[8] = (int32_t)cd;
  e.l[8] = (int32_t)ce;
}

// Nine-limb signed value -> nine 32-bit words, two's complement.
__host__ __device__ __forceinline__ void s30_to_words(const Signed30& s, uint32_t w[9]) {
  uint64_t acc = 0;
  int nb = 0, j = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    acc |= (uint64_t)(uint32_t)s.l[i] << nb;
    nb += 30;
    if (nb >= 32) {
      w[j++] = (uint32_t)acc;
      acc >>= 32;
      nb -= 32;
    }
  }
  const int64_t top = (int64_t)s.l[8] * ((int64_t)1 << nb) + (int64_t)acc;  // nb = 16 here
  w[7] = (uint32_t)top;
  w[8] = (uint32_t)(top >> 32);
}

// w += a on nine words.
__host__ __device__ __forceinline__ void words9_add(uint32_t w[9], const uint32_t a[9]) {
  uint64_t c = 0;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    c += (uint64_t)w[i] + a[i];
    w[i] = (uint32_t)c;
    c >>= 32;
  }
}

// w -= a when w >= a (both nonnegative nine-word values).
__host__ __device__ __forceinline__ void words9_csub(uint32_t w[9], const uint32_t a[9]) {
  uint32_t t[9];
  int64_t b = 0;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    b += (int64_t)w[i] - a[i];
    t[i] = (uint32_t)b;
    b >>= 32;
  }
  if (b == 0) {
#pragma unroll
    for (int i = 0; i < 9; ++i) w[i] = t[i];
  }
}

// x = A^-1 mod m for 0 < A < m (m odd, below 2^254); false if g did not reach
// 0 within the batch guard (unreachable for such inputs).
__host__ __device__ inline bool inverse_divsteps(const uint32_t A[8], const uint32_t mw[8], uint32_t x[8]) {
  uint32_t minv30 = 1;  // m^-1 mod 2^32 by Newton's iteration (each step doubles the correct bits)
#pragma unroll
  for (int i = 0; i < 5; ++i) minv30 *= 2u - mw[0] * minv30;
  minv30 &= 0x3fffffffu;
  const Signed30 m = s30_from_words(mw);
  Signed30 f = m, g = s30_from_words(A), d, e;
#pragma unroll
  for (int i = 0; i < 9; ++i) d.l[i] = e.l[i] = 0;
  e.l[0] = 1;
  int32_t eta = 1;
  bool done = false;
  for (int batch = 0; batch < 24; ++batch) {
    int32_t any = 0;
#pragma unroll
    for (int i = 0; i < 9; ++i) any |= g.l[i];
    if (!any) {
      done = true;
      break;
    }
    uint32_t fl = (uint32_t)f.l[0] | ((uint32_t)f.l[1] << 30), gl = (uint32_t)g.l[0] | ((uint32_t)g.l[1] << 30);
    int32_t u = 1, v = 0, q = 0, r = 1;
#pragma unroll 6
    for (int i = 0; i < 30; ++i) {
      // delta > 0 and g odd: (f, g) <- (g, -f), the rows swap and negate,
      // eta <- -eta; then the g-odd step adds f to g.
      const uint32_t odd = 0u - (gl & 1u);
      const uint32_t sw = odd & (0u - ((uint32_t)(-eta) >> 31));
      const uint32_t tf = (fl ^ gl) & sw;
      fl ^= tf;
      gl ^= tf;
      gl = (gl ^ sw) - sw;
      const int32_t ssw = (int32_t)sw;
      const int32_t tu = (u ^ q) & ssw, tv = (v ^ r) & ssw;
      u ^= tu;
      q ^= tu;
      v ^= tv;
      r ^= tv;
      q = (q ^ ssw) - ssw;
      r = (r ^ ssw) - ssw;
      eta = (eta ^ ssw) - ssw;
      gl += fl & odd;
      q += u & (int32_t)odd;
      r += v & (int32_t)odd;
      gl >>= 1;
      u *= 2;
      v *= 2;
      eta += 2;
    }
    s30_update_fg(f, g, u, v, q, r);
    s30_update_de(d, e, u, v, q, r, m, minv30);
  }
  // d in (-12 m, 12 m): lift by 16 m, reduce by 16 m, 8 m, 4 m, 2 m, m.
  uint32_t w[9], km[5][9];
  s30_to_words(d, w);
#pragma unroll
  for (int k = 0; k < 5; ++k) {  // km[k] = 2^(4-k) m
    const int sh = 4 - k;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      const uint32_t hi = i < 8 ? mw[i] : 0u, lo = i > 0 ? mw[i - 1] : 0u;
      km[k][i] = sh ? (hi << sh) | (lo >> (32 - sh)) : hi;
    }
  }
  words9_add(w, km[0]);
#pragma unroll
  for (int k = 0; k < 5; ++k) words9_csub(w, km[k]);
  // f = +-1: negate the result when f = -1 (its top limb is negative).
  const bool neg = f.l[8] < 0;
  uint32_t z = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) z |= w[i];
  if (neg && z) {
    int64_t b = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      b += (int64_t)mw[i] - w[i];
      w[i] = (uint32_t)b;
      b >>= 32;
    }
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = w[i];
  return done;
}

// Bit a kernel raises in its context's device flags when an inversion did not
// converge (the divsteps above end in fewer batches than their guard for
// every nonzero input below the modulus; the flag makes a broken invariant an
// error instead of a wrong value). The host reads it as DEV_INVERSE.
constexpr uint32_t kFlagInverse = 32u;

// 1/a for a in Montgomery form (0 for 0): the divsteps give A^-1 = a^-1 R^-1,
// and a^-1 R = A^-1 * R^3 (one Montgomery product with R^3 = R2 * R2 reduced
// once). `flags` (nullable) receives kFlagInverse if the batch guard ends it.
template <class C>
__device__ __noinline__ Fe<C> fe_inverse(const Fe<C>& a, uint32_t* flags = nullptr) {
  if (fe_is_zero(a)) return a;
  const uint32_t p[8] = {C::P0, C::P1, C::P2, C::P3, C::P4, C::P5, C::P6, C::P7};
  Fe<C> x;
  if (!inverse_divsteps(a.v, p, x.v) && flags) atomicOr(flags, kFlagInverse);
  Fe<C> r2;
#pragma unroll
  for (int i = 0; i < 8; ++i) r2.v[i] = C::R2(i);
  return fe_mul(x, fe_mul(r2, r2));
}

template <class C>
__device__ __forceinline__ Fe<C> ld_fe(const Fe<C>* p) {
  const uint4* q = reinterpret_cast<const uint4*>(p);
  uint4 x = q[0], y = q[1];
  Fe<C> r;
  r.v[0] = x.x; r.v[1] = x.y; r.v[2] = x.z; r.v[3] = x.w;
  r.v[4] = y.x; r.v[5] = y.y; r.v[6] = y.z; r.v[7] = y.w;
  return r;
}

template <class C>
__device__ __forceinline__ void st_fe(Fe<C>* p, const Fe<C>& a) {
  uint4* q = reinterpret_cast<uint4*>(p);
  q[0] = make_uint4(a.v[0], a.v[1], a.v[2], a.v[3]);
  q[1] = make_uint4(a.v[4], a.v[5], a.v[6], a.v[7]);
}

}  // namespace apg
