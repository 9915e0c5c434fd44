// ORACLE — test infrastructure only. A CPU restatement of the reference's
// BN254 field arithmetic, used by tests/ and bench.py's CPU baseline to check
// and time the CUDA library. Nothing in the product links this file.
//
// Restates crates/field/src/lib.rs (Fr, 4x64 Montgomery CIOS, :44-184) and
// crates/curve/src/fq.rs (Fq, the same kernel with FQ_* constants, :1-446),
// with the moduli and Montgomery constants of crates/constants/src/lib.rs:22-143.
#pragma once
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace oracle {

typedef unsigned __int128 u128;

struct FrParams {
  static constexpr uint64_t MOD[4] = {0x43e1f593f0000001ULL, 0x2833e84879b97091ULL,
                                      0xb85045b68181585dULL, 0x30644e72e131a029ULL};
  static constexpr uint64_t R[4] = {0xac96341c4ffffffbULL, 0x36fc76959f60cd29ULL,
                                    0x666ea36f7879462eULL, 0x0e0a77c19a07df2fULL};
  static constexpr uint64_t R2[4] = {0x1bb8e645ae216da7ULL, 0x53fe3ab1e35c59e3ULL,
                                     0x8c49833d53bb8085ULL, 0x0216d0b17f4e44a5ULL};
  static constexpr uint64_t INV = 0xc2e1f593efffffffULL;
};

struct FqParams {
  static constexpr uint64_t MOD[4] = {0x3c208c16d87cfd47ULL, 0x97816a916871ca8dULL,
                                      0xb85045b68181585dULL, 0x30644e72e131a029ULL};
  static constexpr uint64_t R[4] = {0xd35d438dc58f0d9dULL, 0x0a78eb28f5c70b3dULL,
                                    0x666ea36f7879462cULL, 0x0e0a77c19a07df2fULL};
  static constexpr uint64_t R2[4] = {0xf32cfc5b538afa89ULL, 0xb5e71911d44501fbULL,
                                     0x47ab1eff0a417ff6ULL, 0x06d89f71cab8351fULL};
  static constexpr uint64_t INV = 0x87d20782e4866389ULL;
};

// An element in Montgomery form x*R mod m, fully reduced, little-endian limbs.
template <class P>
struct Fp {
  uint64_t l[4];

  static Fp zero() { return Fp{{0, 0, 0, 0}}; }
  static Fp one() { return Fp{{P::R[0], P::R[1], P::R[2], P::R[3]}}; }

  static bool ge_mod(const uint64_t a[4]) {
    for (int i = 3; i >= 0; --i) {
      if (a[i] != P::MOD[i]) return a[i] > P::MOD[i];
    }
    return true;
  }
  static void sub_mod_once(uint64_t a[4]) {
    if (ge_mod(a)) {
      uint64_t borrow = 0;
      for (int i = 0; i < 4; ++i) {
        u128 t = (u128)a[i] - P::MOD[i] - borrow;
        a[i] = (uint64_t)t;
        borrow = (uint64_t)(t >> 64) & 1;
      }
    }
  }
  // CIOS over four 64-bit limbs: crates/field/src/lib.rs:148-184.
  static Fp mont(const uint64_t a[4], const uint64_t b[4]) {
    uint64_t t[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 4; ++i) {
      uint64_t carry = 0;
      for (int j = 0; j < 4; ++j) {
        u128 s = (u128)t[j] + (u128)a[j] * b[i] + carry;
        t[j] = (uint64_t)s;
        carry = (uint64_t)(s >> 64);
      }
      u128 s4 = (u128)t[4] + carry;
      t[4] = (uint64_t)s4;
      t[5] = (uint64_t)(s4 >> 64);
      uint64_t m = t[0] * P::INV;
      u128 s0 = (u128)t[0] + (u128)m * P::MOD[0];
      carry = (uint64_t)(s0 >> 64);
      for (int j = 1; j < 4; ++j) {
        u128 s = (u128)t[j] + (u128)m * P::MOD[j] + carry;
        t[j - 1] = (uint64_t)s;
        carry = (uint64_t)(s >> 64);
      }
      u128 s3 = (u128)t[4] + carry;
      t[3] = (uint64_t)s3;
      t[4] = t[5] + (uint64_t)(s3 >> 64);
    }
    Fp r{{t[0], t[1], t[2], t[3]}};
    sub_mod_once(r.l);
    return r;
  }

  Fp operator+(const Fp& b) const {
    Fp r;
    uint64_t c = 0;
    for (int i = 0; i < 4; ++i) {
      u128 s = (u128)l[i] + b.l[i] + c;
      r.l[i] = (uint64_t)s;
      c = (uint64_t)(s >> 64);
    }
    sub_mod_once(r.l);
    return r;
  }
  Fp operator-(const Fp& b) const {
    Fp r;
    uint64_t br = 0;
    for (int i = 0; i < 4; ++i) {
      u128 t = (u128)l[i] - b.l[i] - br;
      r.l[i] = (uint64_t)t;
      br = (uint64_t)(t >> 64) & 1;
    }
    if (br) {
      uint64_t c = 0;
      for (int i = 0; i < 4; ++i) {
        u128 s = (u128)r.l[i] + P::MOD[i] + c;
        r.l[i] = (uint64_t)s;
        c = (uint64_t)(s >> 64);
      }
    }
    return r;
  }
  Fp operator-() const { return is_zero() ? *this : zero() - *this; }
  Fp operator*(const Fp& b) const { return mont(l, b.l); }
  Fp& operator+=(const Fp& b) { return *this = *this + b; }
  Fp& operator-=(const Fp& b) { return *this = *this - b; }
  Fp& operator*=(const Fp& b) { return *this = *this * b; }
  bool operator==(const Fp& b) const { return memcmp(l, b.l, 32) == 0; }
  bool operator!=(const Fp& b) const { return !(*this == b); }
  bool is_zero() const { return (l[0] | l[1] | l[2] | l[3]) == 0; }
  Fp square() const { return *this * *this; }
  Fp dbl() const { return *this + *this; }

  static Fp from_u64(uint64_t x) {
    uint64_t a[4] = {x, 0, 0, 0};
    return mont(a, P::R2);
  }
  // Square-and-multiply over a 256-bit exponent, top bit first (lib.rs:204-215).
  Fp pow(const uint64_t e[4]) const {
    Fp acc = one();
    for (int i = 3; i >= 0; --i)
      for (int b = 63; b >= 0; --b) {
        acc = acc.square();
        if ((e[i] >> b) & 1) acc = acc * *this;
      }
    return acc;
  }
  // Fermat: self^(m-2); zero maps to zero (callers test for it).
  Fp inverse() const {
    uint64_t e[4] = {P::MOD[0] - 2, P::MOD[1], P::MOD[2], P::MOD[3]};
    return pow(e);
  }
  // Canonical 32-byte little-endian decoding; false if >= m.
  static bool from_bytes(const uint8_t b[32], Fp& out) {
    uint64_t a[4];
    memcpy(a, b, 32);
    if (ge_mod(a)) return false;
    out = mont(a, P::R2);
    return true;
  }
  void to_bytes(uint8_t b[32]) const {
    uint64_t one_[4] = {1, 0, 0, 0};
    Fp c = mont(l, one_);
    memcpy(b, c.l, 32);
  }
  // In-memory (Montgomery) limbs as bytes: crates/field/src/lib.rs:321.
  static bool from_memory_bytes(const uint8_t b[32], Fp& out) {
    memcpy(out.l, b, 32);
    return !ge_mod(out.l);
  }
  void to_memory_bytes(uint8_t b[32]) const { memcpy(b, l, 32); }
};

typedef Fp<FrParams> Fr;
typedef Fp<FqParams> Fq;

// Montgomery batch inversion, zeros skipped (crates/field/src/lib.rs:357-383).
template <class F>
void batch_inverse(std::vector<F>& xs) {
  std::vector<F> prefix(xs.size());
  F running = F::one();
  for (size_t i = 0; i < xs.size(); ++i) {
    prefix[i] = running;
    if (!xs[i].is_zero()) running = running * xs[i];
  }
  F inv = running.inverse();
  for (size_t i = xs.size(); i-- > 0;) {
    if (xs[i].is_zero()) continue;
    F next = inv * xs[i];
    xs[i] = inv * prefix[i];
    inv = next;
  }
}

template <class F>
void from_bytes_or_die(const uint8_t b[32], F& out) {
  if (!F::from_bytes(b, out)) throw std::string("non-canonical field element");
}

// Big-endian "0x" + 64 hex digits, as the reference's constant tables are
// written (crates/field/src/lib.rs:232-249).
template <class F>
F from_hex_be(const char* s) {
  uint8_t le[32];
  const char* d = s + 2;
  for (int i = 0; i < 32; ++i) {
    auto hv = [](char c) { return c <= '9' ? c - '0' : c - 'a' + 10; };
    le[31 - i] = (uint8_t)((hv(d[2 * i]) << 4) | hv(d[2 * i + 1]));
  }
  F out;
  from_bytes_or_die(le, out);
  return out;
}

}  // namespace oracle
