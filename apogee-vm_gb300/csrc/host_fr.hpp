// Host-side Fr arithmetic and the Poseidon2 duplex transcript for the
// library's sequential glue: Fiat-Shamir challenges, cubic interpolation and
// the O(b) polynomial work of a Mercury opening. The hot passes run on the
// device; these are the O(1)-per-round steps the reference also runs
// serially (crates/transcript/src/lib.rs:214-346,
// crates/sumcheck/src/lib.rs:294-305).
//
// Fr is kept in Montgomery form over four 64-bit limbs (R = 2^256), the same
// bytes the device and the reference hold.
#pragma once
#include <array>
#include <cstdint>
#include <cstring>
#include <vector>

namespace apg {
namespace host {

typedef unsigned __int128 u128;

static constexpr uint64_t kP[4] = {0x43e1f593f0000001ull, 0x2833e84879b97091ull, 0xb85045b68181585dull,
                                   0x30644e72e131a029ull};
static constexpr uint64_t kPInv = 0xc2e1f593efffffffull;  // -p^-1 mod 2^64
static constexpr uint64_t kOne[4] = {0xac96341c4ffffffbull, 0x36fc76959f60cd29ull, 0x666ea36f7879462eull,
                                     0x0e0a77c19a07df2full};
static constexpr uint64_t kR2[4] = {0x1bb8e645ae216da7ull, 0x53fe3ab1e35c59e3ull, 0x8c49833d53bb8085ull,
                                    0x0216d0b17f4e44a5ull};

struct F {
  uint64_t w[4];
  bool operator==(const F& o) const { return memcmp(w, o.w, 32) == 0; }
  bool operator!=(const F& o) const { return !(*this == o); }
  bool zero() const { return (w[0] | w[1] | w[2] | w[3]) == 0; }
};

inline F fzero() { return F{{0, 0, 0, 0}}; }
inline F fone() { return F{{kOne[0], kOne[1], kOne[2], kOne[3]}}; }

inline bool below_p(const uint64_t a[4]) {
  for (int i = 3; i >= 0; --i)
    if (a[i] != kP[i]) return a[i] < kP[i];
  return false;
}

// a - p when a >= p; a < 2p assumed.
inline void cond_sub_p(uint64_t a[4]) {
  if (below_p(a)) return;
  uint64_t borrow = 0;
  for (int i = 0; i < 4; ++i) {
    u128 d = (u128)a[i] - kP[i] - borrow;
    a[i] = (uint64_t)d;
    borrow = (uint64_t)(d >> 127);
  }
}

inline F fadd(const F& a, const F& b) {
  F r;
  uint64_t carry = 0;
  for (int i = 0; i < 4; ++i) {
    u128 s = (u128)a.w[i] + b.w[i] + carry;
    r.w[i] = (uint64_t)s;
    carry = (uint64_t)(s >> 64);
  }
  cond_sub_p(r.w);
  return r;
}

inline F fsub(const F& a, const F& b) {
  F r;
  uint64_t borrow = 0;
  for (int i = 0; i < 4; ++i) {
    u128 d = (u128)a.w[i] - b.w[i] - borrow;
    r.w[i] = (uint64_t)d;
    borrow = (uint64_t)(d >> 127);
  }
  if (borrow) {
    uint64_t carry = 0;
    for (int i = 0; i < 4; ++i) {
      u128 s = (u128)r.w[i] + kP[i] + carry;
      r.w[i] = (uint64_t)s;
      carry = (uint64_t)(s >> 64);
    }
  }
  return r;
}

inline F fneg(const F& a) { return a.zero() ? a : fsub(fzero(), a); }

// The full 512-bit product first (its sixteen limb products are independent),
// then the Montgomery reduction a limb at a time with only the low word of
// the running column on the dependency chain: after adding lo(m_i p_0) the
// column's carry is hi(col_i) + (lo(col_i) != 0) whatever that product is, so
// m_{i+1} waits for two products, not for a whole row. Measured on the Arm
// host cores: 18.2 ns a product against 19.6 ns for the interleaved rows.
// With `reduce` false the result is left in [0, 2p) (inputs below 2p keep
// it there: 4p^2 < p 2^256).
inline F fmul_r(const F& A, const F& B, bool reduce) {
  const uint64_t *a = A.w, *b = B.w;
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
    const uint64_t m = lo * kPInv;
    col[i + 1] += (uint64_t)(col[i] >> 64) + (uint64_t)(lo != 0);
    const u128 q0 = (u128)m * kP[0], q1 = (u128)m * kP[1], q2 = (u128)m * kP[2], q3 = (u128)m * kP[3];
    col[i + 1] += (u128)(uint64_t)(q0 >> 64) + (uint64_t)q1;
    col[i + 2] += (u128)(uint64_t)(q1 >> 64) + (uint64_t)q2;
    col[i + 3] += (u128)(uint64_t)(q2 >> 64) + (uint64_t)q3;
    col[i + 4] += (uint64_t)(q3 >> 64);
  }
  F r;
  u128 c = 0;
  for (int k = 0; k < 4; ++k) {
    c += col[4 + k];
    r.w[k] = (uint64_t)c;
    c >>= 64;
  }
  if (reduce) cond_sub_p(r.w);
  return r;
}

inline F fmul(const F& A, const F& B) { return fmul_r(A, B, true); }

inline F fsqr(const F& a) { return fmul(a, a); }

inline F from_canonical(const uint64_t c[4]) {
  F x{{c[0], c[1], c[2], c[3]}};
  return fmul(x, F{{kR2[0], kR2[1], kR2[2], kR2[3]}});
}

inline F from_u64(uint64_t v) {
  uint64_t c[4] = {v, 0, 0, 0};
  return from_canonical(c);
}

inline void to_canonical(const F& a, uint64_t out[4]) {
  F r = fmul(a, F{{1, 0, 0, 0}});
  memcpy(out, r.w, 32);
}

// Canonical little-endian bytes <-> F; false when the value is >= p.
inline bool from_bytes(const uint8_t b[32], F& out) {
  uint64_t c[4];
  memcpy(c, b, 32);
  if (!below_p(c)) return false;
  out = from_canonical(c);
  return true;
}

inline void to_bytes(const F& a, uint8_t b[32]) {
  uint64_t c[4];
  to_canonical(a, c);
  memcpy(b, c, 32);
}

inline F fpow(F base, const uint64_t e[4]) {
  F acc = fone();
  for (int i = 0; i < 4; ++i)
    for (int bit = 0; bit < 64; ++bit) {
      if ((e[i] >> bit) & 1) acc = fmul(acc, base);
      base = fsqr(base);
    }
  return acc;
}

inline F finv(const F& a) {
  uint64_t e[4] = {kP[0] - 2, kP[1], kP[2], kP[3]};
  return fpow(a, e);
}

inline F fpow_u64(F base, uint64_t e) {
  F acc = fone();
  while (e) {
    if (e & 1) acc = fmul(acc, base);
    base = fsqr(base);
    e >>= 1;
  }
  return acc;
}

// ---- Poseidon2 (width 3, x^5, 4 + 56 + 4 rounds) ----------------------------

#include "poseidon2_rc.inc"

inline F rc(int i) { return F{{kPoseidon2Rc[i][0], kPoseidon2Rc[i][1], kPoseidon2Rc[i][2], kPoseidon2Rc[i][3]}}; }

// Inside the permutation values stay in [0, 2p) (products unreduced, sums
// reduced by 2p), and the state is made canonical once at the end: the same
// field elements, 16 % faster on the Arm host cores than reducing every step.
static constexpr uint64_t k2P[4] = {0x87c3eb27e0000002ull, 0x5067d090f372e122ull, 0x70a08b6d0302b0baull,
                                    0x60c89ce5c2634053ull};

// a + b for a, b < 2p, the result below 2p.
inline F fadd_2p(const F& a, const F& b) {
  F r;
  uint64_t carry = 0;
  for (int i = 0; i < 4; ++i) {
    u128 s = (u128)a.w[i] + b.w[i] + carry;
    r.w[i] = (uint64_t)s;
    carry = (uint64_t)(s >> 64);
  }
  int i = 3;
  while (i >= 0 && r.w[i] == k2P[i]) --i;
  if (i < 0 || r.w[i] > k2P[i]) {
    uint64_t borrow = 0;
    for (int k = 0; k < 4; ++k) {
      u128 d = (u128)r.w[k] - k2P[k] - borrow;
      r.w[k] = (uint64_t)d;
      borrow = (uint64_t)(d >> 127);
    }
  }
  return r;
}

inline F pow5_2p(const F& x) {
  F x2 = fmul_r(x, x, false);
  return fmul_r(fmul_r(x2, x2, false), x, false);
}

inline void permute(F s[3]) {
  auto full_mix = [&]() {
    F t = fadd_2p(fadd_2p(s[0], s[1]), s[2]);
    for (int j = 0; j < 3; ++j) s[j] = fadd_2p(s[j], t);
  };
  full_mix();
  int k = 0;
  for (int r = 0; r < 4; ++r) {
    for (int j = 0; j < 3; ++j) s[j] = pow5_2p(fadd_2p(s[j], rc(k++)));
    full_mix();
  }
  for (int r = 0; r < 56; ++r) {
    s[0] = pow5_2p(fadd_2p(s[0], rc(k++)));
    F t = fadd_2p(fadd_2p(s[0], s[1]), s[2]);
    s[0] = fadd_2p(s[0], t);
    s[1] = fadd_2p(s[1], t);
    s[2] = fadd_2p(fadd_2p(s[2], s[2]), t);
  }
  for (int r = 0; r < 4; ++r) {
    for (int j = 0; j < 3; ++j) s[j] = pow5_2p(fadd_2p(s[j], rc(k++)));
    full_mix();
  }
  for (int j = 0; j < 3; ++j) cond_sub_p(s[j].w);
}

// ---- the duplex transcript ---------------------------------------------------

enum Tag : uint64_t {
  T_COMMITMENT = 3, T_SUMCHECK_ROUND = 4, T_SUMCHECK_CHALLENGE = 5, T_EVALUATION_CLAIM = 6, T_PCS_OPENING = 7,
  T_WITNESS_DIGEST = 8, T_SUMCHECK_FINAL_EVALS = 9, T_MERCURY_INSTANCE = 10, T_MERCURY_ALPHA = 11,
  T_MERCURY_GAMMA = 12, T_MERCURY_Z = 13, T_BDFG_BATCH = 14, T_BDFG_POINT = 15, T_PAIRING_MERGE = 16,
  T_MERCURY_BATCH = 17, T_PUBLIC_INPUT_STREAM = 20, T_PUBLIC_OUTPUT_STREAM = 21, T_GKR_OUTPUTS = 25,
  T_GKR_OUTPUT_POINT = 26, T_GKR_BATCH = 27, T_GKR_LAYER_CLAIMS = 28, T_GKR_CHILD = 29,
};

// The transcript's four limbs of a canonical 64-byte G1 encoding: the 128-bit
// halves of x and y; infinity (all zero bytes) is 2^128 four times
// (crates/transcript/src/lib.rs:493-510).
inline void g1_limbs(const uint8_t* p, F out[4]) {
  bool inf = true;
  for (int i = 0; i < 64; ++i) inf &= p[i] == 0;
  for (int h = 0; h < 4; ++h) {
    uint64_t c[4] = {0, 0, 0, 0};
    if (inf) c[2] = 1;
    else memcpy(c, p + 16 * h, 16);
    out[h] = from_canonical(c);
  }
}

// Rate 2, capacity 1, overwrite absorption; a squeeze pops from the end of
// the rate. Snapshot bytes: state[3], input[2], input_len, output[2],
// output_len with Fr canonical (226 bytes).
struct Transcript {
  F st[3] = {fzero(), fzero(), fzero()};
  F in[2] = {fzero(), fzero()};
  int in_len = 0;
  F out[2] = {fzero(), fzero()};
  int out_len = 0;

  void duplex() {
    const int pending = in_len;
    for (int i = 0; i < pending; ++i) {
      st[i] = in[i];
      in[i] = fzero();
    }
    in_len = 0;
    if (pending > 0) {
      for (int i = pending; i < 2; ++i) st[i] = fzero();
      st[2] = fadd(st[2], from_u64((uint64_t)pending));
    }
    permute(st);
    out[0] = st[0];
    out[1] = st[1];
    out_len = 2;
  }
  void observe(const F& x) {
    out[0] = out[1] = fzero();
    out_len = 0;
    in[in_len++] = x;
    if (in_len == 2) duplex();
  }
  F sample() {
    if (in_len > 0 || out_len == 0) duplex();
    --out_len;
    F r = out[out_len];
    out[out_len] = fzero();
    return r;
  }
  void absorb(uint64_t tag, const F* xs, size_t n) {
    observe(from_u64(tag));
    observe(from_u64((uint64_t)n));
    for (size_t i = 0; i < n; ++i) observe(xs[i]);
  }
  void absorb(uint64_t tag, const std::vector<F>& xs) { absorb(tag, xs.data(), xs.size()); }
  F challenge(uint64_t tag) {
    observe(from_u64(tag));
    return sample();
  }
  // Transcript::append_bytes (crates/transcript/src/lib.rs:324-338): the tag,
  // the byte length, then the bytes 31 at a time as little-endian limbs, the
  // last one zero-extended.
  void absorb_bytes(uint64_t tag, const uint8_t* b, size_t len) {
    observe(from_u64(tag));
    observe(from_u64((uint64_t)len));
    for (size_t off = 0; off < len; off += 31) {
      uint64_t c[4] = {0, 0, 0, 0};
      memcpy(c, b + off, len - off < 31 ? len - off : 31);
      observe(from_canonical(c));
    }
  }
  // A G1 point list as one message of 4 limbs a point (g1_limbs).
  void absorb_g1(uint64_t tag, const uint8_t* pts, size_t n) {
    std::vector<F> limbs(4 * n);
    for (size_t k = 0; k < n; ++k) g1_limbs(pts + 64 * k, &limbs[4 * k]);
    absorb(tag, limbs);
  }

  bool load(const uint8_t b[226]) {
    const uint8_t* p = b;
    for (int i = 0; i < 3; ++i, p += 32)
      if (!from_bytes(p, st[i])) return false;
    for (int i = 0; i < 2; ++i, p += 32)
      if (!from_bytes(p, in[i])) return false;
    in_len = *p++;
    for (int i = 0; i < 2; ++i, p += 32)
      if (!from_bytes(p, out[i])) return false;
    out_len = *p++;
    if (in_len >= 2 || out_len > 2) return false;
    for (int i = in_len; i < 2; ++i)
      if (!in[i].zero()) return false;
    for (int i = out_len; i < 2; ++i)
      if (!out[i].zero()) return false;
    return true;
  }
  void save(uint8_t b[226]) const {
    uint8_t* p = b;
    for (int i = 0; i < 3; ++i, p += 32) to_bytes(st[i], p);
    for (int i = 0; i < 2; ++i, p += 32) to_bytes(in[i], p);
    *p++ = (uint8_t)in_len;
    for (int i = 0; i < 2; ++i, p += 32) to_bytes(out[i], p);
    *p++ = (uint8_t)out_len;
  }
};

// io_digest (crates/transcript/src/lib.rs:464-475): the public input and
// output byte streams in a sponge of their own, then one raw squeeze.
inline F io_digest(const uint8_t* in, size_t in_len, const uint8_t* out, size_t out_len) {
  Transcript t;
  t.absorb_bytes(T_PUBLIC_INPUT_STREAM, in, in_len);
  t.absorb_bytes(T_PUBLIC_OUTPUT_STREAM, out, out_len);
  return t.sample();
}

// The cubic through (0,v0),(1,v1),(2,v2),(3,v3), ascending coefficients, by
// Newton's forward differences (crates/sumcheck/src/lib.rs:294-305).
inline std::array<F, 4> cubic_through(const F v[4]) {
  static const F inv2 = finv(from_u64(2)), inv3 = finv(from_u64(3)), inv6 = finv(from_u64(6));
  F d1 = fsub(v[1], v[0]);
  F d2 = fsub(fsub(v[2], v[1]), d1);
  F d3 = fsub(fsub(fsub(v[3], v[2]), fsub(v[2], v[1])), d2);
  return {v[0], fadd(fsub(d1, fmul(d2, inv2)), fmul(d3, inv3)), fmul(fsub(d2, d3), inv2), fmul(d3, inv6)};
}

}  // namespace host
}  // namespace apg
