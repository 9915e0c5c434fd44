// ORACLE — test infrastructure only. CPU restatement of BN254 G1 and the
// reference's windowed signed-digit Pippenger, for checking and timing the
// CUDA library.
//
// G1 formulas follow crates/curve/src/g1.rs: add-2007-bl (:155-197),
// madd-2007-bl (:203-243), dbl-2009-l (:246-277), the 4-bit fixed-window
// scalar ladder (:279-304), to_affine (:310-322) and the wire form (:92-127).
// The MSM follows crates/curve/src/msm.rs: window_bits (:112-118), log2
// (:121-127), window_count (:140-142), recode (:180-198), recode_u32
// (:203-224), pippenger's window x chunk split and Horner (:232-274) and
// window_sum's running sum (:277-311).
#pragma once
#include <thread>
#include <vector>

#include "field.hpp"

namespace oracle {

struct G1Affine {
  Fq x, y;
  bool inf;
  static G1Affine identity() { return G1Affine{Fq::zero(), Fq::zero(), true}; }
  static G1Affine generator() { return G1Affine{Fq::one(), Fq::from_u64(2), false}; }
  bool on_curve() const {
    if (inf) return true;
    return y.square() == x.square() * x + Fq::from_u64(3);
  }
  void to_bytes(uint8_t out[64]) const {
    if (inf) {
      memset(out, 0, 64);
      return;
    }
    x.to_bytes(out);
    y.to_bytes(out + 32);
  }
  // All-zero is infinity; otherwise both coordinates canonical and on curve.
  static bool from_bytes(const uint8_t b[64], G1Affine& out) {
    bool allz = true;
    for (int i = 0; i < 64; ++i) allz &= (b[i] == 0);
    if (allz) {
      out = identity();
      return true;
    }
    if (!Fq::from_bytes(b, out.x) || !Fq::from_bytes(b + 32, out.y)) return false;
    out.inf = false;
    return out.on_curve();
  }
  G1Affine neg() const { return inf ? *this : G1Affine{x, -y, false}; }
};

struct G1Jac {
  Fq x, y, z;
  static G1Jac identity() { return G1Jac{Fq::one(), Fq::one(), Fq::zero()}; }
  static G1Jac from(const G1Affine& p) {
    return p.inf ? identity() : G1Jac{p.x, p.y, Fq::one()};
  }
  bool is_identity() const { return z.is_zero(); }

  G1Jac dbl() const {
    if (is_identity()) return identity();
    Fq a = x.square(), b = y.square(), c = b.square();
    Fq t = (x + b).square() - a - c;
    Fq d = t + t;
    Fq e = a + a + a;
    Fq f = e.square();
    Fq x3 = f - d - d;
    Fq c8 = c.dbl().dbl().dbl();
    Fq y3 = e * (d - x3) - c8;
    Fq yz = y * z;
    return G1Jac{x3, y3, yz + yz};
  }
  G1Jac add(const G1Jac& o) const {
    if (is_identity()) return o;
    if (o.is_identity()) return *this;
    Fq z1z1 = z.square(), z2z2 = o.z.square();
    Fq u1 = x * z2z2, u2 = o.x * z1z1;
    Fq s1 = y * z2z2 * o.z, s2 = o.y * z1z1 * z;
    Fq h = u2 - u1;
    Fq d = s2 - s1;
    Fq r = d + d;
    if (h.is_zero()) {
      if (r.is_zero()) return dbl();
      return identity();
    }
    Fq th = h + h;
    Fq i = th.square();
    Fq j = h * i;
    Fq v = u1 * i;
    Fq x3 = r.square() - j - v - v;
    Fq s1j = s1 * j;
    Fq y3 = r * (v - x3) - (s1j + s1j);
    Fq z3 = ((z + o.z).square() - z1z1 - z2z2) * h;
    return G1Jac{x3, y3, z3};
  }
  G1Jac add_affine(const G1Affine& o) const {
    if (o.inf) return *this;
    if (is_identity()) return from(o);
    Fq z1z1 = z.square();
    Fq u2 = o.x * z1z1;
    Fq s2 = o.y * z1z1 * z;
    Fq h = u2 - x;
    Fq d = s2 - y;
    Fq r = d + d;
    if (h.is_zero()) {
      if (r.is_zero()) return dbl();
      return identity();
    }
    Fq hh = h.square();
    Fq i = (hh + hh).dbl();
    Fq j = h * i;
    Fq v = x * i;
    Fq x3 = r.square() - j - v - v;
    Fq y1j = y * j;
    Fq y3 = r * (v - x3) - (y1j + y1j);
    Fq z3 = (z + h).square() - z1z1 - hh;
    return G1Jac{x3, y3, z3};
  }
  // Fixed 4-bit window over a 256-bit little-endian integer (g1.rs:279-304).
  G1Jac mul_le_bytes(const uint8_t s[32]) const {
    G1Jac table[16];
    table[0] = identity();
    table[1] = *this;
    for (int i = 2; i < 16; ++i) table[i] = table[i - 1].add(*this);
    G1Jac acc = identity();
    for (int bi = 31; bi >= 0; --bi) {
      int nib[2] = {s[bi] >> 4, s[bi] & 15};
      for (int k = 0; k < 2; ++k) {
        acc = acc.dbl().dbl().dbl().dbl();
        acc = acc.add(table[nib[k]]);
      }
    }
    return acc;
  }
  G1Jac mul(const Fr& k) const {
    uint8_t b[32];
    k.to_bytes(b);
    return mul_le_bytes(b);
  }
  G1Affine to_affine() const {
    if (is_identity()) return G1Affine::identity();
    Fq zi = z.inverse();
    Fq zi2 = zi.square();
    return G1Affine{x * zi2, y * zi2 * zi, false};
  }
};

// Batch normalisation with one inversion (g1.rs:328-347).
inline std::vector<G1Affine> batch_to_affine(const std::vector<G1Jac>& ps) {
  std::vector<Fq> zs(ps.size());
  for (size_t i = 0; i < ps.size(); ++i) zs[i] = ps[i].z;
  batch_inverse(zs);
  std::vector<G1Affine> out(ps.size());
  for (size_t i = 0; i < ps.size(); ++i) {
    if (zs[i].is_zero()) {
      out[i] = G1Affine::identity();
    } else {
      Fq zi2 = zs[i].square();
      out[i] = G1Affine{ps[i].x * zi2, ps[i].y * zi2 * zs[i], false};
    }
  }
  return out;
}

// ---------------------------------------------------------------------------
// Pippenger, restated from crates/curve/src/msm.rs.
// ---------------------------------------------------------------------------

inline size_t msm_log2(size_t n) {
  if ((n & (n - 1)) == 0) return (size_t)__builtin_ctzll(n);
  return 64 - (size_t)__builtin_clzll(n);
}
inline size_t msm_window_bits(size_t n) { return n < 32 ? 3 : (msm_log2(n) * 69) / 100 + 2; }
inline size_t msm_window_count(size_t bits, size_t w) { return (bits + 1 + w - 1) / w; }

inline uint64_t window_of(const uint64_t limbs[4], size_t offset, size_t w) {
  size_t limb = offset / 64, shift = offset % 64;
  uint64_t v = limbs[limb] >> shift;
  if (shift > 0 && limb + 1 < 4) v |= limbs[limb + 1] << (64 - shift);
  return v & ((1ULL << w) - 1);
}

inline void recode(const uint64_t limbs[4], size_t w, int32_t* out, size_t windows) {
  uint64_t half = 1ULL << (w - 1);
  int64_t radix = 1LL << w;
  uint64_t carry = 0;
  for (size_t i = 0; i < windows; ++i) {
    uint64_t coef = window_of(limbs, i * w, w) + carry;
    if (i == windows - 1) {
      out[i] = (int32_t)coef;
    } else if (coef >= half) {
      out[i] = (int32_t)((int64_t)coef - radix);
      carry = 1;
    } else {
      out[i] = (int32_t)coef;
      carry = 0;
    }
  }
}

inline G1Jac window_sum(const G1Affine* bases, const int32_t* digits, size_t len, size_t windows,
                        size_t window, size_t buckets) {
  if (len == 0) return G1Jac::identity();
  std::vector<G1Jac> bucket(buckets, G1Jac::identity());
  for (size_t j = 0; j < len; ++j) {
    int32_t d = digits[j * windows + window];
    if (d == 0) continue;
    size_t slot = (size_t)(d < 0 ? -d : d) - 1;
    bucket[slot] = d > 0 ? bucket[slot].add_affine(bases[j]) : bucket[slot].add_affine(bases[j].neg());
  }
  G1Jac running = G1Jac::identity(), total = G1Jac::identity();
  for (size_t k = buckets; k-- > 0;) {
    running = running.add(bucket[k]);
    total = total.add(running);
  }
  return total;
}

inline G1Jac pippenger(const G1Affine* bases, const int32_t* digits, size_t n, size_t windows,
                       size_t w, size_t threads) {
  size_t buckets = 1ULL << (w - 1);
  size_t chunks = (threads + windows - 1) / windows;
  size_t hi = std::max<size_t>(n / buckets, 1);
  if (chunks < 1) chunks = 1;
  if (chunks > hi) chunks = hi;
  size_t chunk_len = (n + chunks - 1) / chunks;
  size_t tasks = windows * chunks;
  std::vector<G1Jac> partials(tasks);
  auto run = [&](size_t task) {
    size_t start = std::min((task % chunks) * chunk_len, n);
    size_t end = std::min(start + chunk_len, n);
    partials[task] = window_sum(bases + start, digits + start * windows, end - start, windows,
                                task / chunks, buckets);
  };
  std::vector<std::thread> pool;
  size_t nt = std::max<size_t>(1, std::min(threads, tasks));
  for (size_t t = 0; t < nt; ++t)
    pool.emplace_back([&, t] {
      for (size_t task = t; task < tasks; task += nt) run(task);
    });
  for (auto& th : pool) th.join();
  G1Jac acc = G1Jac::identity();
  for (size_t win = windows; win-- > 0;) {
    for (size_t i = 0; i < w; ++i) acc = acc.dbl();
    for (size_t c = 0; c < chunks; ++c) acc = acc.add(partials[win * chunks + c]);
  }
  return acc;
}

// msm::msm (msm.rs:48-69): 254-bit scalars through the general path.
inline G1Jac msm(const G1Affine* bases, const Fr* scalars, size_t n, size_t threads) {
  if (n == 0) return G1Jac::identity();
  size_t w = msm_window_bits(n);
  size_t windows = msm_window_count(254, w);
  std::vector<int32_t> digits(n * windows);
  for (size_t i = 0; i < n; ++i) {
    uint8_t b[32];
    scalars[i].to_bytes(b);
    uint64_t limbs[4];
    memcpy(limbs, b, 32);
    recode(limbs, w, &digits[i * windows], windows);
  }
  return pippenger(bases, digits.data(), n, windows, w, threads);
}

// msm::msm_small_u32 (msm.rs:79-100).
inline G1Jac msm_u32(const G1Affine* bases, const uint32_t* scalars, size_t n, size_t threads) {
  if (n == 0) return G1Jac::identity();
  size_t w = msm_window_bits(n);
  size_t windows = msm_window_count(32, w);
  std::vector<int32_t> digits(n * windows);
  for (size_t i = 0; i < n; ++i) {
    uint64_t limbs[4] = {scalars[i], 0, 0, 0};
    recode(limbs, w, &digits[i * windows], windows);
  }
  return pippenger(bases, digits.data(), n, windows, w, threads);
}

}  // namespace oracle
