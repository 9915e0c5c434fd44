// ORACLE — test infrastructure only. CPU restatement of the reference's
// width-3 BN254 Poseidon2 permutation and its duplex transcript.
//
// Permutation: crates/transcript/src/lib.rs:44-146 (x^5 S-box, external matrix
// [[2,1,1],[1,2,1],[1,1,2]], internal matrix 1 + diag(1,1,2), 4 + 56 + 4 rounds).
// The round constants are not transcribed: they are regenerated here with the
// Grain LFSR of the Poseidon paper (field = prime, n = 254, t = 3, R_F = 8,
// R_P = 56, R_F*t + R_P constants), the published procedure behind the
// reference's RC3 tables (crates/constants/src/lib.rs:439-560), and the
// permutation is pinned by crates/transcript/tests/vectors/poseidon2_perm.txt.
// Duplex and typed layer: lib.rs:214-346; snapshot: :353-376; g1_limbs: :493-510.
#pragma once
#include <array>
#include <vector>

#include "field.hpp"

namespace oracle {

namespace tags {
enum : uint64_t {
  PROTOCOL_SUITE = 1, PUBLIC_INPUTS = 2, COMMITMENT = 3, SUMCHECK_ROUND = 4,
  SUMCHECK_CHALLENGE = 5, EVALUATION_CLAIM = 6, PCS_OPENING = 7, WITNESS_DIGEST = 8,
  SUMCHECK_FINAL_EVALS = 9, MERCURY_INSTANCE = 10, MERCURY_ALPHA = 11, MERCURY_GAMMA = 12,
  MERCURY_Z = 13, BDFG_BATCH = 14, BDFG_POINT = 15, PAIRING_MERGE = 16, MERCURY_BATCH = 17,
  ACCUMULATOR_DIGEST = 18, ACCUMULATOR_MERGE = 19,
  GKR_OUTPUTS = 25, GKR_OUTPUT_POINT = 26, GKR_BATCH = 27, GKR_LAYER_CLAIMS = 28,
  GKR_CHILD = 29, SHARD_SEED = 39, SHARD_TS_WINDOW = 40,
};
}

struct Poseidon2Constants {
  Fr initial[4][3];
  Fr internal[56];
  Fr terminal[4][3];
};

// Grain LFSR (Poseidon paper, appendix on parameter generation): an 80-bit
// register seeded with the instance description, 160 warm-up clocks, then
// bits taken in pairs (a, b) keeping b when a = 1; each constant is 254 bits
// read most-significant first, rejected when >= p.
inline Poseidon2Constants make_poseidon2_constants() {
  std::vector<int> st;
  auto push_bits = [&](uint64_t v, int width) {
    for (int i = width - 1; i >= 0; --i) st.push_back((int)((v >> i) & 1));
  };
  push_bits(1, 2);    // prime field
  push_bits(0, 4);    // x^alpha S-box
  push_bits(254, 12); // field bits
  push_bits(3, 12);   // width
  push_bits(8, 10);   // full rounds
  push_bits(56, 10);  // partial rounds
  for (int i = 0; i < 30; ++i) st.push_back(1);
  size_t head = 0;
  std::vector<int> reg(st);
  auto clock = [&]() {
    int b = reg[head + 62] ^ reg[head + 51] ^ reg[head + 38] ^ reg[head + 23] ^ reg[head + 13] ^
            reg[head];
    reg.push_back(b);
    ++head;
    return b;
  };
  for (int i = 0; i < 160; ++i) clock();
  auto next_bit = [&]() {
    for (;;) {
      int a = clock();
      int b = clock();
      if (a) return b;
    }
  };
  std::vector<Fr> out;
  while (out.size() < 8 * 3 + 56) {
    uint64_t limbs[4] = {0, 0, 0, 0};
    for (int i = 253; i >= 0; --i) {
      if (next_bit()) limbs[i / 64] |= 1ULL << (i % 64);
    }
    Fr x;
    if (Fr::from_bytes((const uint8_t*)limbs, x)) out.push_back(x);
  }
  Poseidon2Constants c;
  size_t k = 0;
  for (int r = 0; r < 4; ++r)
    for (int j = 0; j < 3; ++j) c.initial[r][j] = out[k++];
  for (int r = 0; r < 56; ++r) c.internal[r] = out[k++];
  for (int r = 0; r < 4; ++r)
    for (int j = 0; j < 3; ++j) c.terminal[r][j] = out[k++];
  return c;
}

inline const Poseidon2Constants& poseidon2_constants() {
  static const Poseidon2Constants c = make_poseidon2_constants();
  return c;
}

inline Fr sbox5(const Fr& x) {
  Fr x2 = x.square();
  return x2.square() * x;
}

inline void poseidon2_permute(Fr s[3]) {
  const Poseidon2Constants& c = poseidon2_constants();
  auto ext = [&]() {
    Fr sum = s[0] + s[1] + s[2];
    s[0] += sum;
    s[1] += sum;
    s[2] += sum;
  };
  ext();
  for (int r = 0; r < 4; ++r) {
    for (int j = 0; j < 3; ++j) s[j] = sbox5(s[j] + c.initial[r][j]);
    ext();
  }
  for (int r = 0; r < 56; ++r) {
    s[0] = sbox5(s[0] + c.internal[r]);
    Fr sum = s[0] + s[1] + s[2];
    s[0] += sum;
    s[1] += sum;
    s[2] = s[2] + s[2] + sum;
  }
  for (int r = 0; r < 4; ++r) {
    for (int j = 0; j < 3; ++j) s[j] = sbox5(s[j] + c.terminal[r][j]);
    ext();
  }
}

// The overwrite-mode rate-2 duplex with the typed tag/length framing.
struct Transcript {
  Fr state[3] = {Fr::zero(), Fr::zero(), Fr::zero()};
  Fr input[2] = {Fr::zero(), Fr::zero()};
  int input_len = 0;
  Fr output[2] = {Fr::zero(), Fr::zero()};
  int output_len = 0;

  void duplex() {
    int n = input_len;
    for (int i = 0; i < n; ++i) {
      state[i] = input[i];
      input[i] = Fr::zero();
    }
    input_len = 0;
    if (n > 0) {
      for (int i = n; i < 2; ++i) state[i] = Fr::zero();
      state[2] += Fr::from_u64((uint64_t)n);
    }
    poseidon2_permute(state);
    output[0] = state[0];
    output[1] = state[1];
    output_len = 2;
  }
  void observe(const Fr& x) {
    output[0] = output[1] = Fr::zero();
    output_len = 0;
    input[input_len++] = x;
    if (input_len == 2) duplex();
  }
  Fr sample() {
    if (input_len > 0 || output_len == 0) duplex();
    output_len -= 1;
    Fr out = output[output_len];
    output[output_len] = Fr::zero();
    return out;
  }
  void append_scalars(uint64_t tag, const Fr* xs, size_t n) {
    observe(Fr::from_u64(tag));
    observe(Fr::from_u64((uint64_t)n));
    for (size_t i = 0; i < n; ++i) observe(xs[i]);
  }
  void append_scalars(uint64_t tag, const std::vector<Fr>& xs) {
    append_scalars(tag, xs.data(), xs.size());
  }
  void append_scalar(uint64_t tag, const Fr& x) { append_scalars(tag, &x, 1); }
  void append_bytes(uint64_t tag, const uint8_t* b, size_t len) {
    observe(Fr::from_u64(tag));
    observe(Fr::from_u64((uint64_t)len));
    for (size_t off = 0; off < len; off += 31) {
      uint8_t limb[32] = {0};
      size_t take = std::min<size_t>(31, len - off);
      memcpy(limb, b + off, take);
      Fr x;
      Fr::from_bytes(limb, x);
      observe(x);
    }
  }
  Fr challenge(uint64_t tag) {
    observe(Fr::from_u64(tag));
    return sample();
  }

  // TranscriptSnapshot's serde tuple (state, input, input_len, output,
  // output_len): Fr as canonical 32 bytes, the lengths as one byte each.
  static constexpr size_t SNAPSHOT_BYTES = 3 * 32 + 2 * 32 + 1 + 2 * 32 + 1;
  void snapshot(uint8_t out[SNAPSHOT_BYTES]) const {
    uint8_t* p = out;
    for (int i = 0; i < 3; ++i, p += 32) state[i].to_bytes(p);
    for (int i = 0; i < 2; ++i, p += 32) input[i].to_bytes(p);
    *p++ = (uint8_t)input_len;
    for (int i = 0; i < 2; ++i, p += 32) output[i].to_bytes(p);
    *p++ = (uint8_t)output_len;
  }
  bool restore(const uint8_t in[SNAPSHOT_BYTES]) {
    const uint8_t* p = in;
    for (int i = 0; i < 3; ++i, p += 32)
      if (!Fr::from_bytes(p, state[i])) return false;
    for (int i = 0; i < 2; ++i, p += 32)
      if (!Fr::from_bytes(p, input[i])) return false;
    input_len = *p++;
    for (int i = 0; i < 2; ++i, p += 32)
      if (!Fr::from_bytes(p, output[i])) return false;
    output_len = *p++;
    return input_len < 2 && output_len <= 2;
  }
};

// A G1 point's four transcript limbs: x low/high and y low/high 128-bit
// halves of the canonical encoding; infinity absorbs 2^128 four times.
inline std::array<Fr, 4> g1_limbs(const uint8_t p[64]) {
  std::array<Fr, 4> out;
  bool allz = true;
  for (int i = 0; i < 64; ++i) allz &= p[i] == 0;
  if (allz) {
    uint8_t s[32] = {0};
    s[16] = 1;
    Fr x;
    Fr::from_bytes(s, x);
    out.fill(x);
    return out;
  }
  for (int k = 0; k < 4; ++k) {
    uint8_t b[32] = {0};
    memcpy(b, p + 16 * k, 16);
    Fr::from_bytes(b, out[k]);
  }
  return out;
}

inline void append_g1_points(Transcript& tr, uint64_t tag, const std::vector<std::array<uint8_t, 64>>& pts) {
  std::vector<Fr> limbs;
  for (auto& p : pts) {
    auto l = g1_limbs(p.data());
    limbs.insert(limbs.end(), l.begin(), l.end());
  }
  tr.append_scalars(tag, limbs);
}

}  // namespace oracle
