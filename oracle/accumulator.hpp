// ORACLE — test infrastructure only. The deferred-pairing accumulator's group
// side, restated from the reference:
//   crates/pcs/src/accumulator.rs   partition :252-270, accumulator_words
//                                   :57-83, discharge :146-163, check_pairings
//                                   :171-218 (everything before the pairing)
//   crates/pcs-verify/src/lib.rs    PairingSide words :244-251, entry_words
//                                   :297-300, accumulator_digest :315-319,
//                                   powers :137-145
// The two-pairing check itself (curve::pairing) is not restated: the caller
// gets A and B and checks e(A, [1]_2) * e(-B, [x]_2) == 1.
#pragma once
#include <vector>

#include "curve.hpp"
#include "transcript.hpp"

namespace oracle {

struct AccEntry {
  int side;  // 0 = G2One (a term of A), 1 = G2X (a term of B)
  Fr scalar;
  G1Affine point;
};

// accumulator.rs:252-270: the counts partition the entries, in order.
inline bool acc_partition(size_t n_entries, const std::vector<size_t>& checks) {
  size_t offset = 0;
  for (size_t count : checks) {
    if (count > n_entries - offset) return false;
    offset += count;
  }
  return offset == n_entries;
}

// accumulator.rs:57-83 with pcs-verify entry_words: per check its count word,
// then six words an entry (side, scalar, the point's four transcript limbs).
inline std::vector<Fr> acc_words(const std::vector<AccEntry>& entries, const std::vector<size_t>& checks) {
  std::vector<Fr> words;
  size_t at = 0;
  for (size_t count : checks) {
    words.push_back(Fr::from_u64(count));
    for (size_t i = at; i < at + count; ++i) {
      const AccEntry& e = entries[i];
      words.push_back(e.side ? Fr::one() : Fr::zero());
      words.push_back(e.scalar);
      uint8_t raw[64];
      e.point.to_bytes(raw);
      for (const Fr& limb : g1_limbs(raw)) words.push_back(limb);
    }
    at += count;
  }
  return words;
}

// pcs-verify/src/lib.rs:315-319: a sponge of its own, the words under
// ACCUMULATOR_DIGEST, one raw squeeze.
inline Fr acc_digest(const std::vector<Fr>& words) {
  Transcript t;
  t.append_scalars(tags::ACCUMULATOR_DIGEST, words);
  return t.sample();
}

// accumulator.rs:155-160: the merge challenge nu from the digest.
inline Fr acc_merge_challenge(const Fr& digest) {
  Transcript t;
  t.append_scalar(tags::ACCUMULATOR_DIGEST, digest);
  return t.challenge(tags::ACCUMULATOR_MERGE);
}

// accumulator.rs:186-214: every entry's scalar times its check's weight, on
// its side, and one MSM per side.
inline void acc_side_msms(const std::vector<AccEntry>& entries, const std::vector<size_t>& checks,
                          const std::vector<Fr>& weights, size_t threads, G1Affine& a, G1Affine& b) {
  std::vector<G1Affine> ab, bb;
  std::vector<Fr> as, bs;
  size_t at = 0;
  for (size_t j = 0; j < checks.size(); ++j) {
    for (size_t i = at; i < at + checks[j]; ++i) {
      const Fr s = weights[j] * entries[i].scalar;
      if (entries[i].side == 0) {
        ab.push_back(entries[i].point);
        as.push_back(s);
      } else {
        bb.push_back(entries[i].point);
        bs.push_back(s);
      }
    }
    at += checks[j];
  }
  a = msm(ab.data(), as.data(), ab.size(), threads).to_affine();
  b = msm(bb.data(), bs.data(), bb.size(), threads).to_affine();
}

// pcs-verify/src/lib.rs:137-145.
inline std::vector<Fr> acc_powers(const Fr& x, size_t k) {
  std::vector<Fr> out;
  Fr acc = Fr::one();
  for (size_t i = 0; i < k; ++i) {
    out.push_back(acc);
    acc = acc * x;
  }
  return out;
}

}  // namespace oracle
