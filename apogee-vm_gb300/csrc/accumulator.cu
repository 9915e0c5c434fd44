// The group side of the deferred-pairing accumulator: pcs::discharge and
// check_pairings (crates/pcs/src/accumulator.rs:146-218) up to the pairing.
//
// An accumulator is a list of (side, scalar, point) entries grouped into
// deferred checks; discharging it weights check j by nu^j and sums every
// entry's weighted term on its side, A over the G2One entries and B over the
// G2X ones. Aggregating many shard proofs makes that two MSMs over as many
// generic bases as there are entries (twelve a Mercury verification).
//
// Device: point validation (on the curve; G1's cofactor is 1, so that is the
// subgroup check too), the per-entry weighted scalars, and both sides as one
// two-column MSM over the shared bases, each column zero where the entry is on
// the other side. Host: the partition, the accumulator's words and their
// Poseidon2 digest (one sequential sponge, computed while the device validates
// the points) and the merge challenge.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "host_fr.hpp"

namespace apg {

using host::F;

namespace {

constexpr uint64_t kTagAccumulatorDigest = 18;  // crates/constants/src/lib.rs:659
constexpr uint64_t kTagAccumulatorMerge = 19;   // crates/constants/src/lib.rs:665

// One thread an entry: its check is the last with first[j] <= i (empty checks
// share their successor's first entry), its term w_j * s_i goes to its side's
// column and zero to the other.
__global__ void k_side_scalars(const Fr* s, const uint8_t* side, size_t n, const uint64_t* first, int nchecks,
                               const Fr* w, Fr* a, Fr* b) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int lo = 0, hi = nchecks - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (first[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  const Fr v = fe_mul(ld_fe(&w[lo]), ld_fe(&s[i]));
  const Fr z = fe_zero<FrConsts>();
  const bool g2x = side[i] != 0;
  st_fe(&a[i], g2x ? z : v);
  st_fe(&b[i], g2x ? v : z);
}

// accumulator.rs:252-270: the counts cover the entries exactly, in order.
// `first` receives each check's first entry.
bool partition(size_t n, const size_t* checks, size_t nchecks, std::vector<uint64_t>& first) {
  first.resize(nchecks);
  size_t offset = 0;
  for (size_t j = 0; j < nchecks; ++j) {
    if (checks[j] > n - offset) return false;
    first[j] = offset;
    offset += checks[j];
  }
  return offset == n;
}

// pcs-verify/src/lib.rs:315-319 over accumulator_words (accumulator.rs:57-83):
// per check its count word, then per entry its side word, scalar and limbs,
// absorbed as one message under ACCUMULATOR_DIGEST, then one raw squeeze;
// accumulator.rs:155-160: nu = challenge(ACCUMULATOR_MERGE) after the digest.
F merge_challenge(const uint8_t* sides, const uint8_t* scalars, const uint8_t* points, const size_t* checks,
                  size_t nchecks, size_t n, F* digest_out) {
  host::Transcript sponge;
  sponge.observe(host::from_u64(kTagAccumulatorDigest));
  sponge.observe(host::from_u64((uint64_t)(nchecks + 6 * n)));
  size_t i = 0;
  for (size_t j = 0; j < nchecks; ++j) {
    sponge.observe(host::from_u64((uint64_t)checks[j]));
    for (size_t e = 0; e < checks[j]; ++e, ++i) {
      sponge.observe(sides[i] ? host::fone() : host::fzero());
      F s;
      memcpy(s.w, scalars + 32 * i, 32);
      sponge.observe(s);
      F limbs[4];
      host::g1_limbs(points + 64 * i, limbs);
      for (const F& l : limbs) sponge.observe(l);
    }
  }
  const F digest = sponge.sample();
  if (digest_out) *digest_out = digest;
  host::Transcript t;
  t.absorb(kTagAccumulatorDigest, &digest, 1);
  return t.challenge(kTagAccumulatorMerge);
}

}  // namespace

int accumulator_msms(Ctx& c, const uint8_t* sides, const uint8_t* scalars, const uint8_t* points, size_t n,
                     const size_t* checks, size_t nchecks, const uint8_t* weights, uint8_t* a_out, uint8_t* b_out,
                     uint8_t* nu_out) {
  if (!a_out || !b_out) return APG_ERR_INVALID_ARGUMENT;
  if (n && (!sides || !scalars || !points)) return APG_ERR_INVALID_ARGUMENT;
  if (nchecks && !checks) return APG_ERR_INVALID_ARGUMENT;
  if (n >= ((size_t)1 << 31) || nchecks >= ((size_t)1 << 31)) return APG_ERR_INVALID_ARGUMENT;
  for (size_t i = 0; i < n; ++i)
    if (sides[i] > 1) {
      c.last_error = "a side tag that is neither 0 (G2One) nor 1 (G2X)";
      return APG_ERR_INVALID_ARGUMENT;
    }
  for (size_t i = 0; i < n; ++i) {
    uint64_t w[4];
    memcpy(w, scalars + 32 * i, 32);
    if (!host::below_p(w)) {
      c.last_error = "a scalar that is not a reduced Fr";
      return APG_ERR_NONCANONICAL;
    }
  }
  const bool discharge = weights == nullptr;
  std::vector<F> w(nchecks);
  for (size_t j = 0; !discharge && j < nchecks; ++j) {
    memcpy(w[j].w, weights + 32 * j, 32);
    if (!host::below_p(w[j].w)) {
      c.last_error = "a weight that is not a reduced Fr";
      return APG_ERR_NONCANONICAL;
    }
  }
  std::vector<uint64_t> first;
  const bool partitioned = partition(n, checks, nchecks, first);
  // check_pairings refuses a bad partition before it looks at a point;
  // discharge validates every point first (accumulator.rs:151, :177-185).
  if (!discharge && !partitioned) {
    c.last_error = "the check counts do not partition the entries";
    return APG_ERR_MALFORMED_ACCUMULATOR;
  }
  Affine* d_pts = c.scratch[S_BASES].as<Affine>(std::max<size_t>(n, 1));
  upload_points_async(c, points, n, d_pts);
  // Nothing returns between here and the flag check, which clears them.
  if (discharge && partitioned) {
    F digest;
    const F nu = merge_challenge(sides, scalars, points, checks, nchecks, n, &digest);
    F acc = host::fone();
    for (size_t j = 0; j < nchecks; ++j) {
      w[j] = acc;
      acc = host::fmul(acc, nu);
    }
    if (nu_out) memcpy(nu_out, nu.w, 32);
  }
  if (n) c.check_flags();
  if (!partitioned) {
    c.last_error = "the check counts do not partition the entries";
    return APG_ERR_MALFORMED_ACCUMULATOR;
  }
  if (n == 0) {
    memset(a_out, 0, 64);
    memset(b_out, 0, 64);
    return APG_OK;
  }

  Fr* d_s = c.scratch[S_TMP5].as<Fr>(n);
  uint8_t* d_side = c.scratch[S_ENTRIES].as<uint8_t>(n);
  uint8_t* d_meta = c.scratch[S_TMP6].as<uint8_t>(40 * nchecks);
  Fr* d_w = reinterpret_cast<Fr*>(d_meta);
  uint64_t* d_first = reinterpret_cast<uint64_t*>(d_meta + 32 * nchecks);
  Fr* d_cols = c.scratch[S_SCALARS].as<Fr>(2 * n);
  APG_CUDA(cudaMemcpyAsync(d_s, scalars, 32 * n, cudaMemcpyHostToDevice, c.stream));
  APG_CUDA(cudaMemcpyAsync(d_side, sides, n, cudaMemcpyHostToDevice, c.stream));
  APG_CUDA(cudaMemcpyAsync(d_w, w.data(), 32 * nchecks, cudaMemcpyHostToDevice, c.stream));
  APG_CUDA(cudaMemcpyAsync(d_first, first.data(), 8 * nchecks, cudaMemcpyHostToDevice, c.stream));
  const unsigned blocks = (unsigned)((n + 255) / 256);
  launch(c, k_side_scalars, blocks, 256, 0, (const Fr*)d_s, (const uint8_t*)d_side, n, (const uint64_t*)d_first,
         (int)nchecks, (const Fr*)d_w, d_cols, d_cols + n);
  const void* cols[2] = {d_cols, d_cols + n};
  const size_t lens[2] = {n, n};
  uint8_t* d_out = c.scratch[S_RESULT].as<uint8_t>(128);
  msm_multi(c, d_pts, nullptr, cols, lens, 2, false, false, d_out);
  uint8_t* h = static_cast<uint8_t*>(c.host_pinned());
  APG_CUDA(cudaMemcpyAsync(h, d_out, 128, cudaMemcpyDeviceToHost, c.stream));
  c.check_flags();
  memcpy(a_out, h, 64);
  memcpy(b_out, h + 64, 64);
  return APG_OK;
}

}  // namespace apg
