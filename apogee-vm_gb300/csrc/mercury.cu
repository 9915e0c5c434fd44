// Mercury opening (crates/pcs/src/lib.rs:313-492) and the batched opening
// (:688-789) with the O(n) passes and every MSM on the device.
//
// Device: the restriction h (one warp per row of the b x b evaluation
// matrix), the column-parallel fold into q and g, the numerator and its
// division by (X - z) -- both linear recurrences, run as multi-level suffix
// Horner scans -- the size-2b transforms behind S, the batch combination and
// all eight MSMs over the resident SRS. Host: the batch's cm* over a few
// commitments (host_g1.hpp), the transcript and the O(1)
// and O(b) scalar glue of the BDFG20 step (crates/pcs-verify/src/bdfg.rs),
// exactly the reference's formulas.
#include <algorithm>

#include "host_g1.hpp"
#include "host_pairing.hpp"
#include "sumcheck.cuh"

namespace apg {

// Commitments a stacked opening sums on the host (host_g1.hpp) rather than
// through the device MSM.
constexpr size_t kHostMsmMax = 32;

using host::F;

namespace {

Fr dv(const F& a) {
  Fr r;
  memcpy(r.v, a.w, 32);
  return r;
}

// h_j = sum_i eq1[i] * f[j*b + i]: one warp per row.
__global__ void k_row_dot(const Fr* f, const Fr* eq1, size_t b, size_t rows, Fr* h) {
  const size_t warp = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (warp >= rows) return;
  Fr acc = fe_zero<FrConsts>();
  for (size_t i = lane; i < b; i += 32) acc = fe_add(acc, fe_mul(ld_fe(&eq1[i]), ld_fe(&f[warp * b + i])));
  for (int off = 16; off > 0; off >>= 1) {
    Fr o;
#pragma unroll
    for (int w = 0; w < 8; ++w) o.v[w] = __shfl_down_sync(0xffffffffu, acc.v[w], off);
    acc = fe_add(acc, o);
  }
  if (lane == 0) st_fe(&h[warp], acc);
}

// out[0] = sum_i a[i] * b[i] (one block).
__global__ void k_dot(const Fr* a, const Fr* b, size_t n, Fr* out) {
  __shared__ Fr red[256];
  Fr acc = fe_zero<FrConsts>();
  for (size_t i = threadIdx.x; i < n; i += blockDim.x) acc = fe_add(acc, fe_mul(ld_fe(&a[i]), ld_fe(&b[i])));
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if (threadIdx.x < (unsigned)off) red[threadIdx.x] = fe_add(red[threadIdx.x], red[threadIdx.x + off]);
    __syncthreads();
  }
  if (threadIdx.x == 0) st_fe(out, red[0]);
}

// Suffix Horner over `count` positions of `cols` interleaved columns
// (element j of column c at j*stride + c): acc_j = sum_{k>=j} x_k r^(k-j).
// Pass 1: every segment of L positions folds locally from its top and keeps
// its bottom value as the segment's aggregate.
__global__ void k_suffix_local(const Fr* in, Fr* out, size_t stride, size_t count, size_t cols, int L, Fr r,
                               Fr* agg) {
  const size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t nseg = (count + L - 1) / L;
  if (id >= nseg * cols) return;
  const size_t seg = id / cols, col = id % cols;
  const size_t lo = seg * L, hi = min(lo + (size_t)L, count);
  Fr acc = fe_zero<FrConsts>();
  for (size_t j = hi; j-- > lo;) {
    acc = fe_add(ld_fe(&in[j * stride + col]), fe_mul(r, acc));
    st_fe(&out[j * stride + col], acc);
  }
  st_fe(&agg[seg * cols + col], acc);
}

// Pass 2: with upper[s] = acc at the bottom of segment s (the next level's
// result), acc_j = local_j + r^(lo_{s+1} - j) * upper[s+1].
__global__ void k_suffix_fix(Fr* out, size_t stride, size_t count, size_t cols, int L, const Fr* upper,
                             const Fr* pows) {
  const size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (id >= count * cols) return;
  const size_t j = id / cols, col = id % cols;
  const size_t seg = j / L;
  const size_t nseg = (count + L - 1) / L;
  if (seg + 1 >= nseg) return;
  const size_t next = (seg + 1) * L;
  Fr carry = ld_fe(&upper[(seg + 1) * cols + col]);
  Fr* p = &out[j * stride + col];
  st_fe(p, fe_add(ld_fe(p), fe_mul(ld_fe(&pows[next - j]), carry)));
}

// out[i] = base^i.
__global__ void k_powers(Fr base, size_t count, Fr* out) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= count) return;
  Fr acc = fe_one<FrConsts>(), b = base;
  for (size_t e = i; e; e >>= 1) {
    if (e & 1) acc = fe_mul(acc, b);
    b = fe_sqr(b);
  }
  st_fe(&out[i], acc);
}

__global__ void k_bitrev(Fr* a, size_t m, int bits) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= m) return;
  size_t j = __brevll((unsigned long long)i) >> (64 - bits);
  if (i < j) {
    Fr x = ld_fe(&a[i]), y = ld_fe(&a[j]);
    st_fe(&a[i], y);
    st_fe(&a[j], x);
  }
}

// One radix-2 decimation-in-time stage at half-width `half` (the reference's
// butterflies, crates/pcs/src/fft.rs:100-134): tw holds w^k for k < m/2.
__global__ void k_fft_stage(Fr* a, size_t m, size_t half, const Fr* tw) {
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= m / 2) return;
  size_t start = (t / half) * 2 * half, k = t % half;
  Fr w = ld_fe(&tw[k * (m / (2 * half))]);
  Fr lo = ld_fe(&a[start + k]), hi = fe_mul(ld_fe(&a[start + k + half]), w);
  st_fe(&a[start + k], fe_add(lo, hi));
  st_fe(&a[start + k + half], fe_sub(lo, hi));
}

// The four padded operands of S: g, rev(eq1), h, rev(eq2), each b long in 2b.
__global__ void k_sym_pad(const Fr* g, const Fr* eq1, const Fr* h, const Fr* eq2, size_t b, Fr* G, Fr* P1, Fr* H,
                          Fr* P2) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= 2 * b) return;
  const Fr z = fe_zero<FrConsts>();
  st_fe(&G[i], i < b ? ld_fe(&g[i]) : z);
  st_fe(&P1[i], i < b ? ld_fe(&eq1[b - 1 - i]) : z);
  st_fe(&H[i], i < b ? ld_fe(&h[i]) : z);
  st_fe(&P2[i], i < b ? ld_fe(&eq2[b - 1 - i]) : z);
}

__global__ void k_sym_mix(const Fr* G, const Fr* P1, const Fr* H, const Fr* P2, size_t m, Fr gamma, Fr* R) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= m) return;
  Fr a = fe_mul(ld_fe(&G[i]), ld_fe(&P1[i]));
  Fr c = fe_mul(gamma, fe_mul(ld_fe(&H[i]), ld_fe(&P2[i])));
  st_fe(&R[i], fe_add(a, c));
}

__global__ void k_scale(Fr* a, size_t m, Fr s) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < m) st_fe(&a[i], fe_mul(ld_fe(&a[i]), s));
}

// S[k - b] = R[k] + R[2b - 2 - k] for k in [b, 2b - 1); checks R[2b-1] = 0 and
// R[b-1] = h(alpha) + gamma v (symmetric_witness's two assertions).
__global__ void k_sym_out(const Fr* R, size_t b, Fr expect_mid, Fr* S, uint32_t* flags) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i == 0) {
    if (!fe_is_zero(ld_fe(&R[2 * b - 1])) || !fe_eq(ld_fe(&R[b - 1]), expect_mid))
      atomicOr(flags, (uint32_t)DEV_NONZERO_REM);
  }
  if (i >= b - 1) return;
  size_t k = b + i;
  st_fe(&S[i], fe_add(ld_fe(&R[k]), ld_fe(&R[2 * b - 2 - k])));
}

__global__ void k_reverse(const Fr* src, size_t b, Fr* dst) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < b) st_fe(&dst[i], ld_fe(&src[b - 1 - i]));
}

// numerator = f - (z^b - alpha) q - g(z), with q the n - b coefficients.
__global__ void k_numerator(const Fr* f, const Fr* q, size_t n, size_t nq, Fr c, Fr gz, Fr* out) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  Fr v = ld_fe(&f[i]);
  if (i < nq) v = fe_sub(v, fe_mul(c, ld_fe(&q[i])));
  if (i == 0) v = fe_sub(v, gz);
  st_fe(&out[i], v);
}

// f* = sum_j w_j stack_j: stack j's column in slot s (cols[j * maxlen + s],
// null past the stack's end) covers entries [s * 2^width, (s + 1) * 2^width).
__global__ void k_combine_stacked(const Fr* const* cols, const Fr* w, int nstacks, size_t maxlen, int width,
                                  size_t n, Fr* out) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const size_t slot = i >> width, row = i & (((size_t)1 << width) - 1);
  Fr acc = fe_zero<FrConsts>();
  if (slot < maxlen)
    for (int j = 0; j < nstacks; ++j) {
      const Fr* col = cols[(size_t)j * maxlen + slot];
      if (col) acc = fe_add(acc, fe_mul(ld_fe(&w[j]), ld_fe(&col[row])));
    }
  st_fe(&out[i], acc);
}

__global__ void k_expect_zero(const Fr* x, uint32_t* flags) {
  if (!fe_is_zero(ld_fe(x))) atomicOr(flags, (uint32_t)DEV_NONZERO_REM);
}

inline unsigned nb(size_t n, int t) { return (unsigned)((n + t - 1) / t); }

// ---- host helpers -------------------------------------------------------------

F read_fr(Ctx& c, const Fr* d) {
  F x;
  APG_CUDA(cudaMemcpyAsync(x.w, d, 32, cudaMemcpyDeviceToHost, c.stream));
  APG_CUDA(cudaStreamSynchronize(c.stream));
  return x;
}

std::vector<F> read_frs(Ctx& c, const Fr* d, size_t n) {
  std::vector<F> v(n);
  if (n) APG_CUDA(cudaMemcpyAsync(v.data(), d, 32 * n, cudaMemcpyDeviceToHost, c.stream));
  APG_CUDA(cudaStreamSynchronize(c.stream));
  return v;
}

// MSM of the first `len` SRS powers against device scalars, canonical bytes.
void srs_commit(Ctx& c, const Fr* d, size_t len, uint8_t out[64]) {
  if (len == 0) {
    memset(out, 0, 64);
    return;
  }
  const SrsTable* t = srs_table_for(c, len, false);
  if (!t) throw Error(APG_ERR_SRS_TOO_SMALL, "the SRS holds fewer powers than the polynomial has coefficients");
  msm_device(c, nullptr, t, d, false, false, len, nullptr, out);
}

// Two independent SRS MSMs in one group (one sort, accumulation and bucket
// reduction for both).
void srs_commit2(Ctx& c, const Fr* d0, size_t len0, const Fr* d1, size_t len1, uint8_t out0[64],
                 uint8_t out1[64]) {
  if (len0 == 0 || len1 == 0) {
    srs_commit(c, d0, len0, out0);
    srs_commit(c, d1, len1, out1);
    return;
  }
  const SrsTable* t = srs_table_for(c, std::max(len0, len1), false);
  if (!t) throw Error(APG_ERR_SRS_TOO_SMALL, "the SRS holds fewer powers than the polynomial has coefficients");
  const void* ptrs[2] = {d0, d1};
  const size_t lens[2] = {len0, len1};
  uint8_t* d_out = c.scratch[S_RESULT].as<uint8_t>(128);
  msm_multi(c, nullptr, t, ptrs, lens, 2, false, false, d_out);
  uint8_t both[128];
  APG_CUDA(cudaMemcpyAsync(both, d_out, 128, cudaMemcpyDeviceToHost, c.stream));
  c.check_flags();
  memcpy(out0, both, 64);
  memcpy(out1, both + 64, 64);
}

// acc_j = sum_{k >= j} x_k r^(k - j) for every position, in place or not.
void suffix_horner(Ctx& c, const Fr* in, Fr* out, size_t stride, size_t count, size_t cols, const F& r,
                   int depth = 0) {
  if (count == 0) return;
  const int L = 32;
  const size_t nseg = (count + L - 1) / L;
  // Scratch per level: aggregates (nseg x cols) and the power table r^0..r^L,
  // stream-ordered so every recursion level owns its own.
  Fr* agg;
  APG_CUDA(cudaMallocAsync((void**)&agg, 32 * nseg * cols + 32 * (L + 1), c.stream));
  Fr* pows = agg + nseg * cols;
  launch(c, k_powers, 1, L + 1, 0, dv(r), (size_t)(L + 1), pows);
  launch(c, k_suffix_local, nb(nseg * cols, 128), 128, 0, in, out, stride, count, cols, L, dv(r), agg);
  if (nseg > 1) {
    F rL = host::fpow_u64(r, L);
    suffix_horner(c, agg, agg, cols, nseg, cols, rL, depth + 1);
    launch(c, k_suffix_fix, nb(count * cols, 256), 256, 0, out, stride, count, cols, L, (const Fr*)agg,
           (const Fr*)pows);
  }
  APG_CUDA(cudaFreeAsync(agg, c.stream));
}

F two_adic_root() {
  // 5^((p - 1) / 2^28), derived rather than transcribed.
  uint64_t e[4] = {host::kP[0] - 1, host::kP[1], host::kP[2], host::kP[3]};
  for (int s = 0; s < 28; ++s) {
    for (int i = 0; i < 3; ++i) e[i] = (e[i] >> 1) | (e[i + 1] << 63);
    e[3] >>= 1;
  }
  return host::fpow(host::from_u64(5), e);
}

void fft_inplace(Ctx& c, Fr* a, size_t m, const Fr* tw) {
  int bits = 0;
  while (((size_t)1 << bits) < m) ++bits;
  launch(c, k_bitrev, nb(m, 256), 256, 0, a, m, bits);
  for (size_t half = 1; half < m; half *= 2) launch(c, k_fft_stage, nb(m / 2, 256), 256, 0, a, m, half, tw);
}

// ---- univariate helpers on the host (O(b), crates/pcs-verify/src/uni.rs) -------

typedef std::vector<F> Poly;

F ueval(const Poly& p, const F& x) {
  F acc = host::fzero();
  for (size_t i = p.size(); i-- > 0;) acc = host::fadd(host::fmul(acc, x), p[i]);
  return acc;
}

Poly umul(const Poly& a, const Poly& b) {
  if (a.empty() || b.empty()) return {};
  Poly out(a.size() + b.size() - 1, host::fzero());
  for (size_t i = 0; i < a.size(); ++i)
    for (size_t j = 0; j < b.size(); ++j) out[i + j] = host::fadd(out[i + j], host::fmul(a[i], b[j]));
  return out;
}

void uadd_scaled(Poly& acc, const Poly& src, const F& k) {
  if (src.size() > acc.size()) acc.resize(src.size(), host::fzero());
  for (size_t i = 0; i < src.size(); ++i) acc[i] = host::fadd(acc[i], host::fmul(k, src[i]));
}

Poly uvanishing(const std::vector<F>& roots) {
  Poly out{host::fone()};
  for (auto& r : roots) out = umul(out, {host::fneg(r), host::fone()});
  return out;
}

Poly uinterpolate(const std::vector<std::pair<F, F>>& pts) {
  Poly out(pts.size(), host::fzero());
  for (size_t i = 0; i < pts.size(); ++i) {
    Poly num{host::fone()};
    F den = host::fone();
    for (size_t j = 0; j < pts.size(); ++j) {
      if (i == j) continue;
      num = umul(num, {host::fneg(pts[j].first), host::fone()});
      den = host::fmul(den, host::fsub(pts[i].first, pts[j].first));
    }
    uadd_scaled(out, num, host::fmul(pts[i].second, host::finv(den)));
  }
  return out;
}

std::pair<Poly, F> udiv_linear(const Poly& p, const F& r) {
  if (p.empty()) return {{}, host::fzero()};
  Poly q(p.size() - 1);
  F acc = p.back();
  for (size_t i = p.size() - 1; i-- > 0;) {
    q[i] = acc;
    acc = host::fadd(p[i], host::fmul(acc, r));
  }
  return {q, acc};
}

F tensor_eval(const std::vector<F>& u, F x) {
  F acc = host::fone();
  for (auto& uk : u) {
    acc = host::fmul(acc, host::fadd(host::fmul(uk, x), host::fsub(host::fone(), uk)));
    x = host::fsqr(x);
  }
  return acc;
}

}  // namespace

// ---------------------------------------------------------------------------
// The verifier's field side (crates/pcs-verify/src/lib.rs:355-434) and the
// point checks around it (crates/pcs/src/lib.rs:509-548, 586-602): the
// opening's transcript schedule replayed, h(alpha) and D(z) derived, the
// BDFG20 batch at z', and the twelve accumulator entries of a deferred check.
// ---------------------------------------------------------------------------

namespace {

struct Entries {
  uint8_t side[12];
  F scalar[12];
  uint8_t point[12][64];
};

// pcs::accumulate (lib.rs:509-548) with pcs_verify::scalars (:366-434).
// `info` names the refused point: 0..7 the proof's points in field order
// (h, q, g, s, d, pi_z, w, w'), 8 the commitment.
int accumulate(const uint8_t cm[64], const std::vector<F>& u, const F& v, const uint8_t proof[704],
               host::Transcript& tr, Entries& out, uint64_t* info) {
  using namespace host;
  const size_t nv = u.size();
  if (nv < 2 || nv > 54 || nv % 2) return APG_ERR_UNSUPPORTED_NUM_VARS;
  for (int i = 0; i < 8; ++i)
    if (!host::g1::valid_encoding(proof + 64 * i)) {
      if (info) *info = (uint64_t)i;
      return APG_ERR_INVALID_POINT;
    }
  if (!host::g1::valid_encoding(cm)) {
    if (info) *info = 8;
    return APG_ERR_INVALID_POINT;
  }
  F ev[6];
  for (int i = 0; i < 6; ++i)
    if (!from_bytes(proof + 512 + 32 * i, ev[i])) return APG_ERR_NONCANONICAL;
  const size_t t = nv / 2, b = (size_t)1 << t;
  const std::vector<F> u1(u.begin(), u.begin() + t), u2(u.begin() + t, u.end());
  const uint8_t* pt[8];
  for (int i = 0; i < 8; ++i) pt[i] = proof + 64 * i;

  // The opening's schedule, step for step.
  tr.absorb(T_MERCURY_INSTANCE, std::vector<F>{from_u64((uint64_t)1 << nv)});
  tr.absorb_g1(T_COMMITMENT, cm, 1);
  std::vector<F> claim = u;
  claim.push_back(v);
  tr.absorb(T_EVALUATION_CLAIM, claim);
  tr.absorb_g1(T_PCS_OPENING, pt[0], 1);
  const F alpha = tr.challenge(T_MERCURY_ALPHA);
  tr.absorb_g1(T_PCS_OPENING, pt[1], 2);
  const F gamma = tr.challenge(T_MERCURY_GAMMA);
  tr.absorb_g1(T_PCS_OPENING, pt[3], 2);
  F z;
  do {
    z = tr.challenge(T_MERCURY_Z);
  } while (z.zero());
  if (fsqr(z) == fone() || z == alpha || fmul(z, alpha) == fone()) return APG_ERR_DEGENERATE_CHALLENGE;
  const F zi = finv(z);
  tr.absorb(T_PCS_OPENING, ev, 6);
  tr.absorb_g1(T_PCS_OPENING, pt[5], 1);
  const F delta = tr.challenge(T_BDFG_BATCH);
  tr.absorb_g1(T_PCS_OPENING, pt[6], 1);
  const F zp = tr.challenge(T_BDFG_POINT);
  tr.absorb_g1(T_PCS_OPENING, pt[7], 1);
  const F rho = tr.challenge(T_PAIRING_MERGE);

  // h(alpha) from the symmetrized identity at z (derive_h_alpha, :205-227)
  // and D(z) = z^(b-1) g(1/z).
  F inner = fadd(fadd(fmul(ev[0], tensor_eval(u1, zi)), fmul(ev[1], tensor_eval(u1, z))),
                 fmul(gamma, fsub(fsub(fadd(fmul(ev[2], tensor_eval(u2, zi)), fmul(ev[3], tensor_eval(u2, z))), v), v)));
  inner = fsub(fsub(inner, fmul(z, ev[4])), fmul(zi, ev[5]));
  const F h_alpha = fmul(inner, finv(from_u64(2)));
  const F d_z = fmul(fpow_u64(z, b - 1), ev[1]);
  // The BDFG20 batch at z' (bdfg::items, crates/pcs-verify/src/bdfg.rs):
  // c_i = delta^i Z_{T minus S_i}(z'), constant = sum_i c_i r_i(z').
  const Poly wa = uvanishing({alpha});
  const Poly zc[4] = {wa, Poly{fone()}, wa, uvanishing({zi, alpha})};
  const Poly rr[4] = {uinterpolate({{z, ev[0]}, {zi, ev[1]}}),
                      uinterpolate({{z, ev[2]}, {zi, ev[3]}, {alpha, h_alpha}}),
                      uinterpolate({{z, ev[4]}, {zi, ev[5]}}), Poly{d_z}};
  F c[4], constant = fzero(), dp = fone();
  for (int i = 0; i < 4; ++i) {
    c[i] = fmul(dp, ueval(zc[i], zp));
    constant = fadd(constant, fmul(c[i], ueval(rr[i], zp)));
    dp = fmul(dp, delta);
  }
  const F z_t = ueval(uvanishing({z, zi, alpha}), zp);
  const F z_pow_b = fpow_u64(z, b);
  // Check A (the fold identity at z) plus rho times check B (the batch).
  const F sc[12] = {fone(),
                    fmul(rho, c[1]),
                    fneg(fsub(z_pow_b, alpha)),
                    fmul(rho, c[0]),
                    fmul(rho, c[2]),
                    fmul(rho, c[3]),
                    z,
                    fneg(fmul(rho, z_t)),
                    fmul(rho, zp),
                    fneg(fadd(ev[0], fmul(rho, constant))),
                    fone(),
                    rho};
  // ENTRY_POINTS (:271-284): the points [cm, h, q, g, s, d, pi_z, w, w',
  // [1]_1], ten on the [1]_2 side, then pi_z and w' on the [x]_2 side.
  uint8_t gen[64] = {0};
  gen[0] = 1;
  gen[32] = 2;
  const uint8_t* at[10] = {cm, pt[0], pt[1], pt[2], pt[3], pt[4], pt[5], pt[6], pt[7], gen};
  const int idx[12] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 6, 8};
  for (int i = 0; i < 12; ++i) {
    out.side[i] = i < 10 ? 0 : 1;
    out.scalar[i] = sc[i];
    memcpy(out.point[i], at[idx[i]], 64);
  }
  return APG_OK;
}

void write_entries(const Entries& e, uint8_t* sides, uint8_t* scalars, uint8_t* points) {
  memcpy(sides, e.side, 12);
  memcpy(scalars, e.scalar, 12 * 32);
  memcpy(points, e.point, 12 * 64);
}

bool read_frs_mem(const uint8_t* p, size_t n, std::vector<F>& out) {
  out.resize(n);
  for (size_t i = 0; i < n; ++i) {
    memcpy(out[i].w, p + 32 * i, 32);
    if (!host::below_p(out[i].w)) return false;
  }
  return true;
}

}  // namespace

// pcs::verify_deferred (crates/pcs/src/lib.rs:632-641).
int mercury_verify_deferred_impl(const uint8_t cm[64], const uint8_t* u, size_t u_len, const uint8_t v[32],
                                 const uint8_t proof[704], uint8_t* transcript, uint8_t* sides, uint8_t* scalars,
                                 uint8_t* points, uint64_t* info) {
  if (info) *info = 0;
  if (!cm || (u_len && !u) || !v || !proof || !transcript || !sides || !scalars || !points)
    return APG_ERR_INVALID_ARGUMENT;
  std::vector<F> uu, vv;
  if (!read_frs_mem(u, u_len, uu) || !read_frs_mem(v, 1, vv)) return APG_ERR_NONCANONICAL;
  host::Transcript tr;
  if (!tr.load(transcript)) return APG_ERR_INVALID_ARGUMENT;
  Entries e;
  const int st = accumulate(cm, uu, vv[0], proof, tr, e, info);
  if (st) return st;
  write_entries(e, sides, scalars, points);
  tr.save(transcript);
  return APG_OK;
}

// pcs::batch_verify_deferred (crates/pcs/src/lib.rs:661-670) through
// batch_accumulate (:586-602): check_batch, every commitment validated, the
// preamble (the commitments as passed, u || vs, rho), cm* = sum rho^i cm_i
// and v* = sum rho^i v_i, then the single-instance core.
int mercury_batch_verify_deferred_impl(const uint8_t* cms, size_t k, const uint8_t* u, size_t u_len,
                                       const uint8_t* vs, size_t n_vs, const uint8_t proof[704], uint8_t* transcript,
                                       uint8_t* sides, uint8_t* scalars, uint8_t* points, uint64_t* info) {
  using namespace host;
  if (info) *info = 0;
  if ((k && !cms) || (u_len && !u) || (n_vs && !vs) || !proof || !transcript || !sides || !scalars || !points)
    return APG_ERR_INVALID_ARGUMENT;
  if (k == 0) return APG_ERR_EMPTY_BATCH;
  if (k != n_vs) return APG_ERR_BATCH_LENGTH_MISMATCH;
  if (u_len < 2 || u_len > 54 || u_len % 2) return APG_ERR_UNSUPPORTED_NUM_VARS;
  for (size_t j = 0; j < k; ++j)
    if (!host::g1::valid_encoding(cms + 64 * j)) {
      if (info) *info = 8;
      return APG_ERR_INVALID_POINT;
    }
  std::vector<F> uu, vals;
  if (!read_frs_mem(u, u_len, uu) || !read_frs_mem(vs, n_vs, vals)) return APG_ERR_NONCANONICAL;
  Transcript tr;
  if (!tr.load(transcript)) return APG_ERR_INVALID_ARGUMENT;
  // pcs_verify::batch_preamble (:333-347).
  tr.absorb_g1(T_COMMITMENT, cms, k);
  std::vector<F> claim = uu;
  claim.insert(claim.end(), vals.begin(), vals.end());
  tr.absorb(T_EVALUATION_CLAIM, claim);
  const F rho = tr.challenge(T_MERCURY_BATCH);
  std::vector<F> wts(k);
  F acc = fone(), vstar = fzero();
  for (size_t i = 0; i < k; ++i) {
    wts[i] = acc;
    vstar = fadd(vstar, fmul(acc, vals[i]));
    acc = fmul(acc, rho);
  }
  uint8_t cm_star[64];
  host::g1::msm_small(cms, wts.data(), k, cm_star);
  Entries e;
  const int st = accumulate(cm_star, uu, vstar, proof, tr, e, info);
  if (st) return st;
  write_entries(e, sides, scalars, points);
  tr.save(transcript);
  return APG_OK;
}


// ---------------------------------------------------------------------------
// The pairing step (crates/curve/src/pairing.rs, crates/pcs/src/accumulator.rs
// check_pairings :171-214): e(A, [1]_2) e(-B, [x]_2) == 1 with A and B the
// weighted sums of the entries on each side, over the verifier's SRS points
// (SrsVerifier, crates/srs/src/lib.rs:279-283: [1]_1 || [1]_2 || [x]_2).
// ---------------------------------------------------------------------------

namespace {

struct Vsrs {
  host::pairing::G2 g2_gen, g2_tau;
};

int read_vsrs(const uint8_t vsrs[320], Vsrs& out) {
  if (!host::g1::valid_encoding(vsrs)) return APG_ERR_INVALID_POINT;
  if (!host::pairing::g2from_bytes(vsrs + 64, out.g2_gen) || !host::pairing::g2from_bytes(vsrs + 192, out.g2_tau))
    return APG_ERR_INVALID_POINT;
  return APG_OK;
}

// -P for a canonical encoding (infinity stays infinity).
void g1_negate(const uint8_t p[64], uint8_t out[64]) {
  memcpy(out, p, 64);
  bool inf = true;
  for (int i = 0; i < 64; ++i) inf &= p[i] == 0;
  if (inf) return;
  uint64_t y[4];
  memcpy(y, p + 32, 32);
  if ((y[0] | y[1] | y[2] | y[3]) == 0) return;
  uint64_t br = 0;
  for (int i = 0; i < 4; ++i) {
    const host::u128 d = (host::u128)host::g1::kQ[i] - y[i] - br;
    y[i] = (uint64_t)d;
    br = (uint64_t)(d >> 127);
  }
  memcpy(out + 32, y, 32);
}

bool pairings_hold(const Vsrs& vk, const uint8_t a[64], const uint8_t b[64]) {
  uint8_t nb[64];
  g1_negate(b, nb);
  return host::pairing::pairing_check({a, nb}, {vk.g2_gen, vk.g2_tau});
}

// One deferred check with weight one: A and B summed on the host.
int check_entries(const Vsrs& vk, const Entries& e) {
  std::vector<uint8_t> pa, pb;
  std::vector<F> sa, sb;
  for (int i = 0; i < 12; ++i) {
    auto& pts = e.side[i] ? pb : pa;
    pts.insert(pts.end(), e.point[i], e.point[i] + 64);
    (e.side[i] ? sb : sa).push_back(e.scalar[i]);
  }
  uint8_t a[64], b[64];
  host::g1::msm_small(pa.data(), sa.data(), sa.size(), a);
  host::g1::msm_small(pb.data(), sb.data(), sb.size(), b);
  return pairings_hold(vk, a, b) ? APG_OK : APG_ERR_VERIFICATION_FAILED;
}

}  // namespace

int pairing_impl(const uint8_t p[64], const uint8_t q[128], uint8_t out[384]) {
  if (!p || !q || !out) return APG_ERR_INVALID_ARGUMENT;
  host::pairing::G2 qq;
  if (!host::g1::valid_encoding(p) || !host::pairing::g2from_bytes(q, qq)) return APG_ERR_INVALID_POINT;
  host::g1::Q x, y;
  bool inf;
  host::pairing::g1_affine(p, x, y, inf);
  host::pairing::f12to_bytes(host::pairing::final_exponentiation(host::pairing::miller_loop(x, y, inf, qq)), out);
  return APG_OK;
}

int g2_mul_impl(const uint8_t q[128], const uint8_t k[32], uint8_t out[128]) {
  if (!q || !k || !out) return APG_ERR_INVALID_ARGUMENT;
  host::pairing::G2 qq;
  if (!host::pairing::g2from_bytes(q, qq)) return APG_ERR_INVALID_POINT;
  host::pairing::Big kb(4);
  memcpy(kb.data(), k, 32);
  host::pairing::big_trim(kb);
  host::pairing::g2to_bytes(host::pairing::g2mul(qq, kb), out);
  return APG_OK;
}

int pairing_check_impl(const uint8_t* ps, const uint8_t* qs, size_t n, int* holds) {
  if ((n && (!ps || !qs)) || !holds) return APG_ERR_INVALID_ARGUMENT;
  std::vector<const uint8_t*> pp(n);
  std::vector<host::pairing::G2> qq(n);
  for (size_t i = 0; i < n; ++i) {
    pp[i] = ps + 64 * i;
    if (!host::g1::valid_encoding(pp[i]) || !host::pairing::g2from_bytes(qs + 128 * i, qq[i]))
      return APG_ERR_INVALID_POINT;
  }
  *holds = host::pairing::pairing_check(pp, qq) ? 1 : 0;
  return APG_OK;
}

// pcs::verify (crates/pcs/src/lib.rs:614-628): the deferred check, then its
// pairing.
int mercury_verify_impl(const uint8_t vsrs[320], const uint8_t cm[64], const uint8_t* u, size_t u_len,
                        const uint8_t v[32], const uint8_t proof[704], uint8_t* transcript, uint64_t* info) {
  if (!vsrs) return APG_ERR_INVALID_ARGUMENT;
  uint8_t snap[226], sides[12], scalars[12 * 32], points[12 * 64];
  if (!transcript) return APG_ERR_INVALID_ARGUMENT;
  memcpy(snap, transcript, 226);
  int st = mercury_verify_deferred_impl(cm, u, u_len, v, proof, snap, sides, scalars, points, info);
  if (st) return st;
  Vsrs vk;
  if ((st = read_vsrs(vsrs, vk))) return st;
  Entries e;
  memcpy(e.side, sides, 12);
  memcpy(e.scalar, scalars, sizeof(scalars));
  memcpy(e.point, points, sizeof(points));
  if ((st = check_entries(vk, e))) return st;
  memcpy(transcript, snap, 226);
  return APG_OK;
}

// pcs::batch_verify (lib.rs:648-658).
int mercury_batch_verify_impl(const uint8_t vsrs[320], const uint8_t* cms, size_t k, const uint8_t* u, size_t u_len,
                              const uint8_t* vs, size_t n_vs, const uint8_t proof[704], uint8_t* transcript,
                              uint64_t* info) {
  if (!vsrs || !transcript) return APG_ERR_INVALID_ARGUMENT;
  uint8_t snap[226], sides[12], scalars[12 * 32], points[12 * 64];
  memcpy(snap, transcript, 226);
  int st = mercury_batch_verify_deferred_impl(cms, k, u, u_len, vs, n_vs, proof, snap, sides, scalars, points, info);
  if (st) return st;
  Vsrs vk;
  if ((st = read_vsrs(vsrs, vk))) return st;
  Entries e;
  memcpy(e.side, sides, 12);
  memcpy(e.scalar, scalars, sizeof(scalars));
  memcpy(e.point, points, sizeof(points));
  if ((st = check_entries(vk, e))) return st;
  memcpy(transcript, snap, 226);
  return APG_OK;
}

// The pairing step of pcs::discharge (accumulator.rs:146-163) over the A and B
// its MSMs produced (apg_discharge_msms).
int discharge_pairing_impl(const uint8_t vsrs[320], const uint8_t a[64], const uint8_t b[64]) {
  if (!vsrs || !a || !b) return APG_ERR_INVALID_ARGUMENT;
  Vsrs vk;
  const int st = read_vsrs(vsrs, vk);
  if (st) return st;
  return pairings_hold(vk, a, b) ? APG_OK : APG_ERR_VERIFICATION_FAILED;
}

// ---------------------------------------------------------------------------

int mercury_open_impl(Ctx& c, const Fr* d_f, size_t nv, const uint8_t cm[64], const std::vector<F>& u,
                      host::Transcript& tr, F& v_out, uint8_t proof_out[704]) {
  using namespace host;
  if (nv < 2 || nv > 54 || nv % 2) return APG_ERR_UNSUPPORTED_NUM_VARS;
  if (u.size() != nv) return APG_ERR_POINT_LENGTH_MISMATCH;
  if (!c.srs) return APG_ERR_NO_SRS;
  const size_t n = (size_t)1 << nv;
  if (c.srs_n < n) return APG_ERR_SRS_TOO_SMALL;
  if (nv > 40) return APG_ERR_OUT_OF_MEMORY;
  const size_t t = nv / 2, b = (size_t)1 << t;
  std::vector<F> u1(u.begin(), u.begin() + t), u2(u.begin() + t, u.end());

  Fr* work;
  // eq1 | eq2 | h | g | S | D | acc(n) | num(n) | 4 x (2b) transforms | twiddles
  const size_t words = 6 * b + 2 * n + 8 * b + b + 16;
  APG_CUDA(cudaMallocAsync((void**)&work, 32 * words, c.stream));
  struct Guard {
    Ctx& c;
    Fr* p;
    ~Guard() { cudaFreeAsync(p, c.stream); }
  } guard{c, work};
  Fr *eq1 = work, *eq2 = eq1 + b, *h = eq2 + b, *g = h + b, *S = g + b, *D = S + b, *acc = D + b, *num = acc + n;
  Fr *TG = num + n, *TP1 = TG + 2 * b, *TH = TP1 + 2 * b, *TP2 = TH + 2 * b, *tw = TP2 + 2 * b, *tmp = tw + b;

  // Step 1: h, v.
  build_eq_table(c, u1, eq1);
  build_eq_table(c, u2, eq2);
  launch(c, k_row_dot, nb(b * 32, 256), 256, 0, d_f, (const Fr*)eq1, b, b, h);
  launch(c, k_dot, 1, 256, 0, (const Fr*)eq2, (const Fr*)h, b, tmp);
  F v = read_fr(c, tmp);
  uint8_t pts[8][64];
  srs_commit(c, h, b, pts[0]);
  tr.absorb(T_MERCURY_INSTANCE, std::vector<F>{from_u64(n)});
  tr.absorb_g1(T_COMMITMENT, cm, 1);
  std::vector<F> claim = u;
  claim.push_back(v);
  tr.absorb(T_EVALUATION_CLAIM, claim);
  tr.absorb_g1(T_PCS_OPENING, pts[0], 1);
  F alpha = tr.challenge(T_MERCURY_ALPHA);

  // Step 2: the fold. acc rows: acc_j = sum_{k>=j} alpha^(k-j) row_k; q is
  // rows 1..b-1 of acc, g is row 0.
  cudaEvent_t tp = c.timer_begin();
  suffix_horner(c, d_f, acc, b, b, b, alpha);
  c.timer_end(APG_TIMER_MERCURY_PASS, tp);
  APG_CUDA(cudaMemcpyAsync(g, acc, 32 * b, cudaMemcpyDeviceToDevice, c.stream));
  const Fr* q = acc + b;
  const size_t nq = n - b;
  srs_commit2(c, q, nq, g, b, pts[1], pts[2]);
  tr.absorb_g1(T_PCS_OPENING, &pts[1][0], 2);
  F gamma = tr.challenge(T_MERCURY_GAMMA);

  // Step 3: S and D.
  std::vector<F> hh = read_frs(c, h, b);
  F h_alpha = ueval(hh, alpha);
  {
    const size_t m = 2 * b;
    int k = 0;
    while (((size_t)1 << k) < m) ++k;
    F w = two_adic_root();
    for (int i = k; i < 28; ++i) w = fsqr(w);
    launch(c, k_sym_pad, nb(m, 256), 256, 0, (const Fr*)g, (const Fr*)eq1, (const Fr*)h, (const Fr*)eq2, b, TG, TP1,
           TH, TP2);
    launch(c, k_powers, nb(m / 2, 256), 256, 0, dv(w), m / 2, tw);
    fft_inplace(c, TG, m, tw);
    fft_inplace(c, TP1, m, tw);
    fft_inplace(c, TH, m, tw);
    fft_inplace(c, TP2, m, tw);
    launch(c, k_sym_mix, nb(m, 256), 256, 0, (const Fr*)TG, (const Fr*)TP1, (const Fr*)TH, (const Fr*)TP2, m,
           dv(gamma), TG);
    launch(c, k_powers, nb(m / 2, 256), 256, 0, dv(finv(w)), m / 2, tw);
    fft_inplace(c, TG, m, tw);
    launch(c, k_scale, nb(m, 256), 256, 0, TG, m, dv(finv(from_u64(m))));
    launch(c, k_sym_out, nb(b, 256), 256, 0, (const Fr*)TG, b, dv(fadd(h_alpha, fmul(gamma, v))), S, c.d_flags);
    launch(c, k_reverse, nb(b, 256), 256, 0, (const Fr*)g, b, D);
  }
  srs_commit2(c, S, b - 1, D, b, pts[3], pts[4]);
  tr.absorb_g1(T_PCS_OPENING, &pts[3][0], 2);
  F z;
  do {
    z = tr.challenge(T_MERCURY_Z);
  } while (z.zero());
  if (fsqr(z) == fone() || z == alpha || fmul(z, alpha) == fone()) {
    c.last_error = "degenerate challenge set {z, 1/z, alpha}";
    return APG_ERR_DEGENERATE_CHALLENGE;
  }
  F zi = finv(z);

  // Step 4: the six values, the numerator and its quotient by (X - z).
  std::vector<F> gg = read_frs(c, g, b), ss = read_frs(c, S, b - 1);
  F ev[6] = {ueval(gg, z), ueval(gg, zi), ueval(hh, z), ueval(hh, zi), ueval(ss, z), ueval(ss, zi)};
  tr.absorb(T_PCS_OPENING, ev, 6);
  F zb = fpow_u64(z, b);
  launch(c, k_numerator, nb(n, 256), 256, 0, d_f, q, n, nq, dv(fsub(zb, alpha)), dv(ev[0]), num);
  tp = c.timer_begin();
  suffix_horner(c, num, num, 1, n, 1, z);
  c.timer_end(APG_TIMER_MERCURY_PASS, tp);
  launch(c, k_expect_zero, 1, 1, 0, (const Fr*)num, c.d_flags);  // the remainder f(z) - ... = 0
  srs_commit(c, num + 1, n - 1, pts[5]);
  tr.absorb_g1(T_PCS_OPENING, pts[5], 1);

  // Step 4(e): BDFG20 over T = {z, 1/z, alpha} (crates/pcs-verify/src/bdfg.rs).
  F two_inv = finv(from_u64(2));
  F inner = fadd(fadd(fmul(ev[0], tensor_eval(u1, zi)), fmul(ev[1], tensor_eval(u1, z))),
                 fmul(gamma, fsub(fsub(fadd(fmul(ev[2], tensor_eval(u2, zi)), fmul(ev[3], tensor_eval(u2, z))), v), v)));
  inner = fsub(fsub(inner, fmul(z, ev[4])), fmul(zi, ev[5]));
  F ha = fmul(inner, two_inv);
  if (ha != h_alpha) throw Error(APG_ERR_INTERNAL, "h(alpha) does not re-derive from the six values");
  F d_z = fmul(fpow_u64(z, b - 1), ev[1]);
  std::vector<F> tset = {z, zi, alpha};
  Poly wa = uvanishing({alpha});
  Poly zc[4] = {wa, Poly{fone()}, wa, uvanishing({zi, alpha})};
  Poly rr[4] = {uinterpolate({{z, ev[0]}, {zi, ev[1]}}), uinterpolate({{z, ev[2]}, {zi, ev[3]}, {alpha, h_alpha}}),
                uinterpolate({{z, ev[4]}, {zi, ev[5]}}), Poly{d_z}};
  Poly dd(gg.rbegin(), gg.rend());
  const Poly* polys[4] = {&gg, &hh, &ss, &dd};
  F delta = tr.challenge(T_BDFG_BATCH);
  Poly f;
  F pw = fone();
  for (int i = 0; i < 4; ++i) {
    Poly sh = *polys[i];
    uadd_scaled(sh, rr[i], fneg(fone()));
    uadd_scaled(f, umul(zc[i], sh), pw);
    pw = fmul(pw, delta);
  }
  Poly W = f;
  for (auto& root : tset) {
    auto d = udiv_linear(W, root);
    if (!d.second.zero()) throw Error(APG_ERR_INTERNAL, "F is not divisible by Z_T");
    W = d.first;
  }
  Fr* dW = TH;  // reuse a transform buffer (2b >= |W|)
  APG_CUDA(cudaMemcpyAsync(dW, W.data(), 32 * W.size(), cudaMemcpyHostToDevice, c.stream));
  srs_commit(c, dW, W.size(), pts[6]);
  tr.absorb_g1(T_PCS_OPENING, pts[6], 1);
  F zp = tr.challenge(T_BDFG_POINT);
  Poly Lp;
  F cst = fzero();
  uadd_scaled(Lp, W, fneg(ueval(uvanishing(tset), zp)));
  for (int i = 0; i < 4; ++i) {
    F cc = fmul(fpow_u64(delta, i), ueval(zc[i], zp));
    uadd_scaled(Lp, *polys[i], cc);
    cst = fadd(cst, fmul(cc, ueval(rr[i], zp)));
  }
  if (Lp.empty()) Lp.push_back(fzero());
  Lp[0] = fsub(Lp[0], cst);
  auto wp = udiv_linear(Lp, zp);
  if (!wp.second.zero()) throw Error(APG_ERR_INTERNAL, "the linearization does not vanish at z'");
  Fr* dWp = TP2;
  APG_CUDA(cudaMemcpyAsync(dWp, wp.first.data(), 32 * wp.first.size(), cudaMemcpyHostToDevice, c.stream));
  srs_commit(c, dWp, wp.first.size(), pts[7]);
  tr.absorb_g1(T_PCS_OPENING, pts[7], 1);
  (void)tr.challenge(T_PAIRING_MERGE);
  c.check_flags();

  v_out = v;
  for (int i = 0; i < 8; ++i) memcpy(proof_out + 64 * i, pts[i], 64);
  for (int i = 0; i < 6; ++i) to_bytes(ev[i], proof_out + 512 + 32 * i);
  return APG_OK;
}

// batch_open_stacked (crates/pcs/src/lib.rs:705-789) past its refusals, which
// the caller has checked: stack j's columns (d_cols, stack after stack, each
// 2^width entries on the device) fill its first stack_lens[j] slots of a
// (width + |r|)-variable table. Each column's value at u comes from one row
// dot against eq(u_lo) and one dot against eq(u_hi); v_j = sum_s eq(r, s) *
// col_{j,s}(u); the preamble absorbs the commitments, u || r and the values
// and draws rho (:568-581); cm* = sum_j rho^j cm_j is a generic-base MSM and
// f* = sum_j rho^j stack_j is opened at u || r. batch_open is r = [] with one
// column a stack.
int mercury_batch_open_stacked_impl(Ctx& c, const Fr* const* d_cols, const size_t* stack_lens, size_t nstacks,
                                    size_t width, const uint8_t* cms, const std::vector<F>& u,
                                    const std::vector<F>& r, host::Transcript& tr, std::vector<F>& vs,
                                    uint8_t proof_out[704]) {
  using namespace host;
  const size_t nv = width + r.size();
  const size_t n = (size_t)1 << nv;
  size_t ncols = 0, maxlen = 0;
  for (size_t j = 0; j < nstacks; ++j) {
    ncols += stack_lens[j];
    maxlen = std::max(maxlen, stack_lens[j]);
  }
  const size_t w1 = width / 2, b1 = (size_t)1 << w1, b2 = (size_t)1 << (width - w1);
  std::vector<F> u1(u.begin(), u.begin() + w1), u2(u.begin() + w1, u.end());
  Fr* work;
  const size_t words = b1 + 2 * b2 + ncols + nstacks + n;
  APG_CUDA(cudaMallocAsync((void**)&work, 32 * words, c.stream));
  struct Guard {
    Ctx& c;
    Fr* p;
    ~Guard() { cudaFreeAsync(p, c.stream); }
  } guard{c, work};
  Fr *eq1 = work, *eq2 = eq1 + b1, *h = eq2 + b2, *cv = h + b2, *w = cv + ncols, *fstar = w + nstacks;
  build_eq_table(c, u1, eq1);
  build_eq_table(c, u2, eq2);
  for (size_t col = 0; col < ncols; ++col) {
    launch(c, k_row_dot, nb(b2 * 32, 256), 256, 0, d_cols[col], (const Fr*)eq1, b1, b2, h);
    launch(c, k_dot, 1, 256, 0, (const Fr*)eq2, (const Fr*)h, b2, cv + col);
  }
  const std::vector<F> vals = read_frs(c, cv, ncols);
  vs.assign(nstacks, fzero());
  for (size_t j = 0, idx = 0; j < nstacks; ++j)
    for (size_t s = 0; s < stack_lens[j]; ++s, ++idx) {
      F e = fone();  // eq(r, s): variable i is bit i of the slot
      for (size_t i = 0; i < r.size(); ++i) e = fmul(e, (s >> i) & 1 ? r[i] : fsub(fone(), r[i]));
      vs[j] = fadd(vs[j], fmul(e, vals[idx]));
    }
  std::vector<F> point = u;
  point.insert(point.end(), r.begin(), r.end());
  tr.absorb_g1(T_COMMITMENT, cms, nstacks);
  std::vector<F> claim = point;
  claim.insert(claim.end(), vs.begin(), vs.end());
  tr.absorb(T_EVALUATION_CLAIM, claim);
  F rho = tr.challenge(T_MERCURY_BATCH);
  std::vector<F> wts(nstacks);
  F acc = fone();
  for (size_t i = 0; i < nstacks; ++i) {
    wts[i] = acc;
    acc = fmul(acc, rho);
  }
  // cm* = sum rho^j cm_j (crates/pcs/src/lib.rs:568-581). The commitments
  // are validated on their way to the device (status codes of the general
  // MSM); a few of them are summed on the host, where the sum's chain of 252
  // doublings runs many times faster than in one device thread (eight
  // commitments: about 0.2 ms against 2.2 ms), more through the device MSM.
  Affine* d_cms = c.scratch[S_BASES].as<Affine>(nstacks);
  upload_points(c, cms, nstacks, d_cms);
  APG_CUDA(cudaMemcpyAsync(w, wts.data(), 32 * nstacks, cudaMemcpyHostToDevice, c.stream));
  uint8_t cm_star[64];
  if (nstacks <= kHostMsmMax)
    host::g1::msm_small(cms, wts.data(), nstacks, cm_star);
  else
    msm_device(c, d_cms, nullptr, w, false, false, nstacks, nullptr, cm_star);
  std::vector<const Fr*> table(nstacks * maxlen, nullptr);
  for (size_t j = 0, idx = 0; j < nstacks; ++j)
    for (size_t s = 0; s < stack_lens[j]; ++s) table[j * maxlen + s] = d_cols[idx++];
  const Fr** d_table = c.scratch[S_TMP5].as<const Fr*>(table.size());
  APG_CUDA(cudaMemcpyAsync(d_table, table.data(), sizeof(Fr*) * table.size(), cudaMemcpyHostToDevice, c.stream));
  launch(c, k_combine_stacked, nb(n, 256), 256, 0, (const Fr* const*)d_table, (const Fr*)w, (int)nstacks, maxlen,
         (int)width, n, fstar);
  F v;
  int st = mercury_open_impl(c, fstar, nv, cm_star, point, tr, v, proof_out);
  if (st) return st;
  F vstar = fzero();
  for (size_t i = 0; i < nstacks; ++i) vstar = fadd(vstar, fmul(wts[i], vs[i]));
  if (v != vstar) throw Error(APG_ERR_INTERNAL, "the combined value is not the combination of the values");
  return APG_OK;
}

}  // namespace apg
