// ORACLE — test infrastructure only. CPU restatement of the reference's
// Mercury commitment and opening (crates/pcs, crates/pcs-verify), used by
// tests/ to check the CUDA library's proofs byte for byte.
//
//  * commit (crates/pcs/src/lib.rs:237-247), open (:313-492), batch_preamble
//    (:568-581 and crates/pcs-verify/src/lib.rs:333), batch_open and
//    batch_open_stacked (:688-789), symmetric_witness (:812-864).
//  * fft::Domain (crates/pcs/src/fft.rs:37-134); uni::{eval, div_by_linear,
//    mul, add_scaled, vanishing, interpolate, pow_usize}
//    (crates/pcs-verify/src/uni.rs:18-116); bdfg::{items, quotient,
//    linearization} (crates/pcs-verify/src/bdfg.rs:67-142); check_num_vars,
//    challenge_z, degenerate, tensor_eval, derive_h_alpha
//    (crates/pcs-verify/src/lib.rs:97-241).
#pragma once
#include "curve.hpp"
#include "prover.hpp"

namespace oracle {

typedef std::array<uint8_t, 64> G1Bytes;

inline G1Bytes g1_bytes(const G1Jac& p) {
  G1Bytes b;
  p.to_affine().to_bytes(b.data());
  return b;
}

struct Srs {
  std::vector<G1Affine> g1;
};

// [tau^i]G for i < count, by the 4-bit ladder on G (the reference's toy SRS,
// crates/pcs/tests/common/mod.rs:41-60).
inline Srs toy_srs(const Fr& tau, size_t count, size_t threads) {
  std::vector<Fr> sc(count);
  Fr acc = Fr::one();
  for (size_t i = 0; i < count; ++i) {
    sc[i] = acc;
    acc *= tau;
  }
  // Fixed-base comb: comb[8j + ...] holds d * 2^(8j) G for every byte value d,
  // so [s]G is 32 mixed additions (the points are the recipe's; only the
  // arithmetic that reaches them is faster than a scalar multiplication each).
  std::vector<G1Jac> cj(32 * 256);
  G1Jac base = G1Jac::from(G1Affine::generator());
  for (int j = 0; j < 32; ++j) {
    cj[256 * j] = G1Jac::identity();
    for (int d = 1; d < 256; ++d) cj[256 * j + d] = cj[256 * j + d - 1].add(base);
    base = cj[256 * j + 255].add(base);  // 256 * 2^(8j) G
  }
  std::vector<G1Affine> comb = batch_to_affine(cj);
  std::vector<G1Jac> pj(count);
  std::vector<std::thread> pool;
  for (size_t t = 0; t < threads; ++t)
    pool.emplace_back([&, t] {
      uint8_t b[32];
      for (size_t i = t; i < count; i += threads) {
        sc[i].to_bytes(b);
        G1Jac acc = G1Jac::identity();
        for (int j = 0; j < 32; ++j)
          if (b[j]) acc = acc.add_affine(comb[256 * j + b[j]]);
        pj[i] = acc;
      }
    });
  for (auto& th : pool) th.join();
  return Srs{batch_to_affine(pj)};
}

// --- uni -------------------------------------------------------------------
namespace uni {
inline Fr eval(const std::vector<Fr>& c, const Fr& x) {
  Fr acc = Fr::zero();
  for (size_t i = c.size(); i-- > 0;) acc = acc * x + c[i];
  return acc;
}
inline std::pair<std::vector<Fr>, Fr> div_by_linear(const std::vector<Fr>& c, const Fr& r) {
  if (c.empty()) return {{}, Fr::zero()};
  std::vector<Fr> q(c.size() - 1);
  Fr acc = c.back();
  for (size_t i = c.size() - 1; i-- > 0;) {
    q[i] = acc;
    acc = c[i] + acc * r;
  }
  return {q, acc};
}
inline std::vector<Fr> mul(const std::vector<Fr>& a, const std::vector<Fr>& b) {
  if (a.empty() || b.empty()) return {};
  std::vector<Fr> out(a.size() + b.size() - 1, Fr::zero());
  for (size_t i = 0; i < a.size(); ++i)
    for (size_t j = 0; j < b.size(); ++j) out[i + j] += a[i] * b[j];
  return out;
}
inline void add_scaled(std::vector<Fr>& acc, const std::vector<Fr>& src, const Fr& c) {
  if (src.size() > acc.size()) acc.resize(src.size(), Fr::zero());
  for (size_t i = 0; i < src.size(); ++i) acc[i] += c * src[i];
}
inline std::vector<Fr> vanishing(const std::vector<Fr>& roots) {
  std::vector<Fr> out{Fr::one()};
  for (auto& r : roots) out = mul(out, {-r, Fr::one()});
  return out;
}
inline std::vector<Fr> interpolate(const std::vector<std::pair<Fr, Fr>>& pts) {
  std::vector<Fr> out(pts.size(), Fr::zero());
  for (size_t i = 0; i < pts.size(); ++i) {
    std::vector<Fr> num{Fr::one()};
    Fr den = Fr::one();
    for (size_t j = 0; j < pts.size(); ++j) {
      if (i == j) continue;
      num = mul(num, {-pts[j].first, Fr::one()});
      den *= pts[i].first - pts[j].first;
    }
    add_scaled(out, num, pts[i].second * den.inverse());
  }
  return out;
}
inline Fr pow_usize(Fr x, size_t e) {
  Fr acc = Fr::one();
  while (e) {
    if (e & 1) acc *= x;
    x = x.square();
    e >>= 1;
  }
  return acc;
}
}  // namespace uni

// --- FFT over the two-adic subgroup ------------------------------------------
inline Fr two_adic_root() {
  // 5^((p-1) / 2^28): derived, not transcribed.
  uint64_t e[4] = {FrParams::MOD[0] - 1, FrParams::MOD[1], FrParams::MOD[2], FrParams::MOD[3]};
  for (int s = 0; s < 28; ++s) {
    for (int i = 0; i < 3; ++i) e[i] = (e[i] >> 1) | (e[i + 1] << 63);
    e[3] >>= 1;
  }
  return Fr::from_u64(5).pow(e);
}

inline void butterflies(std::vector<Fr>& a, const std::vector<Fr>& tw) {
  size_t m = a.size();
  if (m <= 1) return;
  int bits = __builtin_ctzll(m);
  for (size_t i = 0; i < m; ++i) {
    size_t j = 0;
    for (int b = 0; b < bits; ++b) j |= ((i >> b) & 1) << (bits - 1 - b);
    if (i < j) std::swap(a[i], a[j]);
  }
  for (size_t half = 1; half < m; half *= 2) {
    size_t step = m / (2 * half);
    for (size_t start = 0; start < m; start += 2 * half)
      for (size_t k = 0; k < half; ++k) {
        Fr w = tw[k * step];
        Fr lo = a[start + k], hi = a[start + k + half] * w;
        a[start + k] = lo + hi;
        a[start + k + half] = lo - hi;
      }
  }
}

struct Domain {
  std::vector<Fr> fwd, inv;
  Fr m_inv;
  explicit Domain(size_t half) {
    size_t m = 2 * half;
    int k = __builtin_ctzll(m);
    Fr w = two_adic_root();
    for (int i = k; i < 28; ++i) w = w.square();
    Fr wi = w.inverse();
    fwd = powers(w, m / 2);
    inv = powers(wi, m / 2);
    m_inv = Fr::from_u64(m).inverse();
  }
  void fft(std::vector<Fr>& a) const { butterflies(a, fwd); }
  void ifft(std::vector<Fr>& a) const {
    butterflies(a, inv);
    for (auto& x : a) x *= m_inv;
  }
};

// --- Mercury -----------------------------------------------------------------
enum PcsStatus { PCS_OK = 0, PCS_UNSUPPORTED_NUM_VARS = 1, PCS_POINT_LENGTH = 2, PCS_SRS_TOO_SMALL = 3,
                 PCS_DEGENERATE = 4, PCS_EMPTY_BATCH = 5, PCS_BATCH_LENGTH = 6, PCS_MIXED_SIZES = 7 };

inline bool check_num_vars(size_t nv) { return nv >= 2 && nv <= 54 && nv % 2 == 0; }

inline Fr dot(const std::vector<Fr>& a, const std::vector<Fr>& b) {
  Fr acc = Fr::zero();
  for (size_t i = 0; i < a.size(); ++i) acc += a[i] * b[i];
  return acc;
}

inline G1Bytes commit_to(const Srs& srs, const std::vector<Fr>& c, size_t threads) {
  return g1_bytes(msm(srs.g1.data(), c.data(), c.size(), threads));
}

inline void append_g1(Transcript& tr, uint64_t tag, const std::vector<G1Bytes>& ps) {
  std::vector<std::array<uint8_t, 64>> v(ps.begin(), ps.end());
  append_g1_points(tr, tag, v);
}

inline Fr tensor_eval(const std::vector<Fr>& u, const Fr& x) {
  Fr acc = Fr::one(), power = x;
  for (auto& uk : u) {
    acc *= uk * power + (Fr::one() - uk);
    power = power.square();
  }
  return acc;
}

inline Fr derive_h_alpha(const std::vector<Fr>& u1, const std::vector<Fr>& u2, const Fr& z, const Fr& zi,
                         const Fr& gamma, const Fr& v, const Fr ev[6]) {
  Fr inner = ev[0] * tensor_eval(u1, zi) + ev[1] * tensor_eval(u1, z) +
             gamma * (ev[2] * tensor_eval(u2, zi) + ev[3] * tensor_eval(u2, z) - v - v) - z * ev[4] - zi * ev[5];
  return inner * Fr::from_u64(2).inverse();
}

inline std::vector<Fr> symmetric_witness(const std::vector<Fr>& g, const std::vector<Fr>& h, const std::vector<Fr>& eq1,
                                         const std::vector<Fr>& eq2, const Fr& gamma) {
  size_t b = g.size();
  Domain dom(b);
  auto padded = [&](const std::vector<Fr>& c, bool rev) {
    std::vector<Fr> out(2 * b, Fr::zero());
    for (size_t i = 0; i < b; ++i) out[i] = rev ? c[b - 1 - i] : c[i];
    dom.fft(out);
    return out;
  };
  auto gh = padded(g, false), p1 = padded(eq1, true), hh = padded(h, false), p2 = padded(eq2, true);
  std::vector<Fr> r(2 * b);
  for (size_t k = 0; k < 2 * b; ++k) r[k] = gh[k] * p1[k] + gamma * hh[k] * p2[k];
  dom.ifft(r);
  std::vector<Fr> s;
  for (size_t k = b; k < 2 * b - 1; ++k) s.push_back(r[k] + r[2 * b - 2 - k]);
  return s;
}

struct MercuryProof {
  G1Bytes pts[8];
  Fr ev[6];
  void to_bytes(uint8_t out[704]) const {
    for (int i = 0; i < 8; ++i) memcpy(out + 64 * i, pts[i].data(), 64);
    for (int i = 0; i < 6; ++i) ev[i].to_bytes(out + 512 + 32 * i);
  }
};

struct BdfgItem {
  std::vector<Fr> zc, r;
};

inline int mercury_open(const Srs& srs, const Table& coeffs, const G1Bytes& cm, const std::vector<Fr>& u,
                        Transcript& tr, Fr& v_out, MercuryProof& pf, size_t threads) {
  size_t nv = u.size();
  if (!check_num_vars(nv)) return PCS_UNSUPPORTED_NUM_VARS;
  size_t n = (size_t)1 << nv;
  if (coeffs.size() != n) return PCS_POINT_LENGTH;
  if (srs.g1.size() < n) return PCS_SRS_TOO_SMALL;
  size_t t = nv / 2, b = (size_t)1 << t;
  std::vector<Fr> u1(u.begin(), u.begin() + t), u2(u.begin() + t, u.end());
  Table eq1 = eq_table(u1), eq2 = eq_table(u2);
  std::vector<Fr> hc(b);
  for (size_t j = 0; j < b; ++j) {
    Fr acc = Fr::zero();
    for (size_t i = 0; i < b; ++i) acc += eq1[i] * coeffs[j * b + i];
    hc[j] = acc;
  }
  Fr v = dot(eq2, hc);
  G1Bytes h_pt = commit_to(srs, hc, threads);
  tr.append_scalar(tags::MERCURY_INSTANCE, Fr::from_u64(n));
  append_g1(tr, tags::COMMITMENT, {cm});
  std::vector<Fr> claim = u;
  claim.push_back(v);
  tr.append_scalars(tags::EVALUATION_CLAIM, claim);
  append_g1(tr, tags::PCS_OPENING, {h_pt});
  Fr alpha = tr.challenge(tags::MERCURY_ALPHA);

  std::vector<Fr> acc(coeffs.begin() + (b - 1) * b, coeffs.end());
  std::vector<Fr> qc((b - 1) * b);
  for (size_t j = b - 1; j-- > 0;) {
    for (size_t i = 0; i < b; ++i) qc[j * b + i] = acc[i];
    for (size_t i = 0; i < b; ++i) acc[i] = coeffs[j * b + i] + acc[i] * alpha;
  }
  std::vector<Fr> gc = acc;
  G1Bytes q_pt = commit_to(srs, qc, threads), g_pt = commit_to(srs, gc, threads);
  append_g1(tr, tags::PCS_OPENING, {q_pt, g_pt});
  Fr gamma = tr.challenge(tags::MERCURY_GAMMA);

  Fr h_alpha = uni::eval(hc, alpha);
  std::vector<Fr> sc = symmetric_witness(gc, hc, eq1, eq2, gamma);
  std::vector<Fr> dc(gc.rbegin(), gc.rend());
  G1Bytes s_pt = commit_to(srs, sc, threads), d_pt = commit_to(srs, dc, threads);
  append_g1(tr, tags::PCS_OPENING, {s_pt, d_pt});
  Fr z;
  do {
    z = tr.challenge(tags::MERCURY_Z);
  } while (z.is_zero());
  if (z.square() == Fr::one() || z == alpha || z * alpha == Fr::one()) return PCS_DEGENERATE;
  Fr zi = z.inverse();
  Fr ev[6] = {uni::eval(gc, z), uni::eval(gc, zi), uni::eval(hc, z), uni::eval(hc, zi), uni::eval(sc, z), uni::eval(sc, zi)};
  tr.append_scalars(tags::PCS_OPENING, ev, 6);

  Fr zb = uni::pow_usize(z, b);
  std::vector<Fr> num = coeffs;
  for (size_t i = 0; i < qc.size(); ++i) num[i] -= (zb - alpha) * qc[i];
  num[0] -= ev[0];
  auto qr = uni::div_by_linear(num, z);
  if (!qr.second.is_zero()) throw std::runtime_error("fold identity does not vanish");
  G1Bytes piz = commit_to(srs, qr.first, threads);
  append_g1(tr, tags::PCS_OPENING, {piz});

  Fr ha = derive_h_alpha(u1, u2, z, zi, gamma, v, ev);
  if (ha != h_alpha) throw std::runtime_error("h(alpha) re-derivation mismatch");
  Fr d_z = uni::pow_usize(z, b - 1) * ev[1];
  std::vector<Fr> tset = {z, zi, alpha};
  std::vector<Fr> wa = uni::vanishing({alpha});
  BdfgItem items[4] = {
      {wa, uni::interpolate({{z, ev[0]}, {zi, ev[1]}})},
      {{Fr::one()}, uni::interpolate({{z, ev[2]}, {zi, ev[3]}, {alpha, h_alpha}})},
      {wa, uni::interpolate({{z, ev[4]}, {zi, ev[5]}})},
      {uni::vanishing({zi, alpha}), {d_z}},
  };
  const std::vector<Fr>* polys[4] = {&gc, &hc, &sc, &dc};
  Fr delta = tr.challenge(tags::BDFG_BATCH);
  std::vector<Fr> f;
  Fr pw = Fr::one();
  for (int i = 0; i < 4; ++i) {
    std::vector<Fr> sh = *polys[i];
    uni::add_scaled(sh, items[i].r, -Fr::one());
    uni::add_scaled(f, uni::mul(items[i].zc, sh), pw);
    pw *= delta;
  }
  std::vector<Fr> w = f;
  for (auto& root : tset) {
    auto d = uni::div_by_linear(w, root);
    if (!d.second.is_zero()) throw std::runtime_error("F not divisible by Z_T");
    w = d.first;
  }
  G1Bytes w_pt = commit_to(srs, w, threads);
  append_g1(tr, tags::PCS_OPENING, {w_pt});
  Fr zp = tr.challenge(tags::BDFG_POINT);
  std::vector<Fr> l;
  Fr cst = Fr::zero();
  uni::add_scaled(l, w, -uni::eval(uni::vanishing(tset), zp));
  for (int i = 0; i < 4; ++i) {
    Fr cc = uni::pow_usize(delta, i) * uni::eval(items[i].zc, zp);
    uni::add_scaled(l, *polys[i], cc);
    cst += cc * uni::eval(items[i].r, zp);
  }
  if (l.empty()) l.push_back(Fr::zero());
  l[0] -= cst;
  auto wp = uni::div_by_linear(l, zp);
  if (!wp.second.is_zero()) throw std::runtime_error("linearization does not vanish");
  G1Bytes wp_pt = commit_to(srs, wp.first, threads);
  append_g1(tr, tags::PCS_OPENING, {wp_pt});
  (void)tr.challenge(tags::PAIRING_MERGE);

  v_out = v;
  G1Bytes pts[8] = {h_pt, q_pt, g_pt, s_pt, d_pt, piz, w_pt, wp_pt};
  for (int i = 0; i < 8; ++i) pf.pts[i] = pts[i];
  for (int i = 0; i < 6; ++i) pf.ev[i] = ev[i];
  return PCS_OK;
}

// batch_open_stacked (crates/pcs/src/lib.rs:705-789): stack j's column s sits
// at slot s of a (width + |r|)-variable table; v_j = sum_s eq_r[s] * col_{j,s}(u)
// (:756-764), the preamble absorbs the commitments, then u || r and the values
// (:568-581), and f* = sum_j rho^j stack_j is opened at u || r (:766-788).
// `stacks[j]` lists stack j's columns, each a table of 2^width entries.
inline int mercury_batch_open_stacked(const Srs& srs, const std::vector<std::vector<const Table*>>& stacks,
                                      const std::vector<G1Bytes>& cms, const std::vector<Fr>& u,
                                      const std::vector<Fr>& r, Transcript& tr, std::vector<Fr>& vs,
                                      MercuryProof& pf, size_t threads) {
  if (stacks.empty()) return PCS_EMPTY_BATCH;
  for (auto& st : stacks)
    if (st.empty()) return PCS_EMPTY_BATCH;
  if (stacks.size() != cms.size()) return PCS_BATCH_LENGTH;
  const size_t column = stacks[0][0]->size();
  for (auto& st : stacks)
    for (const Table* c : st)
      if (c->size() != column) return PCS_MIXED_SIZES;
  const size_t width = (size_t)__builtin_ctzll(column);
  if (!check_num_vars(width + r.size())) return PCS_UNSUPPORTED_NUM_VARS;
  if (u.size() != width) return PCS_POINT_LENGTH;
  const size_t slots = (size_t)1 << r.size();
  for (auto& st : stacks)
    if (st.size() > slots) return PCS_BATCH_LENGTH;
  const size_t n = column << r.size();
  if (srs.g1.size() < n) return PCS_SRS_TOO_SMALL;
  std::vector<Fr> point = u;
  point.insert(point.end(), r.begin(), r.end());
  const Table eq_r = eq_table(r);
  vs.clear();
  for (auto& st : stacks) {
    Fr v = Fr::zero();
    for (size_t s = 0; s < st.size(); ++s) v += eq_r[s] * evaluate(*st[s], u);
    vs.push_back(v);
  }
  append_g1(tr, tags::COMMITMENT, cms);
  std::vector<Fr> claim = point;
  claim.insert(claim.end(), vs.begin(), vs.end());
  tr.append_scalars(tags::EVALUATION_CLAIM, claim);
  Fr rho = tr.challenge(tags::MERCURY_BATCH);
  std::vector<Fr> wts = powers(rho, cms.size());
  std::vector<G1Affine> cmp(cms.size());
  for (size_t i = 0; i < cms.size(); ++i) G1Affine::from_bytes(cms[i].data(), cmp[i]);
  G1Bytes cm_star = g1_bytes(msm(cmp.data(), wts.data(), cmp.size(), threads));
  Table comb(n, Fr::zero());
  for (size_t i = 0; i < n; ++i) {
    const size_t slot = i / column, row = i % column;
    for (size_t j = 0; j < stacks.size(); ++j)
      if (slot < stacks[j].size()) comb[i] += wts[j] * (*stacks[j][slot])[row];
  }
  Fr v;
  int st = mercury_open(srs, comb, cm_star, point, tr, v, pf, threads);
  if (st) return st;
  if (v != dot(wts, vs)) throw std::runtime_error("combined value mismatch");
  return PCS_OK;
}

// batch_open = batch_open_stacked at r = [], every stack one column
// (crates/pcs/src/lib.rs:688-703).
inline int mercury_batch_open(const Srs& srs, const std::vector<Table>& cols, const std::vector<G1Bytes>& cms,
                              const std::vector<Fr>& u, Transcript& tr, std::vector<Fr>& vs, MercuryProof& pf,
                              size_t threads) {
  std::vector<std::vector<const Table*>> stacks;
  for (auto& c : cols) stacks.push_back({&c});
  return mercury_batch_open_stacked(srs, stacks, cms, u, {}, tr, vs, pf, threads);
}

}  // namespace oracle
