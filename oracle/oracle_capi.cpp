// ORACLE — test infrastructure only. A C ABI over the CPU restatement so that
// tests/ (via ctypes) and bench.py's CPU-baseline leg can drive it. Every
// field element crosses as 32 canonical little-endian bytes, every G1 point as
// 64 canonical bytes (all-zero = infinity), transcripts as the 226-byte
// snapshot tuple. Returns 0 on success, a nonzero status otherwise.
#include <thread>
#include <chrono>
#include <memory>

#include "accumulator.hpp"
#include "mercury.hpp"

using namespace oracle;

namespace {

bool read_fr(const uint8_t* b, Fr& x) { return Fr::from_bytes(b, x); }

std::vector<Table> read_tables(const uint8_t* data, size_t k, size_t n) {
  std::vector<Table> out(k, Table(n));
  for (size_t c = 0; c < k; ++c)
    for (size_t i = 0; i < n; ++i)
      if (!read_fr(data + 32 * (c * n + i), out[c][i])) throw std::runtime_error("non-canonical Fr");
  return out;
}

Challenges read_challenges(const uint32_t* slots, const uint8_t* values, size_t n) {
  Challenges ch;
  for (size_t i = 0; i < n; ++i) {
    Fr v;
    if (!read_fr(values + 32 * i, v)) throw std::runtime_error("non-canonical challenge");
    ch.slots.push_back({slots[i], v});
  }
  return ch;
}

template <class F>
int field_op(int op, const uint8_t* a, const uint8_t* b, uint8_t* out) {
  F x, y;
  if (!F::from_bytes(a, x)) return 2;
  switch (op) {
    case 0: if (!F::from_bytes(b, y)) return 2; (x + y).to_bytes(out); return 0;
    case 1: if (!F::from_bytes(b, y)) return 2; (x - y).to_bytes(out); return 0;
    case 2: if (!F::from_bytes(b, y)) return 2; (x * y).to_bytes(out); return 0;
    case 3: x.square().to_bytes(out); return 0;
    case 4: if (x.is_zero()) return 1; x.inverse().to_bytes(out); return 0;
    case 5: { uint64_t e[4]; memcpy(e, b, 32); x.pow(e).to_bytes(out); return 0; }
    case 6: (-x).to_bytes(out); return 0;
  }
  return 3;
}

}  // namespace

extern "C" {

int oracle_fr_op(int op, const uint8_t* a, const uint8_t* b, uint8_t* out) { return field_op<Fr>(op, a, b, out); }
int oracle_fq_op(int op, const uint8_t* a, const uint8_t* b, uint8_t* out) { return field_op<Fq>(op, a, b, out); }

// op 0: P+Q (Jacobian add), 1: 2P, 2: k*P (k canonical 32 B, any 256-bit integer),
// 3: -P, 4: (2P) + Q through the mixed add, the accumulator 2P at Z != 1.
int oracle_g1_op(int op, const uint8_t* p, const uint8_t* q, uint8_t* out) {
  G1Affine a, b;
  if (!G1Affine::from_bytes(p, a)) return 2;
  G1Jac r;
  switch (op) {
    case 0: if (!G1Affine::from_bytes(q, b)) return 2; r = G1Jac::from(a).add(G1Jac::from(b)); break;
    case 1: r = G1Jac::from(a).dbl(); break;
    case 2: r = G1Jac::from(a).mul_le_bytes(q); break;
    case 3: a.neg().to_bytes(out); return 0;
    case 4: if (!G1Affine::from_bytes(q, b)) return 2; r = G1Jac::from(a).dbl().add_affine(b); break;
    default: return 3;
  }
  r.to_affine().to_bytes(out);
  return 0;
}

int oracle_g1_check(const uint8_t* p) {
  G1Affine a;
  return G1Affine::from_bytes(p, a) ? 0 : 1;
}

int oracle_msm(const uint8_t* bases, const uint8_t* scalars, size_t n, size_t threads, uint8_t* out) {
  try {
    std::vector<G1Affine> b(n);
    std::vector<Fr> s(n);
    for (size_t i = 0; i < n; ++i) {
      if (!G1Affine::from_bytes(bases + 64 * i, b[i])) return 2;
      if (!read_fr(scalars + 32 * i, s[i])) return 2;
    }
    msm(b.data(), s.data(), n, threads ? threads : 1).to_affine().to_bytes(out);
    return 0;
  } catch (...) {
    return 9;
  }
}

int oracle_msm_u32(const uint8_t* bases, const uint32_t* scalars, size_t n, size_t threads, uint8_t* out) {
  std::vector<G1Affine> b(n);
  for (size_t i = 0; i < n; ++i)
    if (!G1Affine::from_bytes(bases + 64 * i, b[i])) return 2;
  msm_u32(b.data(), scalars, n, threads ? threads : 1).to_affine().to_bytes(out);
  return 0;
}

// Seconds spent in one MSM over already-decoded inputs (the CPU baseline leg):
// bases/scalars are decoded outside the timed region.
double oracle_time_msm(const uint8_t* bases, const uint8_t* scalars, size_t n, size_t threads, uint8_t* out) {
  std::vector<G1Affine> b(n);
  std::vector<Fr> s(n);
  for (size_t i = 0; i < n; ++i) {
    if (!G1Affine::from_bytes(bases + 64 * i, b[i])) return -1.0;
    if (!read_fr(scalars + 32 * i, s[i])) return -1.0;
  }
  auto t0 = std::chrono::steady_clock::now();
  G1Jac r = msm(b.data(), s.data(), n, threads ? threads : 1);
  auto t1 = std::chrono::steady_clock::now();
  r.to_affine().to_bytes(out);
  return std::chrono::duration<double>(t1 - t0).count();
}

int oracle_poseidon2(const uint8_t* in, uint8_t* out) {
  Fr s[3];
  for (int i = 0; i < 3; ++i)
    if (!read_fr(in + 32 * i, s[i])) return 2;
  poseidon2_permute(s);
  for (int i = 0; i < 3; ++i) s[i].to_bytes(out + 32 * i);
  return 0;
}

// Transcript scripting over a snapshot buffer (226 bytes, in/out).
// op 0: observe(x); 1: sample -> out; 2: append_scalars(tag, n, xs);
// 3: append_bytes(tag, n bytes); 4: challenge(tag) -> out.
int oracle_transcript_op(uint8_t* snap, int op, uint64_t tag, const uint8_t* data, size_t n, uint8_t* out) {
  Transcript tr;
  if (!tr.restore(snap)) return 2;
  switch (op) {
    case 0: { Fr x; if (!read_fr(data, x)) return 2; tr.observe(x); break; }
    case 1: tr.sample().to_bytes(out); break;
    case 2: {
      std::vector<Fr> xs(n);
      for (size_t i = 0; i < n; ++i)
        if (!read_fr(data + 32 * i, xs[i])) return 2;
      tr.append_scalars(tag, xs);
      break;
    }
    case 3: tr.append_bytes(tag, data, n); break;
    case 4: tr.challenge(tag).to_bytes(out); break;
    default: return 3;
  }
  tr.snapshot(snap);
  return 0;
}

void oracle_transcript_new(uint8_t* snap) {
  Transcript tr;
  tr.snapshot(snap);
}

int oracle_g1_limbs(const uint8_t* p, uint8_t* out) {
  auto l = g1_limbs(p);
  for (int i = 0; i < 4; ++i) l[i].to_bytes(out + 32 * i);
  return 0;
}

int oracle_eq_table(const uint8_t* r, size_t n, uint8_t* out) {
  std::vector<Fr> rv(n);
  for (size_t i = 0; i < n; ++i)
    if (!read_fr(r + 32 * i, rv[i])) return 2;
  Table t = eq_table(rv);
  for (size_t i = 0; i < t.size(); ++i) t[i].to_bytes(out + 32 * i);
  return 0;
}

// Bind `k` challenges in order into a table of 2^nv entries (in/out, the
// result in the first 2^(nv-k) slots).
int oracle_bind(uint8_t* table, size_t nv, const uint8_t* rs, size_t k) {
  Table t = read_tables(table, 1, (size_t)1 << nv)[0];
  for (size_t i = 0; i < k; ++i) {
    Fr r;
    if (!read_fr(rs + 32 * i, r)) return 2;
    bind_table(t, r);
  }
  for (size_t i = 0; i < t.size(); ++i) t[i].to_bytes(table + 32 * i);
  return 0;
}

int oracle_evaluate(const uint8_t* table, size_t nv, const uint8_t* point, uint8_t* out) {
  Table t = read_tables(table, 1, (size_t)1 << nv)[0];
  std::vector<Fr> p(nv);
  for (size_t i = 0; i < nv; ++i)
    if (!read_fr(point + 32 * i, p[i])) return 2;
  evaluate(t, p).to_bytes(out);
  return 0;
}

int oracle_witness_digest(const uint8_t* cols, size_t k, size_t nv, uint8_t* out) {
  witness_digest(read_tables(cols, k, (size_t)1 << nv)).to_bytes(out);
  return 0;
}

// Gate terms: coefs (k x 32 B), a[k], b[k] with 0xffffffff for "no factor".
int oracle_prove_zerocheck(size_t arity, const uint8_t* coefs, const uint32_t* ta, const uint32_t* tb, size_t nterms,
                           const uint8_t* polys, size_t nv, uint8_t* snap, uint8_t* rounds_out, uint8_t* finals_out) {
  try {
    Gate g;
    g.arity = arity;
    for (size_t i = 0; i < nterms; ++i) {
      GateTerm t;
      if (!read_fr(coefs + 32 * i, t.coef)) return 2;
      t.a = ta[i];
      t.b = tb[i] == 0xffffffffu ? -1 : (int64_t)tb[i];
      g.terms.push_back(t);
    }
    auto ps = read_tables(polys, arity, (size_t)1 << nv);
    Transcript tr;
    if (!tr.restore(snap)) return 2;
    SumcheckProof p = prove_zerocheck(g, ps, tr);
    for (size_t r = 0; r < p.rounds.size(); ++r)
      for (int j = 0; j < 4; ++j) p.rounds[r][j].to_bytes(rounds_out + 32 * (4 * r + j));
    for (size_t i = 0; i < p.final_evals.size(); ++i) p.final_evals[i].to_bytes(finals_out + 32 * i);
    tr.snapshot(snap);
    return 0;
  } catch (...) {
    return 9;
  }
}

// GKR prove over an APGC circuit blob. `base` holds the committed columns in
// layout order, 2^trace_vars entries each. The proof is written as, for each
// gate list k = 0..depth-1: its rounds (4 Fr each) then its final evals; the
// caller sizes `proof_out` from the circuit. `top_out` receives the top
// layer's columns (width x 2^n_top), for checking forward.
int oracle_gkr_prove(const uint8_t* blob, size_t blob_len, const uint8_t* base, const uint32_t* slots,
                     const uint8_t* slot_values, size_t nslots, uint8_t* snap, uint8_t* proof_out, uint8_t* top_out) {
  try {
    Circuit c = parse_circuit(blob, blob_len);
    Challenges ch = read_challenges(slots, slot_values, nslots);
    auto b = read_tables(base, c.n_committed, (size_t)1 << c.trace_vars);
    LayerValues vals = forward(c, b, ch);
    Transcript tr;
    if (!tr.restore(snap)) return 2;
    auto proofs = gkr_prove(c, vals, ch, tr);
    size_t off = 0;
    for (auto& p : proofs) {
      for (auto& r : p.rounds)
        for (int j = 0; j < 4; ++j, off += 32) r[j].to_bytes(proof_out + off);
      for (auto& f : p.final_evals) {
        f.to_bytes(proof_out + off);
        off += 32;
      }
    }
    size_t o2 = 0;
    for (auto& col : vals.back())
      for (auto& x : col) {
        x.to_bytes(top_out + o2);
        o2 += 32;
      }
    tr.snapshot(snap);
    return 0;
  } catch (...) {
    return 9;
  }
}

// gkr::prove_sumcheck (crates/gkr/src/lib.rs:792-899) for gate list `layer`
// over the caller's tables (canonical Fr): `lower` holds width tables of 2^n
// entries, `upper` (a halving list's child-1 tables) width more. Writes the
// rounds (4n), the point (n) and the tables' bound values (lower then upper).
int oracle_gkr_prove_sumcheck(const uint8_t* blob, size_t blob_len, size_t layer, const uint8_t* weights,
                              size_t n_weights, const uint32_t* slots, const uint8_t* slot_values, size_t nslots,
                              const uint8_t* eq_point, size_t n, const uint8_t* lower, const uint8_t* upper,
                              size_t width, uint8_t* snap, uint8_t* rounds_out, uint8_t* point_out,
                              uint8_t* finals_out) {
  try {
    Circuit c = parse_circuit(blob, blob_len);
    if (layer >= c.layers.size()) return 2;
    Challenges ch = read_challenges(slots, slot_values, nslots);
    std::vector<Fr> w = n_weights ? read_tables(weights, 1, n_weights)[0] : std::vector<Fr>();
    std::vector<Fr> pt = n ? read_tables(eq_point, 1, n)[0] : std::vector<Fr>();
    std::vector<Table> lo = read_tables(lower, width, (size_t)1 << n), up;
    if (c.layers[layer].halving) up = read_tables(upper, width, (size_t)1 << n);
    Transcript tr;
    if (!tr.restore(snap)) return 2;
    auto rp = prove_layer_sumcheck(c, layer, pt, w, lo, up, ch, tr);
    size_t off = 0;
    for (auto& g : rp.first)
      for (int j = 0; j < 4; ++j, off += 32) g[j].to_bytes(rounds_out + off);
    for (size_t i = 0; i < rp.second.size(); ++i) rp.second[i].to_bytes(point_out + 32 * i);
    off = 0;
    for (auto* ts : {&lo, &up})
      for (auto& t : *ts) {
        t[0].to_bytes(finals_out + off);
        off += 32;
      }
    tr.snapshot(snap);
    return 0;
  } catch (...) {
    return 9;
  }
}

int oracle_toy_srs(const uint8_t* tau, size_t count, size_t threads, uint8_t* out) {
  Fr t;
  if (!read_fr(tau, t)) return 2;
  Srs s = toy_srs(t, count, threads ? threads : 1);
  for (size_t i = 0; i < count; ++i) s.g1[i].to_bytes(out + 64 * i);
  return 0;
}

static Srs read_srs(const uint8_t* pts, size_t n) {
  Srs s;
  s.g1.resize(n);
  for (size_t i = 0; i < n; ++i)
    if (!G1Affine::from_bytes(pts + 64 * i, s.g1[i])) throw std::runtime_error("bad SRS point");
  return s;
}

// f(tau) = sum_i coeffs[i] tau^i for n canonical coefficients: the scalar of
// the known-tau identity commit(f) = [f(tau)]G over a seeded-tau SRS
// (crates/pcs/src/lib.rs:237-247 reads the table as coefficients). Horner per
// chunk on `threads` host threads, chunks joined by tau^(chunk start).
int oracle_poly_at(const uint8_t* coeffs, size_t n, const uint8_t* tau, size_t threads, uint8_t* out) {
  Fr t;
  if (!read_fr(tau, t)) return 2;
  size_t nt = std::max<size_t>(1, std::min<size_t>(threads ? threads : 1, n / 4096 + 1));
  size_t step = (n + nt - 1) / nt;
  std::vector<Fr> part(nt, Fr::zero());
  std::vector<int> bad(nt, 0);
  std::vector<std::thread> pool;
  for (size_t w = 0; w < nt; ++w) {
    pool.emplace_back([&, w] {
      size_t b = w * step, e = std::min(n, b + step);
      Fr acc = Fr::zero();
      for (size_t i = e; i-- > b;) {
        Fr c;
        if (!read_fr(coeffs + 32 * i, c)) {
          bad[w] = 1;
          return;
        }
        acc = acc * t + c;
      }
      part[w] = acc;
    });
  }
  for (auto& th : pool) th.join();
  Fr acc = Fr::zero();
  for (size_t w = nt; w-- > 0;) {
    if (bad[w]) return 2;
    size_t b = w * step;
    if (b >= n) continue;
    // acc currently holds the value of the chunks above w, relative to their start
    Fr tp = Fr::one(), base = t;
    for (size_t e = std::min(n, b + step) - b; e; e >>= 1, base = base * base)
      if (e & 1) tp = tp * base;
    acc = acc * tp + part[w];
  }
  acc.to_bytes(out);
  return 0;
}

int oracle_commit(const uint8_t* srs_pts, size_t srs_n, const uint8_t* evals, size_t nv, size_t threads, uint8_t* out) {
  try {
    if (!check_num_vars(nv)) return 10 + PCS_UNSUPPORTED_NUM_VARS;
    size_t n = (size_t)1 << nv;
    if (srs_n < n) return 10 + PCS_SRS_TOO_SMALL;
    Srs s = read_srs(srs_pts, n);
    Table t = read_tables(evals, 1, n)[0];
    auto b = commit_to(s, t, threads ? threads : 1);
    memcpy(out, b.data(), 64);
    return 0;
  } catch (...) {
    return 9;
  }
}

int oracle_mercury_open(const uint8_t* srs_pts, size_t srs_n, const uint8_t* evals, size_t nv, const uint8_t* cm,
                        const uint8_t* u, uint8_t* snap, size_t threads, uint8_t* v_out, uint8_t* proof_out) {
  try {
    Srs s = read_srs(srs_pts, srs_n);
    Table t = read_tables(evals, 1, (size_t)1 << nv)[0];
    std::vector<Fr> uv(nv);
    for (size_t i = 0; i < nv; ++i)
      if (!read_fr(u + 32 * i, uv[i])) return 2;
    G1Bytes c;
    memcpy(c.data(), cm, 64);
    Transcript tr;
    if (!tr.restore(snap)) return 2;
    Fr v;
    MercuryProof pf;
    int st = mercury_open(s, t, c, uv, tr, v, pf, threads ? threads : 1);
    if (st) return 10 + st;
    v.to_bytes(v_out);
    pf.to_bytes(proof_out);
    tr.snapshot(snap);
    return 0;
  } catch (...) {
    return 9;
  }
}

// batch_open_stacked: n_cols columns back to back (column c has 2^col_nv[c]
// entries), stack j taking the next stack_lens[j] of them; n_cms commitments.
// Returns 10 + the PcsStatus on a refusal.
int oracle_mercury_batch_open_stacked(const uint8_t* srs_pts, size_t srs_n, const uint8_t* cols,
                                      const size_t* col_nv, const size_t* stack_lens, size_t n_stacks,
                                      const uint8_t* cms, size_t n_cms, const uint8_t* u, size_t u_len,
                                      const uint8_t* r, size_t r_len, uint8_t* snap, size_t threads,
                                      uint8_t* vs_out, uint8_t* proof_out) {
  try {
    Srs s = read_srs(srs_pts, srs_n);
    size_t n_cols = 0;
    for (size_t j = 0; j < n_stacks; ++j) n_cols += stack_lens[j];
    std::vector<Table> tabs;
    tabs.reserve(n_cols);
    size_t off = 0;
    for (size_t c = 0; c < n_cols; ++c) {
      const size_t len = (size_t)1 << col_nv[c];
      tabs.push_back(read_tables(cols + off, 1, len)[0]);
      off += 32 * len;
    }
    std::vector<std::vector<const Table*>> stacks(n_stacks);
    size_t c = 0;
    for (size_t j = 0; j < n_stacks; ++j)
      for (size_t e = 0; e < stack_lens[j]; ++e) stacks[j].push_back(&tabs[c++]);
    std::vector<Fr> uv(u_len), rv(r_len);
    for (size_t i = 0; i < u_len; ++i)
      if (!read_fr(u + 32 * i, uv[i])) return 2;
    for (size_t i = 0; i < r_len; ++i)
      if (!read_fr(r + 32 * i, rv[i])) return 2;
    std::vector<G1Bytes> cm(n_cms);
    for (size_t i = 0; i < n_cms; ++i) memcpy(cm[i].data(), cms + 64 * i, 64);
    Transcript tr;
    if (!tr.restore(snap)) return 2;
    std::vector<Fr> vs;
    MercuryProof pf;
    int st = mercury_batch_open_stacked(s, stacks, cm, uv, rv, tr, vs, pf, threads ? threads : 1);
    if (st) return 10 + st;
    for (size_t j = 0; j < n_stacks; ++j) vs[j].to_bytes(vs_out + 32 * j);
    pf.to_bytes(proof_out);
    tr.snapshot(snap);
    return 0;
  } catch (...) {
    return 9;
  }
}

int oracle_mercury_batch_open(const uint8_t* srs_pts, size_t srs_n, const uint8_t* cols, size_t k, size_t nv,
                              const uint8_t* cms, const uint8_t* u, uint8_t* snap, size_t threads, uint8_t* vs_out,
                              uint8_t* proof_out) {
  try {
    Srs s = read_srs(srs_pts, srs_n);
    auto t = read_tables(cols, k, (size_t)1 << nv);
    std::vector<Fr> uv(nv);
    for (size_t i = 0; i < nv; ++i)
      if (!read_fr(u + 32 * i, uv[i])) return 2;
    std::vector<G1Bytes> c(k);
    for (size_t i = 0; i < k; ++i) memcpy(c[i].data(), cms + 64 * i, 64);
    Transcript tr;
    if (!tr.restore(snap)) return 2;
    std::vector<Fr> vs;
    MercuryProof pf;
    int st = mercury_batch_open(s, t, c, uv, tr, vs, pf, threads ? threads : 1);
    if (st) return 10 + st;
    for (size_t i = 0; i < k; ++i) vs[i].to_bytes(vs_out + 32 * i);
    pf.to_bytes(proof_out);
    tr.snapshot(snap);
    return 0;
  } catch (...) {
    return 9;
  }
}

// The deferred-pairing accumulator (accumulator.hpp). Entries: n side bytes,
// n canonical Fr scalars, n 64-byte points; checks: the group counts.
// weights == null: pcs::discharge (points validated first, then the
// partition; nu from the digest of the words); otherwise check_pairings with
// the caller's weights, one per check (the partition first). Returns 0,
// 2 (a non-canonical scalar or weight), 3 (a side tag other than 0 and 1),
// 9 (a point off the curve), 10 (counts that do not partition the entries).
// nu_out / digest_out are written in the discharge form only.
static int read_entries(const uint8_t* sides, const uint8_t* scalars, const uint8_t* points, size_t n,
                        std::vector<AccEntry>& out) {
  out.resize(n);
  for (size_t i = 0; i < n; ++i) {
    if (sides[i] > 1) return 3;
    out[i].side = sides[i];
    if (!G1Affine::from_bytes(points + 64 * i, out[i].point)) return 9;
  }
  for (size_t i = 0; i < n; ++i)
    if (!read_fr(scalars + 32 * i, out[i].scalar)) return 2;
  return 0;
}

int oracle_accumulator_msms(const uint8_t* sides, const uint8_t* scalars, const uint8_t* points, size_t n,
                            const uint64_t* checks, size_t n_checks, const uint8_t* weights, size_t threads,
                            uint8_t* a_out, uint8_t* b_out, uint8_t* nu_out, uint8_t* digest_out) {
  std::vector<size_t> cs(checks, checks + n_checks);
  std::vector<AccEntry> entries;
  std::vector<Fr> w(n_checks);
  if (weights) {
    if (!acc_partition(n, cs)) return 10;
    if (int st = read_entries(sides, scalars, points, n, entries)) return st;
    for (size_t j = 0; j < n_checks; ++j)
      if (!read_fr(weights + 32 * j, w[j])) return 2;
  } else {
    if (int st = read_entries(sides, scalars, points, n, entries)) return st;
    if (!acc_partition(n, cs)) return 10;
    const Fr digest = acc_digest(acc_words(entries, cs));
    const Fr nu = acc_merge_challenge(digest);
    w = acc_powers(nu, n_checks);
    if (nu_out) nu.to_bytes(nu_out);
    if (digest_out) digest.to_bytes(digest_out);
  }
  G1Affine a, b;
  acc_side_msms(entries, cs, w, threads ? threads : 1, a, b);
  a.to_bytes(a_out);
  b.to_bytes(b_out);
  return 0;
}

// accumulator_words (accumulator.rs:57-83): n_checks + 6n canonical Fr.
int oracle_accumulator_words(const uint8_t* sides, const uint8_t* scalars, const uint8_t* points, size_t n,
                             const uint64_t* checks, size_t n_checks, uint8_t* out) {
  std::vector<size_t> cs(checks, checks + n_checks);
  std::vector<AccEntry> entries;
  if (int st = read_entries(sides, scalars, points, n, entries)) return st;
  if (!acc_partition(n, cs)) return 10;
  const std::vector<Fr> words = acc_words(entries, cs);
  for (size_t i = 0; i < words.size(); ++i) words[i].to_bytes(out + 32 * i);
  return 0;
}

}  // extern "C"
