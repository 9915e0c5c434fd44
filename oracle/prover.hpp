// ORACLE — test infrastructure only. CPU restatement of the reference's
// multilinear tables, gate zerocheck and GKR layer prover, used by tests/ to
// check the CUDA library and by bench.py's CPU baseline.
//
//  * poly: bind (crates/poly/src/lib.rs:156-185), evaluate (:189-219),
//    eq_table (:233-248).
//  * sumcheck: Gate::evaluate (crates/sumcheck/src/lib.rs:151-167),
//    witness_digest (:228-256), interpolate_cubic (:294-305),
//    round_evaluations (:324-349), prove_zerocheck (:359-408).
//  * gkr: eval_gate (crates/gkr-verify/src/lib.rs:142-202), virtual_at_row /
//    virtual_at_point (:205-286), ResolvedList (:315-480), powers (:553-561);
//    forward / produce (crates/gkr/src/lib.rs:279-336), prove_sumcheck
//    (:792-899), children (:910-919), prove (:933-1016).
//
// Circuits arrive in the library's compact resolved form (the "APGC" blob the
// C ABI takes); parse_circuit reads it.
#pragma once
#include <algorithm>
#include <array>
#include <stdexcept>
#include <thread>
#include <vector>

#include "transcript.hpp"

namespace oracle {

// Runs f(begin, end, worker) over [0, n) split into contiguous chunks, one
// per host thread (the reference splits the same loops into rayon blocks,
// crates/gkr/src/lib.rs:189,302-336). Sums taken per chunk and added after
// are the same field elements in any order, so the results do not depend
// on the thread count.
template <class F>
inline void parallel_chunks(size_t n, F f) {
  size_t hw = std::max<size_t>(1, std::thread::hardware_concurrency());
  size_t nt = std::min<size_t>(hw, std::max<size_t>(1, n / 1024));
  if (nt <= 1) {
    f((size_t)0, n, (size_t)0);
    return;
  }
  std::vector<std::thread> pool;
  size_t step = (n + nt - 1) / nt;
  for (size_t w = 0; w < nt; ++w) {
    size_t b = w * step, e = std::min(n, b + step);
    if (b >= e) break;
    pool.emplace_back([=, &f] { f(b, e, w); });
  }
  for (auto& t : pool) t.join();
}

inline size_t parallel_workers() { return std::max<size_t>(1, std::thread::hardware_concurrency()); }

typedef std::vector<Fr> Table;

inline void bind_table(Table& t, const Fr& r) {
  size_t half = t.size() / 2;
  if (half >= (1u << 14)) {  // large tables: out of place, split across threads
    Table out(half);
    parallel_chunks(half, [&](size_t b, size_t e, size_t) {
      for (size_t i = b; i < e; ++i) out[i] = t[2 * i] + r * (t[2 * i + 1] - t[2 * i]);
    });
    t.swap(out);
    return;
  }
  for (size_t i = 0; i < half; ++i) {
    Fr lo = t[2 * i], hi = t[2 * i + 1];
    t[i] = lo + r * (hi - lo);
  }
  t.resize(half);
}

inline Fr evaluate(const Table& t, const std::vector<Fr>& point) {
  Table s = t;
  for (auto& r : point) bind_table(s, r);
  return s[0];
}

inline Table eq_table(const std::vector<Fr>& r) {
  Table t(1, Fr::one());
  for (size_t j = 0; j < r.size(); ++j) {
    size_t half = (size_t)1 << j;
    t.resize(2 * half, Fr::zero());
    for (size_t i = 0; i < half; ++i) {
      Fr v = t[i];
      Fr w = v * r[j];
      t[i + half] = w;
      t[i] = v - w;
    }
  }
  return t;
}

inline std::array<Fr, 3> interpolation_constants() {
  return {Fr::from_u64(2).inverse(), Fr::from_u64(3).inverse(), Fr::from_u64(6).inverse()};
}

inline std::array<Fr, 4> interpolate_cubic(const std::array<Fr, 4>& v) {
  static const std::array<Fr, 3> c = interpolation_constants();
  Fr d1 = v[1] - v[0];
  Fr d2 = (v[2] - v[1]) - d1;
  Fr d3 = ((v[3] - v[2]) - (v[2] - v[1])) - d2;
  return {v[0], d1 - d2 * c[0] + d3 * c[1], (d2 - d3) * c[0], d3 * c[2]};
}

// ---------------------------------------------------------------------------
// Zerocheck
// ---------------------------------------------------------------------------

struct GateTerm {
  Fr coef;
  uint32_t a;
  int64_t b;  // -1: no second factor
};
struct Gate {
  size_t arity;
  std::vector<GateTerm> terms;
  Fr evaluate(const Fr* v) const {
    Fr acc = Fr::zero();
    for (auto& t : terms) {
      Fr x = t.coef * v[t.a];
      if (t.b >= 0) x = x * v[t.b];
      acc += x;
    }
    return acc;
  }
};

inline Fr witness_digest(const std::vector<Table>& cols) {
  Transcript sponge;
  size_t n_vars = (size_t)__builtin_ctzll(cols[0].size());
  Fr hdr[2] = {Fr::from_u64(cols.size()), Fr::from_u64(n_vars)};
  sponge.append_scalars(tags::WITNESS_DIGEST, hdr, 2);
  for (auto& c : cols) sponge.append_scalars(tags::WITNESS_DIGEST, c);
  return sponge.sample();
}

struct SumcheckProof {
  std::vector<std::array<Fr, 4>> rounds;
  std::vector<Fr> final_evals;
};

inline SumcheckProof prove_zerocheck(const Gate& gate, std::vector<Table>& polys, Transcript& t) {
  size_t n = (size_t)__builtin_ctzll(polys[0].size());
  std::vector<Fr> r(n);
  for (size_t i = 0; i < n; ++i) r[i] = t.challenge(tags::SUMCHECK_CHALLENGE);
  Table eq = eq_table(r);
  SumcheckProof proof;
  size_t k = polys.size();
  std::vector<Fr> cur(k), step(k);
  for (size_t round = 0; round < n; ++round) {
    std::array<Fr, 4> acc = {Fr::zero(), Fr::zero(), Fr::zero(), Fr::zero()};
    size_t half = eq.size() / 2;
    for (size_t j = 0; j < half; ++j) {
      for (size_t c = 0; c < k; ++c) {
        cur[c] = polys[c][2 * j];
        step[c] = polys[c][2 * j + 1] - cur[c];
      }
      Fr e = eq[2 * j], es = eq[2 * j + 1] - eq[2 * j];
      for (int node = 0; node < 4; ++node) {
        acc[node] += e * gate.evaluate(cur.data());
        e += es;
        for (size_t c = 0; c < k; ++c) cur[c] += step[c];
      }
    }
    auto g = interpolate_cubic(acc);
    t.append_scalars(tags::SUMCHECK_ROUND, g.data(), 4);
    proof.rounds.push_back(g);
    Fr ch = t.challenge(tags::SUMCHECK_CHALLENGE);
    for (auto& p : polys) bind_table(p, ch);
    bind_table(eq, ch);
  }
  for (auto& p : polys) proof.final_evals.push_back(p[0]);
  t.append_scalars(tags::SUMCHECK_FINAL_EVALS, proof.final_evals);
  return proof;
}

// ---------------------------------------------------------------------------
// GKR
// ---------------------------------------------------------------------------

enum GateKind : uint32_t { LINEAR = 0, PRODUCT = 1, MASK = 2, AFFINE = 3, TREE_PRODUCT = 4, TREE_CROSS = 5, QUADRATIC = 6 };
enum SrcKind : uint32_t { SRC_COLUMN = 0, SRC_VIRTUAL = 1, SRC_CACHED = 2 };
enum VirtualKind : uint32_t { V_ROW = 0, V_RAM_LIVE = 1, V_RANGE19 = 2, V_RANGE16 = 3, V_XOR8A = 4, V_XOR8B = 5, V_XOR8OUT = 6 };

struct Coeff {
  bool challenge;
  Fr value;
  uint32_t slot;
};
struct GateDef {
  uint32_t kind, p1, p2;
  std::vector<std::pair<uint32_t, uint32_t>> operands;
  std::vector<Coeff> coeffs;
};
struct LayerSpec {
  bool halving;
  uint32_t num_vars, width;
  std::vector<GateDef> cached, producing, enforcing;
};
struct Circuit {
  uint32_t trace_vars, n_committed;
  std::vector<uint32_t> virtuals, outputs;
  std::vector<LayerSpec> layers;
  uint32_t layer_vars(size_t k) const { return k == 0 ? trace_vars : layers[k - 1].num_vars; }
  uint32_t layer_width(size_t k) const { return k == 0 ? n_committed : layers[k - 1].width; }
};

struct Reader {
  const uint8_t* p;
  const uint8_t* end;
  uint32_t u32() {
    if (p + 4 > end) throw std::runtime_error("circuit blob truncated");
    uint32_t v;
    memcpy(&v, p, 4);
    p += 4;
    return v;
  }
  Fr fr() {
    if (p + 32 > end) throw std::runtime_error("circuit blob truncated");
    Fr x;
    if (!Fr::from_bytes(p, x)) throw std::runtime_error("non-canonical coefficient");
    p += 32;
    return x;
  }
};

inline Circuit parse_circuit(const uint8_t* blob, size_t len) {
  Reader r{blob, blob + len};
  if (r.u32() != 0x43475041u || r.u32() != 1) throw std::runtime_error("not an APGC v1 blob");
  Circuit c;
  c.trace_vars = r.u32();
  c.n_committed = r.u32();
  uint32_t nv = r.u32();
  for (uint32_t i = 0; i < nv; ++i) c.virtuals.push_back(r.u32());
  uint32_t no = r.u32();
  for (uint32_t i = 0; i < no; ++i) c.outputs.push_back(r.u32());
  uint32_t depth = r.u32();
  for (uint32_t k = 0; k < depth; ++k) {
    LayerSpec L;
    L.halving = r.u32() != 0;
    L.num_vars = r.u32();
    L.width = r.u32();
    uint32_t nc = r.u32(), np = r.u32(), ne = r.u32();
    for (uint32_t g = 0; g < nc + np + ne; ++g) {
      GateDef d;
      d.kind = r.u32();
      d.p1 = r.u32();
      d.p2 = r.u32();
      uint32_t nop = r.u32();
      for (uint32_t i = 0; i < nop; ++i) {
        uint32_t s = r.u32();
        uint32_t x = r.u32();
        d.operands.push_back({s, x});
      }
      uint32_t ncf = r.u32();
      for (uint32_t i = 0; i < ncf; ++i) {
        Coeff cf{};
        cf.challenge = r.u32() != 0;
        if (cf.challenge) cf.slot = r.u32();
        else cf.value = r.fr();
        d.coeffs.push_back(cf);
      }
      (g < nc ? L.cached : g < nc + np ? L.producing : L.enforcing).push_back(d);
    }
    c.layers.push_back(L);
  }
  return c;
}

struct Challenges {
  std::vector<std::pair<uint32_t, Fr>> slots;
  Fr get(uint32_t s) const {
    for (auto& kv : slots)
      if (kv.first == s) return kv.second;
    throw std::runtime_error("external challenge slot has no value");
  }
};

inline Fr coeff_value(const Coeff& c, const Challenges& ch) { return c.challenge ? ch.get(c.slot) : c.value; }

// The gate kernel over one value per operand read, in GateDef operand order.
inline Fr eval_gate(const GateDef& g, const Fr* v, const Challenges& ch) {
  auto c = [&](size_t i) { return coeff_value(g.coeffs[i], ch); };
  switch (g.kind) {
    case LINEAR: {
      Fr acc = c(g.p1);
      for (uint32_t i = 0; i < g.p1; ++i) acc += c(i) * v[i];
      return acc;
    }
    case PRODUCT: return c(0) * v[0] * v[1];
    case MASK: return v[0] * v[1] + Fr::one() - v[1];
    case AFFINE: {
      uint32_t t = g.p1, u = g.p2;
      Fr l = c(t);
      for (uint32_t i = 0; i < t; ++i) l += c(i) * v[i];
      Fr rr = c(t + 1 + u);
      for (uint32_t j = 0; j < u; ++j) rr += c(t + 1 + j) * v[t + j];
      return l * rr;
    }
    case TREE_PRODUCT: return v[0] * v[1];
    case TREE_CROSS: return v[0] * v[3] + v[1] * v[2];
    case QUADRATIC: {
      uint32_t t = g.p1, u = g.p2;
      Fr acc = c(0);
      for (uint32_t i = 0; i < t; ++i) acc += c(1 + i) * v[i];
      for (uint32_t j = 0; j < u; ++j) acc += c(1 + t + j) * v[t + 2 * j] * v[t + 2 * j + 1];
      return acc;
    }
  }
  throw std::runtime_error("unknown gate kind");
}

inline Fr virtual_at_row(uint32_t kind, uint64_t row) {
  switch (kind) {
    case V_ROW: return Fr::from_u64(row);
    case V_RAM_LIVE: return row >= (1ULL << 14) ? Fr::one() : Fr::zero();
    case V_RANGE19: return Fr::from_u64(row & ((1ULL << 19) - 1));
    case V_RANGE16: return Fr::from_u64(row & ((1ULL << 16) - 1));
    case V_XOR8A: return Fr::from_u64(row & 0xff);
    case V_XOR8B: return Fr::from_u64((row >> 8) & 0xff);
    case V_XOR8OUT: return Fr::from_u64((row & 0xff) ^ ((row >> 8) & 0xff));
  }
  throw std::runtime_error("unknown virtual kind");
}

inline Fr virtual_at_point(uint32_t kind, const std::vector<Fr>& pt) {
  auto horner = [&](size_t lo, size_t hi) {
    Fr acc = Fr::zero();
    for (size_t j = hi; j-- > lo;) acc = acc + acc + (j < pt.size() ? pt[j] : Fr::zero());
    return acc;
  };
  switch (kind) {
    case V_ROW: return horner(0, pt.size());
    case V_RAM_LIVE: {
      Fr prod = Fr::one();
      for (size_t j = std::min<size_t>(pt.size(), 14); j < pt.size(); ++j) prod *= Fr::one() - pt[j];
      return Fr::one() - prod;
    }
    case V_RANGE19: return horner(0, std::min<size_t>(pt.size(), 19));
    case V_RANGE16: return horner(0, std::min<size_t>(pt.size(), 16));
    case V_XOR8A: return horner(0, 8);
    case V_XOR8B: return horner(8, 16);
    case V_XOR8OUT: {
      Fr acc = Fr::zero();
      for (int j = 7; j >= 0; --j) {
        Fr y = (size_t)j < pt.size() ? pt[j] : Fr::zero();
        Fr z = (size_t)(j + 8) < pt.size() ? pt[j + 8] : Fr::zero();
        Fr yz = y * z;
        acc = acc + acc + y + z - (yz + yz);
      }
      return acc;
    }
  }
  throw std::runtime_error("unknown virtual kind");
}

// Gate list k with operands resolved to read positions: cached entries, then
// producing gates, then enforcing gates (halving lists: producing only, every
// operand read at child 0 then child 1).
struct Resolved {
  enum Src { LOWER, UPPER, VIRT, CACHED };
  std::vector<const GateDef*> gates;
  std::vector<std::vector<std::pair<Src, uint32_t>>> sources;
  size_t cached = 0, producing = 0, enforcing = 0;
  const Challenges* ch;

  Resolved(const Circuit& c, size_t k, const Challenges& chal) : ch(&chal) {
    const LayerSpec& L = c.layers[k];
    if (L.halving) {
      for (auto& g : L.producing) {
        gates.push_back(&g);
        std::vector<std::pair<Src, uint32_t>> s;
        for (auto& op : g.operands) {
          s.push_back({LOWER, op.second});
          s.push_back({UPPER, op.second});
        }
        sources.push_back(s);
      }
      producing = L.producing.size();
    } else {
      auto add = [&](const GateDef& g) {
        gates.push_back(&g);
        std::vector<std::pair<Src, uint32_t>> s;
        for (auto& op : g.operands)
          s.push_back({op.first == SRC_COLUMN ? LOWER : op.first == SRC_VIRTUAL ? VIRT : CACHED, op.second});
        sources.push_back(s);
      };
      for (auto& g : L.cached) add(g);
      for (auto& g : L.producing) add(g);
      for (auto& g : L.enforcing) add(g);
      cached = L.cached.size();
      producing = L.producing.size();
      enforcing = L.enforcing.size();
    }
  }
  Fr eval(size_t i, const Fr* lower, const Fr* upper, const Fr* virt, const std::vector<Fr>& cache) const {
    auto& s = sources[i];
    // One operand buffer per host thread (a Linear gate may read a hundred
    // columns); eval_gate consumes it before the next eval on this thread.
    thread_local std::vector<Fr> ops;
    if (ops.size() < s.size() + 1) ops.resize(s.size() + 1);
    for (size_t j = 0; j < s.size(); ++j) {
      switch (s[j].first) {
        case LOWER: ops[j] = lower[s[j].second]; break;
        case UPPER: ops[j] = upper[s[j].second]; break;
        case VIRT: ops[j] = virt[s[j].second]; break;
        case CACHED: ops[j] = cache[s[j].second]; break;
      }
    }
    return eval_gate(*gates[i], ops.data(), *ch);
  }
  void fill_cache(const Fr* lower, const Fr* upper, const Fr* virt, std::vector<Fr>& cache) const {
    cache.resize(cached);
    for (size_t i = 0; i < cached; ++i) cache[i] = eval(i, lower, upper, virt, cache);
  }
  Fr gate(size_t j, const Fr* lower, const Fr* upper, const Fr* virt, const std::vector<Fr>& cache) const {
    return eval(cached + j, lower, upper, virt, cache);
  }
  Fr summand(const std::vector<Fr>& w, const Fr* lower, const Fr* upper, const Fr* virt) const {
    thread_local std::vector<Fr> cache;
    fill_cache(lower, upper, virt, cache);
    Fr acc = Fr::zero();
    for (size_t j = 0; j < w.size(); ++j) acc += gate(j, lower, upper, virt, cache) * w[j];
    return acc;
  }
};

inline std::vector<Fr> powers(const Fr& x, size_t n) {
  std::vector<Fr> out;
  Fr acc = Fr::one();
  for (size_t i = 0; i < n; ++i) {
    out.push_back(acc);
    acc *= x;
  }
  return out;
}

// layers[0] is the base (committed columns in layout order); layers[k] for
// k >= 1 is what gate list k-1 wrote.
typedef std::vector<std::vector<Table>> LayerValues;

inline std::vector<Table> produce(const Circuit& c, const LayerValues& vals, size_t k, const Challenges& ch) {
  const LayerSpec& L = c.layers[k];
  size_t rows_in = (size_t)1 << c.layer_vars(k);
  size_t rows = L.halving ? rows_in / 2 : rows_in;
  Resolved res(c, k, ch);
  const auto& cols = vals[k];
  size_t w = cols.size();
  std::vector<Table> out(L.width, Table(rows));
  parallel_chunks(rows, [&](size_t y0, size_t y1, size_t) {
    std::vector<Fr> lower(w), upper(w), virt(c.virtuals.size()), cache;
    for (size_t y = y0; y < y1; ++y) {
      if (L.halving) {
        for (size_t i = 0; i < w; ++i) {
          lower[i] = cols[i][y];
          upper[i] = cols[i][y + rows];
        }
      } else {
        for (size_t i = 0; i < w; ++i) lower[i] = cols[i][y];
        for (size_t v = 0; v < c.virtuals.size(); ++v) virt[v] = virtual_at_row(c.virtuals[v], y);
      }
      res.fill_cache(lower.data(), upper.data(), virt.data(), cache);
      for (size_t j = 0; j < L.width; ++j) out[j][y] = res.gate(j, lower.data(), upper.data(), virt.data(), cache);
    }
  });
  return out;
}

inline LayerValues forward(const Circuit& c, const std::vector<Table>& base, const Challenges& ch) {
  LayerValues vals;
  vals.push_back(base);
  for (size_t k = 0; k < c.layers.size(); ++k) vals.push_back(produce(c, vals, k, ch));
  return vals;
}

inline std::pair<std::vector<std::array<Fr, 4>>, std::vector<Fr>> prove_layer_sumcheck(
    const Circuit& c, size_t k, const std::vector<Fr>& eq_point, const std::vector<Fr>& weights,
    std::vector<Table>& lower_t, std::vector<Table>& upper_t, const Challenges& ch, Transcript& t) {
  size_t n = eq_point.size();
  const LayerSpec& L = c.layers[k];
  std::vector<uint32_t> kinds = L.halving ? std::vector<uint32_t>() : c.virtuals;
  Resolved res(c, k, ch);
  Table eq = eq_table(eq_point);
  std::vector<std::array<Fr, 4>> rounds;
  std::vector<Fr> point;
  size_t nl = lower_t.size(), nu = upper_t.size(), nv = kinds.size();
  for (size_t round = 0; round < n; ++round) {
    size_t half = eq.size() / 2;
    size_t bound = point.size();
    std::vector<std::array<Fr, 4>> part(parallel_workers(), {Fr::zero(), Fr::zero(), Fr::zero(), Fr::zero()});
    parallel_chunks(half, [&](size_t i0, size_t i1, size_t wk) {
      std::vector<Fr> lo(nl), los(nl), up(nu), ups(nu), vv(nv), vs(nv);
      std::vector<Fr> at(n, Fr::zero());
      for (size_t i = 0; i < bound; ++i) at[i] = point[i];
      std::array<Fr, 4>& acc = part[wk];
      for (size_t i = i0; i < i1; ++i) {
        for (size_t x = 0; x < nl; ++x) {
          lo[x] = lower_t[x][2 * i];
          los[x] = lower_t[x][2 * i + 1] - lo[x];
        }
        for (size_t x = 0; x < nu; ++x) {
          up[x] = upper_t[x][2 * i];
          ups[x] = upper_t[x][2 * i + 1] - up[x];
        }
        if (nv) {
          for (size_t j = bound + 1; j < n; ++j) at[j] = Fr::from_u64((i >> (j - bound - 1)) & 1);
          at[bound] = Fr::zero();
          for (size_t x = 0; x < nv; ++x) vv[x] = virtual_at_point(kinds[x], at);
          at[bound] = Fr::one();
          for (size_t x = 0; x < nv; ++x) vs[x] = virtual_at_point(kinds[x], at) - vv[x];
        }
        Fr e = eq[2 * i], es = eq[2 * i + 1] - eq[2 * i];
        for (int node = 0; node < 4; ++node) {
          acc[node] += e * res.summand(weights, lo.data(), up.data(), vv.data());
          e += es;
          for (size_t x = 0; x < nl; ++x) lo[x] += los[x];
          for (size_t x = 0; x < nu; ++x) up[x] += ups[x];
          for (size_t x = 0; x < nv; ++x) vv[x] += vs[x];
        }
      }
    });
    std::array<Fr, 4> acc = {Fr::zero(), Fr::zero(), Fr::zero(), Fr::zero()};
    for (auto& p : part)
      for (int node = 0; node < 4; ++node) acc[node] += p[node];
    auto g = interpolate_cubic(acc);
    t.append_scalars(tags::SUMCHECK_ROUND, g.data(), 4);
    Fr r = t.challenge(tags::SUMCHECK_CHALLENGE);
    for (auto& tb : lower_t) bind_table(tb, r);
    for (auto& tb : upper_t) bind_table(tb, r);
    bind_table(eq, r);
    rounds.push_back(g);
    point.push_back(r);
  }
  return {rounds, point};
}

inline std::vector<SumcheckProof> gkr_prove(const Circuit& c, const LayerValues& vals, const Challenges& ch, Transcript& t) {
  size_t depth = c.layers.size();
  const auto& top = vals[depth];
  std::vector<Fr> msg;
  for (auto off : c.outputs) msg.insert(msg.end(), top[off].begin(), top[off].end());
  t.append_scalars(tags::GKR_OUTPUTS, msg);
  std::vector<Fr> point;
  for (uint32_t i = 0; i < c.layer_vars(depth); ++i) point.push_back(t.challenge(tags::GKR_OUTPUT_POINT));
  std::vector<SumcheckProof> proofs(depth);
  for (size_t k = depth; k-- > 0;) {
    const LayerSpec& L = c.layers[k];
    Fr lambda = t.challenge(tags::GKR_BATCH);
    std::vector<Fr> weights = powers(lambda, L.producing.size() + L.enforcing.size());
    std::vector<Table> lower, upper;
    if (L.halving) {
      size_t half = (size_t)1 << (c.layer_vars(k) - 1);
      for (auto& col : vals[k]) {
        lower.emplace_back(col.begin(), col.begin() + half);
        upper.emplace_back(col.begin() + half, col.end());
      }
    } else {
      lower = vals[k];
    }
    auto rp = prove_layer_sumcheck(c, k, point, weights, lower, upper, ch, t);
    std::vector<Fr> finals;
    if (L.halving) {
      for (size_t x = 0; x < lower.size(); ++x) {
        finals.push_back(lower[x][0]);
        finals.push_back(upper[x][0]);
      }
    } else {
      for (auto& tb : lower) finals.push_back(tb[0]);
    }
    t.append_scalars(tags::GKR_LAYER_CLAIMS, finals);
    point = rp.second;
    if (L.halving) point.push_back(t.challenge(tags::GKR_CHILD));
    proofs[k].rounds = rp.first;
    proofs[k].final_evals = finals;
  }
  return proofs;
}

}  // namespace oracle
