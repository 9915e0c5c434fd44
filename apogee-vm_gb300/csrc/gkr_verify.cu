// The verifiers on the host: gkr_verify::verify
// (crates/gkr-verify/src/lib.rs:647-748) over a circuit in its APGC form and
// a proof as apg_gkr_prove writes it, and sumcheck::verify_zerocheck
// (crates/sumcheck/src/lib.rs:418-473) over a proof as apg_prove_zerocheck
// writes it.
//
// Every step is a few field products a round except the first: the output
// tables are absorbed into the transcript (one Poseidon2 permutation per two
// values, a serial chain) and evaluated at the output point (one fold per
// variable). Nothing here touches a device.
//
// Order of the checks, as the reference's: every challenge slot a gate names
// (MissingChallenge), the output tables' count and size (OutputShape), the
// proof's size layer by layer (ProofShape), then the transcript schedule O1,
// O2, and per gate list from the top L1 (GKR_BATCH), L2 (the rounds, each
// g(0) + g(1) against the running claim), L3 (GKR_LAYER_CLAIMS), the final
// check eq(p, rho) S(claims) against the last round's value
// (LayerInconsistency), L4 (GKR_CHILD for a halving list).
#include "sumcheck.cuh"

namespace apg {

using host::F;

namespace {

F coeff(const CGate& G, size_t i, const Challenges& ch) {
  return G.coeffs[i].first ? ch.get(G.slots[i]) : G.coeffs[i].second;
}

// sum_i c[c0 + i] v[i] + c[c0 + t]: the affine form of Linear and of the two
// sides of AffineProduct (coefficients in GateDef::coefficients order: the
// terms' then the constant).
F affine(const CGate& G, const Challenges& ch, size_t c0, size_t t, const F* v) {
  F acc = coeff(G, c0 + t, ch);
  for (size_t i = 0; i < t; ++i) acc = host::fadd(acc, host::fmul(coeff(G, c0 + i, ch), v[i]));
  return acc;
}

// eval_gate (lib.rs:142-202): one value per operand, two per column operand
// of a tree gate (child 0, child 1).
F eval_gate(const CGate& G, const F* v, const Challenges& ch) {
  switch (G.kind) {
    case G_LINEAR:
      return affine(G, ch, 0, G.p1, v);
    case G_PRODUCT:
      return host::fmul(host::fmul(coeff(G, 0, ch), v[0]), v[1]);
    case G_MASK:
      return host::fsub(host::fadd(host::fmul(v[0], v[1]), host::fone()), v[1]);
    case G_AFFINE:
      return host::fmul(affine(G, ch, 0, G.p1, v), affine(G, ch, G.p1 + 1, G.p2, v + G.p1));
    case G_TREE_PRODUCT:
      return host::fmul(v[0], v[1]);
    case G_TREE_CROSS:
      return host::fadd(host::fmul(v[0], v[3]), host::fmul(v[1], v[2]));
    case G_QUADRATIC: {
      const size_t t = G.p1, u = G.p2;
      F acc = coeff(G, 0, ch);
      for (size_t i = 0; i < t; ++i) acc = host::fadd(acc, host::fmul(coeff(G, 1 + i, ch), v[i]));
      for (size_t j = 0; j < u; ++j)
        acc = host::fadd(acc, host::fmul(coeff(G, 1 + t + j, ch), host::fmul(v[t + 2 * j], v[t + 2 * j + 1])));
      return acc;
    }
  }
  throw Error(APG_ERR_BAD_CIRCUIT, "unknown gate kind");
}

// sum_j 2^j y_j over y[lo, hi) of the point, by Horner from the top.
F horner(const std::vector<F>& y, size_t lo, size_t hi) {
  F acc = host::fzero();
  for (size_t j = hi; j-- > lo;) acc = host::fadd(host::fadd(acc, acc), y[j]);
  return acc;
}

// y[j], or zero past the point's end.
F coord(const std::vector<F>& y, size_t j) { return j < y.size() ? y[j] : host::fzero(); }

// virtual_at_point (lib.rs:241-286): each table's multilinear extension.
F virtual_at_point(uint32_t kind, const std::vector<F>& y) {
  const size_t n = y.size();
  switch (kind) {
    case V_ROW:
      return horner(y, 0, n);
    case V_RAM_LIVE: {
      F prod = host::fone();
      for (size_t j = 14; j < n; ++j) prod = host::fmul(prod, host::fsub(host::fone(), y[j]));
      return host::fsub(host::fone(), prod);
    }
    case V_RANGE19:
      return horner(y, 0, std::min<size_t>(n, 19));
    case V_RANGE16:
      return horner(y, 0, std::min<size_t>(n, 16));
    case V_XOR8A:
    case V_XOR8B: {
      const size_t first = kind == V_XOR8A ? 0 : 8;
      F acc = host::fzero();
      for (size_t j = 8; j-- > 0;) acc = host::fadd(host::fadd(acc, acc), coord(y, first + j));
      return acc;
    }
    case V_XOR8OUT: {
      F acc = host::fzero();
      for (size_t j = 8; j-- > 0;) {
        const F a = coord(y, j), b = coord(y, j + 8), ab = host::fmul(a, b);
        acc = host::fsub(host::fadd(host::fadd(acc, acc), host::fadd(a, b)), host::fadd(ab, ab));
      }
      return acc;
    }
  }
  throw Error(APG_ERR_BAD_CIRCUIT, "unknown virtual kind");
}

// The weighted sum of gate list k's producing then enforcing gates at one
// point (summand, lib.rs:512-528, through ResolvedList's operand order):
// cached entries first, each reading columns, virtual tables and earlier
// cached entries; a halving list's gates read every column at child 0 then
// child 1 (lower, upper).
F summand(const Circuit& C, size_t k, const std::vector<F>& weights, const std::vector<F>& lower,
          const std::vector<F>& upper, const std::vector<F>& virt, const Challenges& ch) {
  const CLayer& L = C.layers[k];
  std::vector<F> cached, ops;
  auto eval = [&](const CGate& G) {
    ops.clear();
    for (auto& op : G.ops) {
      if (L.halving) {
        ops.push_back(lower[op.second]);
        ops.push_back(upper[op.second]);
      } else if (op.first == 0) {
        ops.push_back(lower[op.second]);
      } else if (op.first == 1) {
        ops.push_back(virt[op.second]);
      } else {
        ops.push_back(cached[op.second]);
      }
    }
    return eval_gate(G, ops.data(), ch);
  };
  for (auto& G : L.cached) cached.push_back(eval(G));
  F acc = host::fzero();
  size_t j = 0;
  for (auto* list : {&L.producing, &L.enforcing})
    for (auto& G : *list) {
      acc = host::fadd(acc, host::fmul(eval(G), weights[j]));
      ++j;
    }
  return acc;
}

// An ascending-coefficient cubic at x, by Horner.
F cubic(const F g[4], const F& x) {
  F acc = g[3];
  for (int i = 2; i >= 0; --i) acc = host::fadd(host::fmul(acc, x), g[i]);
  return acc;
}

// prod_i (p_i r_i + (1 - p_i)(1 - r_i)).
F eq_eval(const std::vector<F>& p, const std::vector<F>& r) {
  F acc = host::fone();
  for (size_t i = 0; i < p.size(); ++i) {
    const F pr = host::fmul(p[i], r[i]);
    // p r + (1 - p)(1 - r) = 1 - p - r + 2 p r
    F t = host::fsub(host::fsub(host::fone(), p[i]), r[i]);
    t = host::fadd(t, host::fadd(pr, pr));
    acc = host::fmul(acc, t);
  }
  return acc;
}

// A table's multilinear extension at the point, variable 0 the low bit of the
// row index: fold the table one variable at a time.
F evaluate(std::vector<F> t, const std::vector<F>& point) {
  for (size_t v = 0; v < point.size(); ++v) {
    const size_t half = t.size() / 2;
    for (size_t i = 0; i < half; ++i)
      t[i] = host::fadd(t[2 * i], host::fmul(point[v], host::fsub(t[2 * i + 1], t[2 * i])));
    t.resize(half);
  }
  return t[0];
}

F read_fr(const uint8_t* p) {
  F x;
  memcpy(x.w, p, 32);
  if (!host::below_p(x.w)) throw Error(APG_ERR_NONCANONICAL, "a field element is not below the modulus");
  return x;
}

}  // namespace

int gkr_verify_impl(const uint8_t* blob, size_t blob_len, const uint8_t* const* outputs, const size_t* output_lens,
                    size_t n_outputs, const uint8_t* proof, size_t proof_len, const uint32_t* slots,
                    const uint8_t* slot_values, size_t n_slots, uint8_t* transcript, uint8_t* point_out,
                    uint8_t* values_out, uint64_t* info) {
  if (info) *info = 0;
  if (!transcript || !point_out || !values_out || (n_slots && (!slots || !slot_values)) ||
      (n_outputs && (!outputs || !output_lens)) || (proof_len && !proof))
    return APG_ERR_INVALID_ARGUMENT;
  const Circuit C = parse_circuit_blob(blob, blob_len);
  const Challenges ch = read_challenges(slots, slot_values, n_slots);
  auto fail = [&](int status, uint64_t what) {
    if (info) *info = what;
    return status;
  };

  // check_challenges (lib.rs:575-598): the first slot a gate names that the
  // caller left out, lists bottom up, cached then producing then enforcing.
  for (auto& L : C.layers)
    for (auto* list : {&L.cached, &L.producing, &L.enforcing})
      for (auto& G : *list)
        for (size_t i = 0; i < G.coeffs.size(); ++i)
          if (G.coeffs[i].first && !ch.has(G.slots[i])) return fail(APG_ERR_MISSING_CHALLENGE, G.slots[i]);

  const size_t depth = C.layers.size();
  const size_t top_vars = C.vars(depth);
  const size_t top_rows = (size_t)1 << top_vars;
  if (n_outputs != C.outputs.size()) return fail(APG_ERR_OUTPUT_SHAPE, 0);
  for (size_t i = 0; i < n_outputs; ++i)
    if (output_lens[i] != top_rows || !outputs[i]) return fail(APG_ERR_OUTPUT_SHAPE, 0);

  // The proof's layout, gate list 0 first: 4 Fr per round, then the claims.
  std::vector<size_t> seg(depth + 1, 0);
  for (size_t k = 0; k < depth; ++k)
    seg[k + 1] = seg[k] + 32 * (4 * (size_t)C.vars(k + 1) + (C.layers[k].halving ? 2 : 1) * (size_t)C.width(k));
  for (size_t k = 0; k < depth; ++k)
    if (proof_len < seg[k + 1]) return fail(APG_ERR_PROOF_SHAPE, k);
  if (proof_len != seg[depth]) return fail(APG_ERR_PROOF_SHAPE, depth);

  host::Transcript tr;
  if (!tr.load(transcript)) return APG_ERR_INVALID_ARGUMENT;

  // O1: the outputs, one message; O2: the point they are claimed at.
  std::vector<std::vector<F>> tables(n_outputs);
  {
    std::vector<F> msg;
    msg.reserve(n_outputs * top_rows);
    for (size_t i = 0; i < n_outputs; ++i) {
      tables[i].resize(top_rows);
      for (size_t r = 0; r < top_rows; ++r) tables[i][r] = read_fr(outputs[i] + 32 * r);
      msg.insert(msg.end(), tables[i].begin(), tables[i].end());
    }
    tr.absorb(host::T_GKR_OUTPUTS, msg);
  }
  std::vector<F> point;
  for (size_t i = 0; i < top_vars; ++i) point.push_back(tr.challenge(host::T_GKR_OUTPUT_POINT));
  // The output map places each table at its top-layer offset; a validated
  // artifact's offsets cover the outputs' own index range.
  for (auto o : C.outputs)
    if (o >= C.outputs.size()) throw Error(APG_ERR_BAD_CIRCUIT, "an output offset lies past the output count");
  std::vector<F> values(C.outputs.size(), host::fzero());
  for (size_t i = 0; i < n_outputs; ++i) values[C.outputs[i]] = evaluate(tables[i], point);

  for (size_t k = depth; k-- > 0;) {
    const CLayer& L = C.layers[k];
    const uint8_t* part = proof + seg[k];
    const size_t nv = C.vars(k + 1);
    // L1: the batch and its powers.
    const F lambda = tr.challenge(host::T_GKR_BATCH);
    std::vector<F> weights;
    F acc = host::fone();
    for (size_t j = 0; j < L.producing.size() + L.enforcing.size(); ++j) {
      weights.push_back(acc);
      acc = host::fmul(acc, lambda);
    }
    F claim = host::fzero();
    for (size_t j = 0; j < values.size() && j < weights.size(); ++j)
      claim = host::fadd(claim, host::fmul(values[j], weights[j]));
    // L2: verify_sumcheck (lib.rs:613-631).
    std::vector<F> rho;
    for (size_t i = 0; i < nv; ++i) {
      F g[4];
      for (int e = 0; e < 4; ++e) g[e] = read_fr(part + 32 * (4 * i + e));
      if (host::fadd(cubic(g, host::fzero()), cubic(g, host::fone())) != claim)
        return fail(APG_ERR_LAYER_INCONSISTENCY, k);
      tr.absorb(host::T_SUMCHECK_ROUND, g, 4);
      const F r = tr.challenge(host::T_SUMCHECK_CHALLENGE);
      claim = cubic(g, r);
      rho.push_back(r);
    }
    // L3: the claims, then the final check.
    const size_t nclaims = (L.halving ? 2 : 1) * (size_t)C.width(k);
    std::vector<F> evals(nclaims);
    for (size_t i = 0; i < nclaims; ++i) evals[i] = read_fr(part + 32 * (4 * nv + i));
    tr.absorb(host::T_GKR_LAYER_CLAIMS, evals);
    F s;
    if (L.halving) {
      std::vector<F> lower, upper;
      for (size_t i = 0; i < nclaims; i += 2) {
        lower.push_back(evals[i]);
        upper.push_back(evals[i + 1]);
      }
      s = summand(C, k, weights, lower, upper, {}, ch);
    } else {
      std::vector<F> virt;
      for (auto kind : C.virtuals) virt.push_back(virtual_at_point(kind, rho));
      s = summand(C, k, weights, evals, {}, virt, ch);
    }
    if (claim != host::fmul(eq_eval(point, rho), s)) return fail(APG_ERR_LAYER_INCONSISTENCY, k);
    // L4: a halving list's children meet on one line.
    if (L.halving) {
      const F tau = tr.challenge(host::T_GKR_CHILD);
      values.clear();
      for (size_t i = 0; i < nclaims; i += 2)
        values.push_back(host::fadd(evals[i], host::fmul(tau, host::fsub(evals[i + 1], evals[i]))));
      point = rho;
      point.push_back(tau);
    } else {
      values = evals;
      point = rho;
    }
  }
  // The base claims: every committed column at one point.
  memcpy(point_out, point.data(), 32 * point.size());
  memcpy(values_out, values.data(), 32 * values.size());
  tr.save(transcript);
  return APG_OK;
}

// sumcheck::verify_zerocheck (crates/sumcheck/src/lib.rs:418-473): the round
// and final counts, the n point challenges drawn up front (the eq point r),
// each round's g(0) + g(1) against the claim (zero in round 0), the finals
// absorbed, then eq(r, point) G(finals) against the last claim. `info`
// receives the count found or the failing round.
int verify_zerocheck_impl(size_t arity, const uint8_t* coefs, const uint32_t* ta, const uint32_t* tb, size_t nterms,
                          size_t num_vars, const uint8_t* rounds, size_t n_rounds, const uint8_t* finals,
                          size_t n_finals, uint8_t* transcript, uint8_t* point_out, uint64_t* info) {
  if (info) *info = 0;
  if (arity == 0 || !transcript || !point_out || (nterms && (!coefs || !ta || !tb)) || (n_rounds && !rounds) ||
      (n_finals && !finals))
    return APG_ERR_INVALID_ARGUMENT;
  std::vector<F> cf(nterms);
  for (size_t t = 0; t < nterms; ++t) {
    cf[t] = read_fr(coefs + 32 * t);
    if (ta[t] >= arity || (tb[t] != 0xffffffffu && tb[t] >= arity)) return APG_ERR_INVALID_ARGUMENT;
  }
  auto fail = [&](int status, uint64_t what) {
    if (info) *info = what;
    return status;
  };
  if (n_rounds != num_vars) return fail(APG_ERR_ROUND_COUNT_MISMATCH, n_rounds);
  if (n_finals != arity) return fail(APG_ERR_FINAL_COUNT_MISMATCH, n_finals);
  std::vector<std::array<F, 4>> g(n_rounds);
  for (size_t i = 0; i < n_rounds; ++i)
    for (int e = 0; e < 4; ++e) g[i][e] = read_fr(rounds + 32 * (4 * i + e));
  std::vector<F> fin(n_finals);
  for (size_t k = 0; k < n_finals; ++k) fin[k] = read_fr(finals + 32 * k);

  host::Transcript tr;
  if (!tr.load(transcript)) return APG_ERR_INVALID_ARGUMENT;
  std::vector<F> r;
  for (size_t i = 0; i < num_vars; ++i) r.push_back(tr.challenge(host::T_SUMCHECK_CHALLENGE));
  F claim = host::fzero();
  std::vector<F> point;
  for (size_t i = 0; i < n_rounds; ++i) {
    if (host::fadd(cubic(g[i].data(), host::fzero()), cubic(g[i].data(), host::fone())) != claim)
      return fail(APG_ERR_ROUND_SUM_MISMATCH, i);
    tr.absorb(host::T_SUMCHECK_ROUND, g[i].data(), 4);
    const F c = tr.challenge(host::T_SUMCHECK_CHALLENGE);
    claim = cubic(g[i].data(), c);
    point.push_back(c);
  }
  tr.absorb(host::T_SUMCHECK_FINAL_EVALS, fin);
  // Gate::evaluate (lib.rs:151-165): sum_t coef_t x_a (x_b).
  F gate = host::fzero();
  for (size_t t = 0; t < nterms; ++t) {
    F term = host::fmul(cf[t], fin[ta[t]]);
    if (tb[t] != 0xffffffffu) term = host::fmul(term, fin[tb[t]]);
    gate = host::fadd(gate, term);
  }
  if (host::fmul(eq_eval(r, point), gate) != claim) return fail(APG_ERR_FINAL_EVAL_MISMATCH, 0);
  memcpy(point_out, point.data(), 32 * point.size());
  tr.save(transcript);
  return APG_OK;
}

}  // namespace apg
