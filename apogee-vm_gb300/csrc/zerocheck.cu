// Gate zerocheck (crates/sumcheck/src/lib.rs:359-408) on the device sumcheck
// engine, and the witness digest (:228-256) in the host sponge.
//
// The transcript script is the reference's: n eq-randomisers as
// SUMCHECK_CHALLENGE, then per round SUMCHECK_ROUND (4 coefficients) and one
// SUMCHECK_CHALLENGE binding variable i, then SUMCHECK_FINAL_EVALS.
#include "sumcheck.cuh"

namespace apg {

using host::F;

// The zerocheck Gate sum_t coef_t * x_a * x_b (x_b optional) as one Quadratic
// gate over the input slots: constant 0, the single-factor terms as its linear
// part, the two-factor terms as its products.
static HostProgram zerocheck_program(const std::vector<F>& coefs, const uint32_t* ta, const uint32_t* tb,
                                     size_t nterms) {
  HostProgram hp;
  DevGate g;
  memset(&g, 0, sizeof(g));
  g.kind = G_QUADRATIC;
  std::vector<uint16_t> lin_ops, prod_ops;
  std::vector<F> lin_c, prod_c;
  for (size_t t = 0; t < nterms; ++t) {
    if (tb[t] == 0xffffffffu) {
      lin_ops.push_back((uint16_t)ta[t]);
      lin_c.push_back(coefs[t]);
    } else {
      prod_ops.push_back((uint16_t)ta[t]);
      prod_ops.push_back((uint16_t)tb[t]);
      prod_c.push_back(coefs[t]);
    }
  }
  g.p1 = (uint16_t)lin_ops.size();
  g.p2 = (uint16_t)prod_c.size();
  g.nops = (uint16_t)(lin_ops.size() + prod_ops.size());
  g.op_off = 0;
  g.cf_off = 0;
  hp.ops = lin_ops;
  hp.ops.insert(hp.ops.end(), prod_ops.begin(), prod_ops.end());
  hp.coeffs.push_back(host::fzero());
  hp.coeffs.insert(hp.coeffs.end(), lin_c.begin(), lin_c.end());
  hp.coeffs.insert(hp.coeffs.end(), prod_c.begin(), prod_c.end());
  hp.gates.push_back(g);
  hp.weights.push_back(host::fone());
  hp.n_cached = 0;
  hp.n_weighted = 1;
  return hp;
}

static bool read_mem_fr(const uint8_t* p, F& out) {
  memcpy(out.w, p, 32);
  return host::below_p(out.w);
}

int prove_zerocheck_impl(Ctx& c, size_t arity, const uint8_t* coefs, const uint32_t* ta, const uint32_t* tb,
                         size_t nterms, const uint8_t* const* polys, bool polys_on_device, size_t num_vars,
                         uint8_t* transcript, uint8_t* rounds_out, uint8_t* finals_out, const uint8_t* bits) {
  if (arity == 0) {
    c.last_error = "a gate with no inputs";
    return APG_ERR_INVALID_ARGUMENT;
  }
  if (!polys || !transcript || !rounds_out || !finals_out || (nterms && (!coefs || !ta || !tb)))
    return APG_ERR_INVALID_ARGUMENT;
  if (num_vars > 40) return APG_ERR_INVALID_ARGUMENT;
  std::vector<F> cf(nterms);
  for (size_t t = 0; t < nterms; ++t) {
    if (!read_mem_fr(coefs + 32 * t, cf[t])) return APG_ERR_NONCANONICAL;
    if (ta[t] >= arity || (tb[t] != 0xffffffffu && tb[t] >= arity)) {
      c.last_error = "a gate term names an undeclared input";
      return APG_ERR_INVALID_ARGUMENT;
    }
  }
  host::Transcript tr;
  if (!tr.load(transcript)) {
    c.last_error = "malformed transcript snapshot";
    return APG_ERR_INVALID_ARGUMENT;
  }
  const size_t n = (size_t)1 << num_vars;
  // Stored widths (empty: all Fr). Narrow tables cross and stay narrow; the
  // first bind lifts them (crates/poly/src/lib.rs:156-185).
  std::vector<uint8_t> src_bits;
  if (bits) {
    for (size_t k = 0; k < arity; ++k)
      if (!narrow_bits_ok(bits[k])) {
        c.last_error = "a column width other than 0, 1, 8, 16, 32";
        return APG_ERR_INVALID_ARGUMENT;
      }
    src_bits.assign(bits, bits + arity);
  }
  std::vector<const Fr*> src(arity);
  for (size_t k = 0; k < arity; ++k)
    if (!polys[k]) return APG_ERR_INVALID_ARGUMENT;
  if (polys_on_device) {
    for (size_t k = 0; k < arity; ++k) src[k] = (const Fr*)polys[k];
  } else {
    std::vector<size_t> off(arity);
    size_t total = 0;
    for (size_t k = 0; k < arity; ++k) {
      off[k] = total;
      total += (narrow_bytes(bits ? bits[k] : 0, n) + 255) / 256 * 256;
    }
    uint8_t* d = c.scratch[S_SCALARS].as<uint8_t>(total);
    for (size_t k = 0; k < arity; ++k) {
      APG_CUDA(cudaMemcpyAsync(d + off[k], polys[k], narrow_bytes(bits ? bits[k] : 0, n), cudaMemcpyHostToDevice,
                               c.stream));
      src[k] = reinterpret_cast<const Fr*>(d + off[k]);
    }
  }
  std::vector<F> r(num_vars);
  for (size_t j = 0; j < num_vars; ++j) r[j] = tr.challenge(host::T_SUMCHECK_CHALLENGE);
  HostProgram hp = zerocheck_program(cf, ta, tb, nterms);
  DevProgram P;
  upload_program(c, hp, P, 0);
  std::vector<std::array<F, 4>> rounds;
  std::vector<F> point, finals;
  HostPairTerms pairs;
  const bool by_pairs = pair_terms_of(hp, (int)arity, pairs);
  run_sumcheck(c, P, (int)arity, {}, 0, src, r, tr, rounds, point, finals, src_bits, by_pairs ? &pairs : nullptr);
  for (auto& f : finals)
    if (!host::below_p(f.w)) throw Error(APG_ERR_INTERNAL, "non-canonical device value");
  tr.absorb(host::T_SUMCHECK_FINAL_EVALS, finals);
  for (size_t i = 0; i < rounds.size(); ++i) memcpy(rounds_out + 128 * i, rounds[i].data(), 128);
  memcpy(finals_out, finals.data(), 32 * finals.size());
  tr.save(transcript);
  c.check_flags();
  return APG_OK;
}

int witness_digest_impl(Ctx& c, const uint8_t* const* cols, size_t k, size_t num_vars, uint8_t out[32]) {
  if (!cols || !out || k == 0) return APG_ERR_INVALID_ARGUMENT;
  host::Transcript sponge;
  F hdr[2] = {host::from_u64(k), host::from_u64(num_vars)};
  sponge.absorb(host::T_WITNESS_DIGEST, hdr, 2);
  const size_t n = (size_t)1 << num_vars;
  std::vector<F> cells(n);
  for (size_t j = 0; j < k; ++j) {
    for (size_t i = 0; i < n; ++i)
      if (!read_mem_fr(cols[j] + 32 * i, cells[i])) return APG_ERR_NONCANONICAL;
    sponge.absorb(host::T_WITNESS_DIGEST, cells);
  }
  F d = sponge.sample();
  memcpy(out, d.w, 32);
  (void)c;
  return APG_OK;
}

}  // namespace apg
