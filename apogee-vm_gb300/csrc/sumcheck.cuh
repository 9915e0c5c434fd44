// Shared declarations of the sumcheck engine (sumcheck.cu) and its callers
// (the zerocheck and GKR entry points).
#pragma once
#include <array>

#include "common.cuh"
#include "host_fr.hpp"
#include "summand.cuh"

namespace apg {

// A resolved gate list as the host builds it. Slot numbering: data tables
// [0, nd), virtual tables [nd, nd + nv), cached entries after them.
struct HostProgram {
  std::vector<DevGate> gates;
  std::vector<uint16_t> ops;
  std::vector<host::F> coeffs;
  std::vector<host::F> weights;
  int n_cached = 0;
  int n_weighted = 0;
  // The weighted gates are only summed (a sumcheck's summand), never read one
  // by one (the forward pass writes gate j to column j): they may be
  // reordered.
  bool summed = false;
};

// Stored widths of a committed column (PolyBacking, crates/poly/src/lib.rs:44-57):
// 0 Fr in memory, 1 a bitset (u64 limbs, entry i = bit i % 64 of limb i / 64),
// 8 / 16 / 32 unsigned integers.
inline bool narrow_bits_ok(int bits) { return bits == 0 || bits == 1 || bits == 8 || bits == 16 || bits == 32; }
// Bytes a column of n entries takes at that width.
inline size_t narrow_bytes(int bits, size_t n) {
  return bits == 0 ? 32 * n : bits == 1 ? 8 * ((n + 63) / 64) : (size_t)(bits / 8) * n;
}

// Entry i of a column in its stored width, lifted into Montgomery Fr: the one
// lift of PolyBacking::entry (crates/poly/src/lib.rs:72-88).
__device__ __forceinline__ Fr narrow_entry(const void* p, int bits, size_t i) {
  uint32_t v;
  switch (bits) {
    case 0:
      return ld_fe(reinterpret_cast<const Fr*>(p) + i);
    case 1:
      return (reinterpret_cast<const uint64_t*>(p)[i >> 6] >> (i & 63)) & 1 ? fe_one<FrConsts>()
                                                                             : fe_zero<FrConsts>();
    case 8:
      v = reinterpret_cast<const uint8_t*>(p)[i];
      break;
    case 16:
      v = reinterpret_cast<const uint16_t*>(p)[i];
      break;
    default:
      v = reinterpret_cast<const uint32_t*>(p)[i];
      break;
  }
  Fr r = fe_zero<FrConsts>();
  r.v[0] = v;
  return fe_to_mont(r);
}

// The first n entries of a column, lifted into an Fr table.
void lift_column(Ctx& c, const void* p, int bits, size_t n, Fr* out);

void upload_program(Ctx& c, const HostProgram& hp, DevProgram& P, int slot_cap);
void build_eq_table(Ctx& c, const std::vector<host::F>& r, Fr* out);

// Prove sum_y eq(eq_point, y) * S(y) over `src` tables (nd of them, each
// 2^|eq_point| entries, device memory), drawing challenges from `tr`. Returns
// the rounds' ascending coefficients, the bound point and each data table's
// final value.
// `src_bits` (empty: every table Fr) gives each data table's stored width;
// narrow tables are read through the lift in the first two rounds and the
// first bind writes Fr (the lazy lift of crates/poly/src/lib.rs:156-185).
// A summand that is a weighted sum of products of two data tables,
// S = sum_j c_j T_{a_j} T_{b_j} (halving lists of TreeProduct / TreeCross
// gates, a zerocheck's product gate): the round kernel for it reads each
// term's two lines and multiplies, with no interpreter between. `rest` lists
// the data tables no term reads (they are still bound every round).
struct HostPairTerms {
  std::vector<uint16_t> a, b, rest;
  std::vector<host::F> c;
};
// The program's terms, when every weighted gate is such a product of data
// tables (slots below nd) and nothing is cached; false otherwise.
bool pair_terms_of(const HostProgram& hp, int nd, HostPairTerms& out);

void run_sumcheck(Ctx& c, const DevProgram& prog, int nd, const std::vector<uint8_t>& vkinds, int n_cached,
                  const std::vector<const Fr*>& src, const std::vector<host::F>& eq_point, host::Transcript& tr,
                  std::vector<std::array<host::F, 4>>& rounds, std::vector<host::F>& point,
                  std::vector<host::F>& finals, const std::vector<uint8_t>& src_bits = {},
                  const HostPairTerms* pairs = nullptr);

// `bits` (null: all Fr) is each table's stored width.
int prove_zerocheck_impl(Ctx& c, size_t arity, const uint8_t* coefs, const uint32_t* ta, const uint32_t* tb,
                         size_t nterms, const uint8_t* const* polys, bool polys_on_device, size_t num_vars,
                         uint8_t* transcript, uint8_t* rounds_out, uint8_t* finals_out,
                         const uint8_t* bits = nullptr);
int witness_digest_impl(Ctx& c, const uint8_t* const* cols, size_t k, size_t num_vars, uint8_t out[32]);

// ---- a circuit in its resolved (APGC) form -------------------------------------

struct CGate {
  uint32_t kind, p1, p2;
  std::vector<std::pair<uint32_t, uint32_t>> ops;  // (source, index)
  std::vector<std::pair<bool, host::F>> coeffs;    // (is_challenge, literal value)
  std::vector<uint32_t> slots;                     // challenge slots (parallel to coeffs)
};
struct CLayer {
  bool halving;
  uint32_t num_vars, width;
  std::vector<CGate> cached, producing, enforcing;
};
struct Circuit {
  uint32_t trace_vars = 0, n_committed = 0;
  std::vector<uint32_t> virtuals, outputs;
  std::vector<CLayer> layers;
  uint32_t vars(size_t k) const { return k == 0 ? trace_vars : layers[k - 1].num_vars; }
  uint32_t width(size_t k) const { return k == 0 ? n_committed : layers[k - 1].width; }
};

// The external challenges, slot -> value (Fr in memory).
struct Challenges {
  std::vector<std::pair<uint32_t, host::F>> kv;
  bool has(uint32_t slot) const {
    for (auto& p : kv)
      if (p.first == slot) return true;
    return false;
  }
  host::F get(uint32_t slot) const {
    for (auto& p : kv)
      if (p.first == slot) return p.second;
    throw Error(APG_ERR_INVALID_ARGUMENT, "external challenge slot " + std::to_string(slot) + " has no value");
  }
};
// Values below p or APG_ERR_NONCANONICAL.
Challenges read_challenges(const uint32_t* slots, const uint8_t* values, size_t n);

struct GkrValues;
Circuit parse_circuit_blob(const uint8_t* blob, size_t len);
size_t gkr_proof_elems(const Circuit& C);
// `bits` (null: all Fr) is each base column's stored width.
GkrValues* gkr_forward_impl(Ctx& c, const uint8_t* blob, size_t blob_len, const void* const* base,
                            const uint8_t* bits, bool base_on_device, const uint32_t* slots,
                            const uint8_t* slot_values, size_t n_slots);
int gkr_prove_impl(Ctx& c, const uint8_t* blob, size_t blob_len, GkrValues* V, const uint32_t* slots,
                   const uint8_t* slot_values, size_t n_slots, uint8_t* transcript, uint8_t* proof_out,
                   size_t proof_cap, size_t* proof_len, uint8_t* point_out);
int gkr_prove_sumcheck_impl(Ctx& c, const uint8_t* blob, size_t blob_len, size_t layer, const uint8_t* weights,
                            size_t n_weights, const uint32_t* slots, const uint8_t* slot_values, size_t n_slots,
                            const uint8_t* eq_point, size_t n, const void* const* d_lower,
                            const void* const* d_upper, size_t width, uint8_t* transcript, uint8_t* rounds_out,
                            uint8_t* point_out, uint8_t* finals_out);
void gkr_values_free(GkrValues* v);
int gkr_values_read_impl(GkrValues* v, size_t layer, size_t col, uint8_t* out);
size_t gkr_values_len(GkrValues* v, size_t layer);
size_t gkr_proof_len_impl(const uint8_t* blob, size_t len);
size_t gkr_device_bytes_impl(const uint8_t* blob, size_t len);
// gkr_verify::verify on the host; `info` receives the failing slot or layer.
int gkr_verify_impl(const uint8_t* blob, size_t blob_len, const uint8_t* const* outputs, const size_t* output_lens,
                    size_t n_outputs, const uint8_t* proof, size_t proof_len, const uint32_t* slots,
                    const uint8_t* slot_values, size_t n_slots, uint8_t* transcript, uint8_t* point_out,
                    uint8_t* values_out, uint64_t* info);
// sumcheck::verify_zerocheck on the host; `info` receives a count or a round.
int verify_zerocheck_impl(size_t arity, const uint8_t* coefs, const uint32_t* ta, const uint32_t* tb, size_t nterms,
                          size_t num_vars, const uint8_t* rounds, size_t n_rounds, const uint8_t* finals,
                          size_t n_finals, uint8_t* transcript, uint8_t* point_out, uint64_t* info);

int mercury_open_impl(Ctx& c, const Fr* d_f, size_t nv, const uint8_t cm[64], const std::vector<host::F>& u,
                      host::Transcript& tr, host::F& v_out, uint8_t proof_out[704]);
// pcs::verify_deferred / batch_verify_deferred on the host: the twelve
// accumulator entries (sides, scalars in memory, canonical points).
int mercury_verify_deferred_impl(const uint8_t cm[64], const uint8_t* u, size_t u_len, const uint8_t v[32],
                                 const uint8_t proof[704], uint8_t* transcript, uint8_t* sides, uint8_t* scalars,
                                 uint8_t* points, uint64_t* info);
int mercury_batch_verify_deferred_impl(const uint8_t* cms, size_t k, const uint8_t* u, size_t u_len,
                                       const uint8_t* vs, size_t n_vs, const uint8_t proof[704], uint8_t* transcript,
                                       uint8_t* sides, uint8_t* scalars, uint8_t* points, uint64_t* info);
// The pairing (host): e(P, Q), a product check, and the verifiers built on it.
int pairing_impl(const uint8_t p[64], const uint8_t q[128], uint8_t out[384]);
int pairing_check_impl(const uint8_t* ps, const uint8_t* qs, size_t n, int* holds);
int g2_mul_impl(const uint8_t q[128], const uint8_t k[32], uint8_t out[128]);
int mercury_verify_impl(const uint8_t vsrs[320], const uint8_t cm[64], const uint8_t* u, size_t u_len,
                        const uint8_t v[32], const uint8_t proof[704], uint8_t* transcript, uint64_t* info);
int mercury_batch_verify_impl(const uint8_t vsrs[320], const uint8_t* cms, size_t k, const uint8_t* u, size_t u_len,
                              const uint8_t* vs, size_t n_vs, const uint8_t proof[704], uint8_t* transcript,
                              uint64_t* info);
int discharge_pairing_impl(const uint8_t vsrs[320], const uint8_t a[64], const uint8_t b[64]);
int mercury_batch_open_stacked_impl(Ctx& c, const Fr* const* d_cols, const size_t* stack_lens, size_t nstacks,
                                    size_t width, const uint8_t* cms, const std::vector<host::F>& u,
                                    const std::vector<host::F>& r, host::Transcript& tr,
                                    std::vector<host::F>& vs, uint8_t proof_out[704]);

}  // namespace apg
