// GKR on the device: the forward pass materialises every layer (one thread
// per row through the gate-list interpreter) and the backward pass runs one
// device sumcheck per gate list, top down, with the reference's transcript
// schedule.
//
// Restates crates/gkr/src/lib.rs: forward / produce (:279-336), prove
// (:933-1016: O1 GKR_OUTPUTS, O2 GKR_OUTPUT_POINT, L1 GKR_BATCH lambda,
// L2 the layer sumcheck, L3 GKR_LAYER_CLAIMS, L4 GKR_CHILD), children
// (:910-919) and the summand of prove_sumcheck (:792-899) through
// ResolvedList (crates/gkr-verify/src/lib.rs:315-480).
//
// Circuits arrive as the library's compact resolved form (the "APGC" blob;
// the layout is documented in include/apogee_gpu.h), which this file
// validates before anything touches the device.
#include "sumcheck.cuh"

namespace apg {

using host::F;

namespace {

struct Cursor {
  const uint8_t* p;
  const uint8_t* end;
  uint32_t u32() {
    if (end - p < 4) throw Error(APG_ERR_BAD_CIRCUIT, "circuit blob truncated");
    uint32_t v;
    memcpy(&v, p, 4);
    p += 4;
    return v;
  }
  F fr() {
    if (end - p < 32) throw Error(APG_ERR_BAD_CIRCUIT, "circuit blob truncated");
    F x;
    if (!host::from_bytes(p, x)) throw Error(APG_ERR_BAD_CIRCUIT, "non-canonical coefficient");
    p += 32;
    return x;
  }
};

size_t expected_operands(const CGate& g) {
  switch (g.kind) {
    case G_LINEAR: return g.p1;
    case G_PRODUCT: case G_MASK: case G_TREE_CROSS: return 2;
    case G_AFFINE: return g.p1 + g.p2;
    case G_TREE_PRODUCT: return 1;
    case G_QUADRATIC: return g.p1 + 2 * (size_t)g.p2;
  }
  throw Error(APG_ERR_BAD_CIRCUIT, "unknown gate kind");
}

size_t expected_coeffs(const CGate& g) {
  switch (g.kind) {
    case G_LINEAR: return g.p1 + 1;
    case G_PRODUCT: return 1;
    case G_MASK: case G_TREE_PRODUCT: case G_TREE_CROSS: return 0;
    case G_AFFINE: return g.p1 + g.p2 + 2;
    case G_QUADRATIC: return 1 + g.p1 + g.p2;
  }
  throw Error(APG_ERR_BAD_CIRCUIT, "unknown gate kind");
}

}  // namespace

Circuit parse_circuit_blob(const uint8_t* blob, size_t len) {
  if (!blob) throw Error(APG_ERR_INVALID_ARGUMENT, "null circuit");
  Cursor r{blob, blob + len};
  if (r.u32() != 0x43475041u || r.u32() != 1) throw Error(APG_ERR_BAD_CIRCUIT, "not an APGC v1 circuit");
  Circuit c;
  c.trace_vars = r.u32();
  c.n_committed = r.u32();
  if (c.trace_vars > 40 || c.n_committed == 0) throw Error(APG_ERR_BAD_CIRCUIT, "bad base shape");
  const uint32_t nv = r.u32();
  if (nv > 7) throw Error(APG_ERR_BAD_CIRCUIT, "too many virtual tables");
  for (uint32_t i = 0; i < nv; ++i) {
    uint32_t k = r.u32();
    if (k > V_XOR8OUT) throw Error(APG_ERR_BAD_CIRCUIT, "unknown virtual kind");
    c.virtuals.push_back(k);
  }
  const uint32_t no = r.u32();
  for (uint32_t i = 0; i < no; ++i) c.outputs.push_back(r.u32());
  const uint32_t depth = r.u32();
  if (depth == 0 || depth > 4096) throw Error(APG_ERR_BAD_CIRCUIT, "bad depth");
  uint32_t prev_vars = c.trace_vars, prev_width = c.n_committed;
  for (uint32_t k = 0; k < depth; ++k) {
    CLayer L;
    L.halving = r.u32() != 0;
    L.num_vars = r.u32();
    L.width = r.u32();
    const uint32_t nc = r.u32(), np = r.u32(), ne = r.u32();
    if (nc + np + ne > 60000) throw Error(APG_ERR_BAD_CIRCUIT, "gate list too long");
    if (L.halving ? (prev_vars == 0 || L.num_vars != prev_vars - 1) : L.num_vars != prev_vars)
      throw Error(APG_ERR_BAD_CIRCUIT, "layer variable count breaks the layering");
    if (np != L.width) throw Error(APG_ERR_BAD_CIRCUIT, "width is not the producing gate count");
    if (L.halving && (nc || ne)) throw Error(APG_ERR_BAD_CIRCUIT, "a halving list holds producing gates only");
    for (uint32_t g = 0; g < nc + np + ne; ++g) {
      CGate G;
      G.kind = r.u32();
      G.p1 = r.u32();
      G.p2 = r.u32();
      if (G.kind > G_QUADRATIC || G.p1 > 4096 || G.p2 > 4096) throw Error(APG_ERR_BAD_CIRCUIT, "bad gate header");
      const bool tree = G.kind == G_TREE_PRODUCT || G.kind == G_TREE_CROSS;
      if (tree != L.halving) throw Error(APG_ERR_BAD_CIRCUIT, "tree gates belong to halving lists only");
      const uint32_t nop = r.u32();
      if (nop != expected_operands(G)) throw Error(APG_ERR_BAD_CIRCUIT, "operand count does not fit the gate");
      for (uint32_t i = 0; i < nop; ++i) {
        uint32_t src = r.u32(), idx = r.u32();
        bool ok = (src == 0 && idx < prev_width) || (src == 1 && !L.halving && idx < nv) ||
                  (src == 2 && !L.halving && idx < std::min<uint32_t>(g, nc));
        if (!ok) throw Error(APG_ERR_BAD_CIRCUIT, "operand out of range");
        G.ops.push_back({src, idx});
      }
      const uint32_t ncf = r.u32();
      if (ncf != expected_coeffs(G)) throw Error(APG_ERR_BAD_CIRCUIT, "coefficient count does not fit the gate");
      for (uint32_t i = 0; i < ncf; ++i) {
        bool ch = r.u32() != 0;
        if (ch) {
          G.coeffs.push_back({true, host::fzero()});
          G.slots.push_back(r.u32());
        } else {
          G.coeffs.push_back({false, r.fr()});
          G.slots.push_back(0);
        }
      }
      (g < nc ? L.cached : g < nc + np ? L.producing : L.enforcing).push_back(G);
    }
    prev_vars = L.num_vars;
    prev_width = L.width;
    c.layers.push_back(L);
  }
  for (auto o : c.outputs)
    if (o >= prev_width) throw Error(APG_ERR_BAD_CIRCUIT, "output outside the top layer");
  if (r.p != r.end) throw Error(APG_ERR_BAD_CIRCUIT, "trailing bytes after the circuit");
  return c;
}

// Layer k's gate list as a device program. Slots: row-wise lists read the
// layer's columns [0, w), the virtual tables [w, w + nv) and the cached
// entries after; halving lists read child 0 of each column in [0, w) and
// child 1 in [w, 2w), every operand expanding to (child 0, child 1).
static HostProgram layer_program(const Circuit& c, size_t k, const Challenges& ch, bool with_enforcing,
                                 const std::vector<F>& weights) {
  const CLayer& L = c.layers[k];
  const uint32_t w = c.width(k);
  const uint32_t nv = L.halving ? 0 : (uint32_t)c.virtuals.size();
  HostProgram hp;
  auto add = [&](const CGate& G) {
    DevGate d;
    memset(&d, 0, sizeof(d));
    d.kind = (uint8_t)G.kind;
    d.p1 = (uint16_t)G.p1;
    d.p2 = (uint16_t)G.p2;
    d.op_off = (uint32_t)hp.ops.size();
    d.cf_off = (uint32_t)hp.coeffs.size();
    for (auto& op : G.ops) {
      if (L.halving) {
        hp.ops.push_back((uint16_t)op.second);
        hp.ops.push_back((uint16_t)(w + op.second));
      } else if (op.first == 0) {
        hp.ops.push_back((uint16_t)op.second);
      } else if (op.first == 1) {
        hp.ops.push_back((uint16_t)(w + op.second));
      } else {
        hp.ops.push_back((uint16_t)(w + nv + op.second));
      }
    }
    d.nops = (uint16_t)(hp.ops.size() - d.op_off);
    for (size_t i = 0; i < G.coeffs.size(); ++i)
      hp.coeffs.push_back(G.coeffs[i].first ? ch.get(G.slots[i]) : G.coeffs[i].second);
    hp.gates.push_back(d);
  };
  for (auto& G : L.cached) add(G);
  for (auto& G : L.producing) add(G);
  if (with_enforcing)
    for (auto& G : L.enforcing) add(G);
  hp.n_cached = (int)L.cached.size();
  hp.n_weighted = (int)(L.producing.size() + (with_enforcing ? L.enforcing.size() : 0));
  hp.weights = weights;
  if (hp.weights.size() < (size_t)hp.n_weighted) hp.weights.resize(hp.n_weighted, host::fone());
  hp.summed = with_enforcing;  // the prover sums the list; the forward pass writes it out gate by gate
  const size_t slots = (L.halving ? 2 * w : w + nv) + L.cached.size();
  if (slots > 60000) throw Error(APG_ERR_BAD_CIRCUIT, "gate list too wide");
  return hp;
}

// ---- forward -------------------------------------------------------------------

namespace {

constexpr int kFwdThreads = 64;

// Row-wise lists over a contiguous Fr layer: the columns are read in place
// (consecutive threads take consecutive rows, so each operand load is one
// coalesced row of a column) and only the virtual and cached entries take
// shared memory.
__global__ void __launch_bounds__(kFwdThreads) k_forward_g(DevProgram P, int w, int nv, VirtualKinds vk,
                                                           const Fr* layer, size_t col_stride, size_t rows, int width,
                                                           Fr* out) {
  extern __shared__ uint32_t sm_raw[];
  const size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (y >= rows) return;
  const GSlots S{layer + y, col_stride, w, thread_slots(sm_raw)};
  for (int v = 0; v < nv; ++v) sm_st(S, w + v, virtual_at_row_dev(vk.k[v], y));
  for (int g = 0; g < P.n_cached; ++g) sm_st(S, P.cached_slot0 + g, eval_gate_dev(P, g, S));
  for (int j = 0; j < width; ++j) st_fe(&out[(size_t)j * rows + y], eval_gate_dev(P, P.n_cached + j, S));
}

// `bits` (null: all Fr) is the stored width of each column of the base.
__global__ void __launch_bounds__(kFwdThreads) k_forward(DevProgram P, int w, int nv, VirtualKinds vk,
                                                         const Fr* const* cols, const uint8_t* bits, size_t rows,
                                                         int halving, int width, Fr* out) {
  extern __shared__ uint32_t sm_raw[];
  const Slots sm = thread_slots(sm_raw);
  size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (y >= rows) return;
  for (int x = 0; x < w; ++x) {
    const int b = bits ? bits[x] : 0;
    sm_st(sm, x, b ? narrow_entry(cols[x], b, y) : ld_fe(&cols[x][y]));
    if (halving) sm_st(sm, w + x, b ? narrow_entry(cols[x], b, y + rows) : ld_fe(&cols[x][y + rows]));
  }
  for (int v = 0; v < nv; ++v) sm_st(sm, w + v, virtual_at_row_dev(vk.k[v], y));
  for (int g = 0; g < P.n_cached; ++g) sm_st(sm, P.cached_slot0 + g, eval_gate_dev(P, g, sm));
  for (int j = 0; j < width; ++j) st_fe(&out[(size_t)j * rows + y], eval_gate_dev(P, P.n_cached + j, sm));
}

}  // namespace

// Layer k >= 1: width(k) Fr columns of 2^vars(k), contiguous. Layer 0, the
// committed base, keeps every column in its stored width (base_bits, 0 = Fr)
// at base_off bytes: the forward pass and gate list 0's first sumcheck rounds
// read narrow columns through the lift. What needs the base as Fr tables
// (reading it back, a halving list over it) lifts it once, on demand.
// The layers come from the stream-ordered pool on the context's stream
// (cudaMallocAsync / cudaFreeAsync): unlike cudaMalloc and cudaFree, they do
// not synchronise the device, so contexts proving shards side by side do not
// stall each other at every forward pass.
struct GkrValues {
  Ctx* ctx = nullptr;
  Circuit circuit;
  std::vector<Fr*> layers;
  std::vector<size_t> base_off;
  std::vector<uint8_t> base_bits;
  bool base_narrow = false;
  Fr* lifted = nullptr;
  ~GkrValues() {
    cudaStream_t st = ctx ? ctx->stream : nullptr;
    for (auto p : layers)
      if (p) cudaFreeAsync(p, st);
    if (lifted) cudaFreeAsync(lifted, st);
  }
  const void* base_raw(size_t x) const { return reinterpret_cast<const uint8_t*>(layers[0]) + base_off[x]; }
  const Fr* col(size_t k, size_t x) {
    const size_t rows = (size_t)1 << circuit.vars(k);
    if (k > 0) return layers[k] + x * rows;
    if (!base_narrow) return reinterpret_cast<const Fr*>(base_raw(x));
    if (!lifted) {
      APG_CUDA(cudaMallocAsync((void**)&lifted, 32 * rows * circuit.n_committed, ctx->stream));
      for (size_t j = 0; j < circuit.n_committed; ++j)
        lift_column(*ctx, base_raw(j), base_bits[j], rows, lifted + j * rows);
    }
    return lifted + x * rows;
  }
};

Challenges read_challenges(const uint32_t* slots, const uint8_t* values, size_t n) {
  Challenges ch;
  for (size_t i = 0; i < n; ++i) {
    F v;
    memcpy(v.w, values + 32 * i, 32);
    if (!host::below_p(v.w)) throw Error(APG_ERR_NONCANONICAL, "non-canonical challenge value");
    ch.kv.push_back({slots[i], v});
  }
  return ch;
}

GkrValues* gkr_forward_impl(Ctx& c, const uint8_t* blob, size_t blob_len, const void* const* base,
                            const uint8_t* bits, bool base_on_device, const uint32_t* slots,
                            const uint8_t* slot_values, size_t n_slots) {
  std::unique_ptr<GkrValues> V(new GkrValues());
  V->ctx = &c;
  V->circuit = parse_circuit_blob(blob, blob_len);
  const Circuit& C = V->circuit;
  if (!base || (n_slots && (!slots || !slot_values))) throw Error(APG_ERR_INVALID_ARGUMENT, "null input");
  Challenges ch = read_challenges(slots, slot_values, n_slots);
  const size_t n0 = (size_t)1 << C.trace_vars;
  V->layers.assign(C.layers.size() + 1, nullptr);
  // The base in its stored widths, each column 256-byte aligned.
  V->base_bits.assign(C.n_committed, 0);
  V->base_off.assign(C.n_committed, 0);
  size_t total = 0;
  for (size_t x = 0; x < C.n_committed; ++x) {
    if (bits) {
      if (!narrow_bits_ok(bits[x])) throw Error(APG_ERR_INVALID_ARGUMENT, "a column width other than 0, 1, 8, 16, 32");
      V->base_bits[x] = bits[x];
      V->base_narrow |= bits[x] != 0;
    }
    if (!base[x]) throw Error(APG_ERR_INVALID_ARGUMENT, "null column");
    V->base_off[x] = total;
    total += (narrow_bytes(V->base_bits[x], n0) + 255) / 256 * 256;
  }
  APG_CUDA(cudaMallocAsync((void**)&V->layers[0], std::max<size_t>(total, 256), c.stream));
  for (size_t x = 0; x < C.n_committed; ++x)
    APG_CUDA(cudaMemcpyAsync(reinterpret_cast<uint8_t*>(V->layers[0]) + V->base_off[x], base[x],
                             narrow_bytes(V->base_bits[x], n0),
                             base_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c.stream));
  const uint8_t* d_bits = nullptr;
  if (V->base_narrow) {
    uint8_t* db = c.scratch[S_ENTRIES].as<uint8_t>(C.n_committed);
    APG_CUDA(cudaMemcpyAsync(db, V->base_bits.data(), C.n_committed, cudaMemcpyHostToDevice, c.stream));
    d_bits = db;
  }
  for (size_t k = 0; k < C.layers.size(); ++k) {
    const CLayer& L = C.layers[k];
    const size_t rows = (size_t)1 << L.num_vars;
    APG_CUDA(cudaMallocAsync((void**)&V->layers[k + 1], 32 * rows * std::max<uint32_t>(L.width, 1), c.stream));
    HostProgram hp = layer_program(C, k, ch, false, {});
    DevProgram P;
    upload_program(c, hp, P, 0);
    const int w = (int)C.width(k);
    const int nv = L.halving ? 0 : (int)C.virtuals.size();
    P.cached_slot0 = L.halving ? 2 * w : w + nv;
    VirtualKinds vk;
    memset(&vk, 0, sizeof(vk));
    for (int v = 0; v < nv; ++v) vk.k[v] = (uint8_t)C.virtuals[v];
    std::vector<const Fr*> cols(w);
    for (int x = 0; x < w; ++x)
      cols[x] = k == 0 ? reinterpret_cast<const Fr*>(V->base_raw(x)) : V->col(k, x);
    const Fr** d_cols = c.scratch[S_TMP5].as<const Fr*>(w);
    APG_CUDA(cudaMemcpyAsync(d_cols, cols.data(), sizeof(Fr*) * w, cudaMemcpyHostToDevice, c.stream));
    // A row-wise list over an Fr layer reads the layer in place; a halving
    // list (two rows of a column a slot pair) or a narrow base is staged.
    const bool in_place = !L.halving && (k > 0 || !V->base_narrow) && w > 0;
    const size_t slots_n = (size_t)P.cached_slot0 + L.cached.size() - (in_place ? (size_t)w : 0);
    int threads = kFwdThreads;
    while (threads > 8 && std::max<size_t>(slots_n, 1) * 32 * threads > 200 * 1024) threads /= 2;
    const size_t smem = std::max<size_t>(slots_n, 1) * 32 * threads;
    if (smem > 200 * 1024) throw Error(APG_ERR_BAD_CIRCUIT, "gate list too wide for one thread block");
    cudaEvent_t t0 = c.timer_begin();
    if (L.width && in_place) {
      APG_CUDA(cudaFuncSetAttribute(k_forward_g, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
      // Columns of the layer lie a fixed stride apart (the base's at its
      // 256-byte-aligned offsets, later layers back to back).
      const size_t stride = w > 1 ? (size_t)(cols[1] - cols[0]) : 0;
      launch(c, k_forward_g, (unsigned)((rows + threads - 1) / threads), threads, smem, P, w, nv, vk, cols[0],
             stride, rows, (int)L.width, V->layers[k + 1]);
    } else if (L.width) {
      APG_CUDA(cudaFuncSetAttribute(k_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
      launch(c, k_forward, (unsigned)((rows + threads - 1) / threads), threads, smem, P, w, nv, vk,
             (const Fr* const*)d_cols, k == 0 ? d_bits : (const uint8_t*)nullptr, rows, L.halving ? 1 : 0,
             (int)L.width, V->layers[k + 1]);
    }
    c.timer_end(APG_TIMER_GKR_FORWARD, t0);
    // The program and column list buffers are reused by the next layer.
    APG_CUDA(cudaStreamSynchronize(c.stream));
  }
  c.check_flags();
  return V.release();
}

// Proof layout (Fr in memory): for k = 0 .. depth-1, gate list k's rounds
// (vars(k+1) x 4) then its claims (width(k), or 2 width(k) for a halving list,
// interleaved child 0, child 1 per column).
size_t gkr_proof_elems(const Circuit& C) {
  size_t n = 0;
  for (size_t k = 0; k < C.layers.size(); ++k)
    n += 4 * (size_t)C.vars(k + 1) + (C.layers[k].halving ? 2 : 1) * (size_t)C.width(k);
  return n;
}

int gkr_prove_impl(Ctx& c, const uint8_t* blob, size_t blob_len, GkrValues* V, const uint32_t* slots,
                   const uint8_t* slot_values, size_t n_slots, uint8_t* transcript, uint8_t* proof_out,
                   size_t proof_cap, size_t* proof_len, uint8_t* point_out) {
  if (!V || !transcript || !proof_len) return APG_ERR_INVALID_ARGUMENT;
  Circuit C = parse_circuit_blob(blob, blob_len);
  const Circuit& VC = V->circuit;
  if (C.layers.size() != VC.layers.size() || C.trace_vars != VC.trace_vars || C.n_committed != VC.n_committed) {
    c.last_error = "the values were produced by a different circuit";
    return APG_ERR_INVALID_ARGUMENT;
  }
  const size_t need = 32 * gkr_proof_elems(C);
  *proof_len = need;
  if (!proof_out || proof_cap < need) {
    c.last_error = "proof buffer too small";
    return APG_ERR_INVALID_ARGUMENT;
  }
  Challenges ch = read_challenges(slots, slot_values, n_slots);
  host::Transcript tr;
  if (!tr.load(transcript)) {
    c.last_error = "malformed transcript snapshot";
    return APG_ERR_INVALID_ARGUMENT;
  }
  const size_t depth = C.layers.size();
  // O1: every output column's values, one message.
  {
    const size_t rows = (size_t)1 << C.vars(depth);
    std::vector<F> msg(rows * C.outputs.size());
    for (size_t i = 0; i < C.outputs.size(); ++i)
      APG_CUDA(cudaMemcpyAsync(msg.data() + i * rows, V->col(depth, C.outputs[i]), 32 * rows,
                               cudaMemcpyDeviceToHost, c.stream));
    APG_CUDA(cudaStreamSynchronize(c.stream));
    tr.absorb(host::T_GKR_OUTPUTS, msg);
  }
  // O2.
  std::vector<F> point;
  for (uint32_t i = 0; i < C.vars(depth); ++i) point.push_back(tr.challenge(host::T_GKR_OUTPUT_POINT));

  std::vector<std::vector<F>> per_layer(depth);
  for (size_t kk = depth; kk-- > 0;) {
    const CLayer& L = C.layers[kk];
    // L1.
    F lambda = tr.challenge(host::T_GKR_BATCH);
    std::vector<F> weights;
    F acc = host::fone();
    for (size_t j = 0; j < L.producing.size() + L.enforcing.size(); ++j) {
      weights.push_back(acc);
      acc = host::fmul(acc, lambda);
    }
    HostProgram hp = layer_program(C, kk, ch, true, weights);
    DevProgram P;
    upload_program(c, hp, P, 0);
    // L2: the tables, child 0 then child 1 of every column for a halving list.
    const uint32_t w = C.width(kk);
    std::vector<const Fr*> src;
    std::vector<uint8_t> vkinds, src_bits;
    if (L.halving) {
      const size_t half = (size_t)1 << (C.vars(kk) - 1);
      for (uint32_t x = 0; x < w; ++x) src.push_back(V->col(kk, x));
      for (uint32_t x = 0; x < w; ++x) src.push_back(V->col(kk, x) + half);
    } else if (kk == 0 && V->base_narrow) {
      // The base in its stored widths: the first bind lifts it.
      for (uint32_t x = 0; x < w; ++x) src.push_back(reinterpret_cast<const Fr*>(V->base_raw(x)));
      src_bits = V->base_bits;
      for (auto k : C.virtuals) vkinds.push_back((uint8_t)k);
    } else {
      for (uint32_t x = 0; x < w; ++x) src.push_back(V->col(kk, x));
      for (auto k : C.virtuals) vkinds.push_back((uint8_t)k);
    }
    std::vector<std::array<F, 4>> rounds;
    std::vector<F> rho, finals;
    HostPairTerms pairs;
    const bool by_pairs = pair_terms_of(hp, (int)src.size(), pairs);
    run_sumcheck(c, P, (int)src.size(), vkinds, (int)L.cached.size(), src, point, tr, rounds, rho, finals,
                 src_bits, by_pairs ? &pairs : nullptr);
    // L3.
    std::vector<F> claims;
    if (L.halving) {
      for (uint32_t x = 0; x < w; ++x) {
        claims.push_back(finals[x]);
        claims.push_back(finals[w + x]);
      }
    } else {
      claims = finals;
    }
    tr.absorb(host::T_GKR_LAYER_CLAIMS, claims);
    // L4.
    point = rho;
    if (L.halving) point.push_back(tr.challenge(host::T_GKR_CHILD));
    std::vector<F>& out = per_layer[kk];
    for (auto& g : rounds) out.insert(out.end(), g.begin(), g.end());
    out.insert(out.end(), claims.begin(), claims.end());
  }
  size_t off = 0;
  for (auto& v : per_layer) {
    memcpy(proof_out + off, v.data(), 32 * v.size());
    off += 32 * v.size();
  }
  // The base layer's point: what the committed columns are opened at.
  if (point_out) memcpy(point_out, point.data(), 32 * point.size());
  tr.save(transcript);
  c.check_flags();
  return APG_OK;
}

// gkr::prove_sumcheck (crates/gkr/src/lib.rs:792-899) on its own: gate list
// `layer`'s summand with the caller's weights over the caller's device tables
// (the list's columns, and for a halving list their upper children), every
// round absorbed and challenged on the caller's transcript. The same program,
// tables and round kernels as gkr_prove_impl's step L2 for that list.
int gkr_prove_sumcheck_impl(Ctx& c, const uint8_t* blob, size_t blob_len, size_t layer, const uint8_t* weights,
                            size_t n_weights, const uint32_t* slots, const uint8_t* slot_values, size_t n_slots,
                            const uint8_t* eq_point, size_t n, const void* const* d_lower,
                            const void* const* d_upper, size_t width, uint8_t* transcript, uint8_t* rounds_out,
                            uint8_t* point_out, uint8_t* finals_out) {
  if (!transcript || !rounds_out || !point_out || !finals_out || (n && !eq_point) || (n_weights && !weights) ||
      (n_slots && (!slots || !slot_values)))
    return APG_ERR_INVALID_ARGUMENT;
  const Circuit C = parse_circuit_blob(blob, blob_len);
  if (layer >= C.layers.size()) {
    c.last_error = "no such gate list";
    return APG_ERR_INVALID_ARGUMENT;
  }
  const CLayer& L = C.layers[layer];
  if (width != C.width(layer) || n != C.vars(layer + 1)) {
    c.last_error = "the tables do not match the gate list (width, or the eq point's variables)";
    return APG_ERR_INVALID_ARGUMENT;
  }
  if (n_weights != L.producing.size() + L.enforcing.size()) {
    c.last_error = "one weight per producing and enforcing gate";
    return APG_ERR_INVALID_ARGUMENT;
  }
  if (width && (!d_lower || (L.halving && !d_upper))) return APG_ERR_INVALID_ARGUMENT;
  for (size_t x = 0; x < width; ++x)
    if (!d_lower[x] || (L.halving && !d_upper[x])) {
      c.last_error = "a table pointer is null";
      return APG_ERR_INVALID_ARGUMENT;
    }
  const Challenges ch = read_challenges(slots, slot_values, n_slots);
  auto read_frs = [](const uint8_t* p, size_t k, std::vector<F>& out) {
    out.resize(k);
    for (size_t i = 0; i < k; ++i) {
      memcpy(out[i].w, p + 32 * i, 32);
      if (!host::below_p(out[i].w)) throw Error(APG_ERR_NONCANONICAL, "a field element is not below the modulus");
    }
  };
  std::vector<F> w, point;
  read_frs(weights, n_weights, w);
  read_frs(eq_point, n, point);
  host::Transcript tr;
  if (!tr.load(transcript)) {
    c.last_error = "malformed transcript snapshot";
    return APG_ERR_INVALID_ARGUMENT;
  }
  HostProgram hp = layer_program(C, layer, ch, true, w);
  DevProgram P;
  upload_program(c, hp, P, 0);
  std::vector<const Fr*> src;
  std::vector<uint8_t> vkinds;
  for (size_t x = 0; x < width; ++x) src.push_back(static_cast<const Fr*>(d_lower[x]));
  if (L.halving)
    for (size_t x = 0; x < width; ++x) src.push_back(static_cast<const Fr*>(d_upper[x]));
  else
    for (auto k : C.virtuals) vkinds.push_back((uint8_t)k);
  std::vector<std::array<F, 4>> rounds;
  std::vector<F> rho, finals;
  HostPairTerms pairs;
  const bool by_pairs = pair_terms_of(hp, (int)src.size(), pairs);
  run_sumcheck(c, P, (int)src.size(), vkinds, (int)L.cached.size(), src, point, tr, rounds, rho, finals, {},
               by_pairs ? &pairs : nullptr);
  for (size_t r = 0; r < rounds.size(); ++r) memcpy(rounds_out + 128 * r, rounds[r].data(), 128);
  memcpy(point_out, rho.data(), 32 * rho.size());
  memcpy(finals_out, finals.data(), 32 * finals.size());
  tr.save(transcript);
  c.check_flags();
  return APG_OK;
}

void gkr_values_free(GkrValues* v) { delete v; }

size_t gkr_proof_len_impl(const uint8_t* blob, size_t len) { return 32 * gkr_proof_elems(parse_circuit_blob(blob, len)); }

// Device bytes a forward pass and proof of this circuit hold at once: the
// base as Fr, every layer, and the largest layer sumcheck's two level
// buffers (its tables, eq and the virtual tables at half and a quarter of
// the bound variables' rows).
size_t gkr_device_bytes_impl(const uint8_t* blob, size_t len) {
  const Circuit C = parse_circuit_blob(blob, len);
  size_t b = 32 * ((size_t)1 << C.trace_vars) * C.n_committed;
  size_t worst = 0;
  for (size_t k = 0; k < C.layers.size(); ++k) {
    const CLayer& L = C.layers[k];
    b += 32 * ((size_t)1 << L.num_vars) * std::max<uint32_t>(L.width, 1);
    const size_t tables = (L.halving ? 2 : 1) * (size_t)C.width(k) + (L.halving ? 0 : C.virtuals.size()) + 1;
    worst = std::max(worst, tables * 24 * ((size_t)1 << L.num_vars));
  }
  return b + worst;
}

int gkr_values_read_impl(GkrValues* v, size_t layer, size_t col, uint8_t* out) {
  if (!v || !out || layer > v->circuit.layers.size() || col >= v->circuit.width(layer)) return APG_ERR_INVALID_ARGUMENT;
  Ctx& c = *v->ctx;
  const size_t rows = (size_t)1 << v->circuit.vars(layer);
  APG_CUDA(cudaMemcpyAsync(out, v->col(layer, col), 32 * rows, cudaMemcpyDeviceToHost, c.stream));
  APG_CUDA(cudaStreamSynchronize(c.stream));
  return APG_OK;
}

size_t gkr_values_len(GkrValues* v, size_t layer) {
  if (!v || layer > v->circuit.layers.size()) return 0;
  return (size_t)1 << v->circuit.vars(layer);
}

}  // namespace apg
