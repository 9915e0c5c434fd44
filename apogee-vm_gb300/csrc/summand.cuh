// The gate kernel on the device: a resolved gate list evaluated from
// per-thread value slots in shared memory.
//
// Restates crates/gkr-verify/src/lib.rs: eval_gate (:142-202) over the seven
// GateDef shapes, ResolvedList's evaluation order (cached entries first, then
// producing, then enforcing gates, :315-480) and the virtual tables' closed
// forms (virtual_at_row / virtual_at_point, :205-286). A zerocheck Gate
// (crates/sumcheck/src/lib.rs:109-169) is the one-gate list
// `Quadratic { 0, linear terms, product terms }` with weight 1.
//
// Slots hold one Fr each in shared memory (Slots below): either a thread's
// own, word-major across the block's threads so that a warp's 32-bit accesses
// fall in distinct banks (word w of slot s of thread t at
// smem[(s * 8 + w) * blockDim.x + t]), or one set a whole warp shares and
// reads at once (wide gate lists, one pair per warp).
#pragma once
#include "field.cuh"

namespace apg {

enum GateKind : uint8_t { G_LINEAR = 0, G_PRODUCT = 1, G_MASK = 2, G_AFFINE = 3, G_TREE_PRODUCT = 4,
                          G_TREE_CROSS = 5, G_QUADRATIC = 6 };

enum VirtualKindDev : uint8_t { V_ROW = 0, V_RAM_LIVE = 1, V_RANGE19 = 2, V_RANGE16 = 3, V_XOR8A = 4, V_XOR8B = 5,
                                V_XOR8OUT = 6 };

struct VirtualKinds {
  uint8_t k[8];
};

// DevGate::flags bit: the gate's weight is 1, so its value is summed as it is.
constexpr uint8_t kGateUnitWeight = 1;

struct DevGate {
  uint8_t kind;
  uint8_t flags;
  uint16_t nops;
  uint16_t p1, p2;   // shape: Linear t; Affine t, u; Quadratic t, u
  uint32_t op_off;   // first operand slot index in ops[]
  uint32_t cf_off;   // first coefficient in coeffs[]
  uint32_t ones;     // bit i: coefficient cf_off + i is 1 (its product is skipped)
  uint32_t negs;     // bit i: coefficient cf_off + i is -1 (a negation instead)
  uint32_t zeros;    // bit i: coefficient cf_off + i is 0 (its term is dropped)
};

// A resolved list on the device. Gates [0, n_cached) fill the cached slots in
// order; gates [n_cached, n_cached + n_weighted) are summed with weights.
struct DevProgram {
  const DevGate* gates;
  const uint16_t* ops;  // slot indices
  const Fr* coeffs;     // Montgomery, challenges already substituted
  const Fr* weights;    // one per weighted gate (lambda^j), Montgomery
  int n_cached;
  int n_weighted;
  int cached_slot0;     // slot of cached entry 0
};

// One evaluation's slots: word w of slot s at base[(s * 8 + w) * stride].
// A thread's own slots (thread_slots) interleave with the block's other
// threads (stride blockDim.x); a warp's shared slots (stride 1) are read by
// all its lanes at once.
struct Slots {
  uint32_t* base;
  int slot_stride;  // words between consecutive slots
  int word_stride;  // words between a slot's consecutive words
};

__device__ __forceinline__ Slots thread_slots(uint32_t* sm) {
  return Slots{sm + threadIdx.x, 8 * (int)blockDim.x, (int)blockDim.x};
}

// A warp's shared set of n slots, word-major (word w of slot s at w * n + s),
// so lanes reading different slots hit different banks.
__device__ __forceinline__ Slots warp_slots(uint32_t* base, int n) { return Slots{base, 1, n}; }

__device__ __forceinline__ Fr sm_ld(const Slots& S, int slot) {
  Fr r;
#pragma unroll
  for (int w = 0; w < 8; ++w) r.v[w] = S.base[slot * S.slot_stride + w * S.word_stride];
  return r;
}

__device__ __forceinline__ void sm_st(const Slots& S, int slot, const Fr& a) {
#pragma unroll
  for (int w = 0; w < 8; ++w) S.base[slot * S.slot_stride + w * S.word_stride] = a.v[w];
}

// Operand slots split in two: slots below `ncols` are the columns of a
// contiguous Fr layer read in place (column x of this row at cols + x *
// stride), the rest per-thread shared memory. The forward pass of a row-wise
// list reads its operands this way, so a block needs no per-thread copy of
// the row and keeps a full complement of threads.
struct GSlots {
  const Fr* cols;
  size_t stride;
  int ncols;
  Slots rest;
};

__device__ __forceinline__ Fr sm_ld(const GSlots& S, int slot) {
  return slot < S.ncols ? ld_fe(S.cols + (size_t)slot * S.stride) : sm_ld(S.rest, slot - S.ncols);
}

// Only the shared-memory slots (virtual tables, cached entries) are written.
__device__ __forceinline__ void sm_st(const GSlots& S, int slot, const Fr& a) { sm_st(S.rest, slot - S.ncols, a); }

__device__ __forceinline__ Fr ld_g(const Fr* p) { return ld_fe(p); }

// The interpreter calls one out-of-line Fr product: its gate kinds would
// otherwise inline a dozen multiplies and overflow the instruction cache of
// the round loop (no_instruction was the top stall of the round kernel).
static __device__ __noinline__ Fr rmul(const Fr a, const Fr b) { return fe_mul(a, b); }

// Two independent products in one out-of-line call: half the calls of a
// small round's thread (its folds and node products come in pairs).
struct FrPair {
  Fr a, b;
};
static __device__ __noinline__ FrPair rmul2(const Fr a, const Fr b, const Fr c, const Fr d) {
  FrPair r;
  r.a = fe_mul(a, b);
  r.b = fe_mul(c, d);
  return r;
}

// c[i] * x, skipping the product when bit i of `ones` marks c[i] = 1.
__device__ __forceinline__ Fr cmul_coef(const Fr* c, int i, uint32_t ones, const Fr& x) {
  return (i < 32 && ((ones >> i) & 1u)) ? x : rmul(ld_g(&c[i]), x);
}

// The same for a gate's own coefficient i, also folding -1 (a negation) and 0.
__device__ __forceinline__ Fr gmul_coef(const DevGate& G, const Fr* c, int i, const Fr& x) {
  if (i < 32) {
    const uint32_t bit = 1u << i;
    if (G.ones & bit) return x;
    if (G.zeros & bit) return fe_zero<FrConsts>();
    if (G.negs & bit) return fe_neg(x);
  }
  return rmul(ld_g(&c[i]), x);
}

// Affine form sum_{i<t} c[i] * x_i + c[t], operands ops[0..t); `ones` is
// the one-mask of c[0..].
template <class S>
__device__ __forceinline__ Fr affine_form(const S& sm, const DevGate& G, const uint16_t* ops, const Fr* c, int c0,
                                          int t) {
  Fr acc = ld_g(&c[c0 + t]);
  for (int i = 0; i < t; ++i) acc = fe_add(acc, gmul_coef(G, c, c0 + i, sm_ld(sm, ops[i])));
  return acc;
}

template <class S>
static __device__ __noinline__ Fr eval_gate_dev(const DevProgram& P, int g, const S sm) {
  const DevGate G = P.gates[g];
  const uint16_t* ops = P.ops + G.op_off;
  const Fr* c = P.coeffs + G.cf_off;
  switch (G.kind) {
    case G_LINEAR:
      return affine_form(sm, G, ops, c, 0, G.p1);
    case G_PRODUCT:
      return rmul(gmul_coef(G, c, 0, sm_ld(sm, ops[0])), sm_ld(sm, ops[1]));
    case G_MASK: {
      Fr x = sm_ld(sm, ops[0]), m = sm_ld(sm, ops[1]);
      return fe_sub(fe_add(rmul(x, m), fe_one<FrConsts>()), m);
    }
    case G_AFFINE: {
      const int t = G.p1, u = G.p2;
      Fr l = affine_form(sm, G, ops, c, 0, t);
      Fr r = affine_form(sm, G, ops + t, c, t + 1, u);
      return rmul(l, r);
    }
    case G_TREE_PRODUCT:
      return rmul(sm_ld(sm, ops[0]), sm_ld(sm, ops[1]));
    case G_TREE_CROSS:
      return fe_add(rmul(sm_ld(sm, ops[0]), sm_ld(sm, ops[3])), rmul(sm_ld(sm, ops[1]), sm_ld(sm, ops[2])));
    case G_QUADRATIC: {
      const int t = G.p1, u = G.p2;
      Fr acc = ld_g(&c[0]);
      for (int i = 0; i < t; ++i) acc = fe_add(acc, gmul_coef(G, c, 1 + i, sm_ld(sm, ops[i])));
      for (int j = 0; j < u; ++j) {
        const int ci = 1 + t + j;
        if (ci < 32 && ((G.zeros >> ci) & 1u)) continue;
        Fr yz = rmul(sm_ld(sm, ops[t + 2 * j]), sm_ld(sm, ops[t + 2 * j + 1]));
        acc = fe_add(acc, gmul_coef(G, c, ci, yz));
      }
      return acc;
    }
  }
  return fe_zero<FrConsts>();
}

// Weighted gate j's contribution: its value times its weight, unless the
// weight is 1.
__device__ __forceinline__ Fr weigh(const DevProgram& P, int j, const Fr& v) {
  return (P.gates[P.n_cached + j].flags & kGateUnitWeight) ? v : rmul(ld_g(&P.weights[j]), v);
}

// Cached entries into their slots, then the weighted sum of the gates.
__device__ __forceinline__ Fr eval_summand(const DevProgram& P, const Slots& sm) {
  for (int g = 0; g < P.n_cached; ++g) sm_st(sm, P.cached_slot0 + g, eval_gate_dev(P, g, sm));
  Fr acc = fe_zero<FrConsts>();
  for (int j = 0; j < P.n_weighted; ++j) {
    Fr v = eval_gate_dev(P, P.n_cached + j, sm);
    acc = fe_add(acc, weigh(P, j, v));
  }
  return acc;
}

// ---- virtual tables ----------------------------------------------------------

__device__ __forceinline__ Fr fr_u64(uint64_t x) { return fe_from_u64<FrConsts>(x); }

// Row y's value of a virtual table (virtual_at_row).
__device__ __forceinline__ Fr virtual_at_row_dev(int kind, uint64_t y) {
  switch (kind) {
    case V_ROW: return fr_u64(y);
    case V_RAM_LIVE: return y >= (1ull << 14) ? fe_one<FrConsts>() : fe_zero<FrConsts>();
    case V_RANGE19: return fr_u64(y & ((1ull << 19) - 1));
    case V_RANGE16: return fr_u64(y & ((1ull << 16) - 1));
    case V_XOR8A: return fr_u64(y & 0xff);
    case V_XOR8B: return fr_u64((y >> 8) & 0xff);
    case V_XOR8OUT: return fr_u64((y & 0xff) ^ ((y >> 8) & 0xff));
  }
  return fe_zero<FrConsts>();
}

// Per-round constants of the closed forms, prepared on the host from the
// challenges bound so far (r_0 .. r_{b-1}).
struct VirtualRound {
  int bound;          // b
  int nvars;          // n: variables of the sumcheck
  Fr row_prefix;      // sum_{j<b} 2^j r_j
  Fr range19_prefix;  // sum_{j<min(b,19)} 2^j r_j
  Fr range16_prefix;  // sum_{j<min(b,16)} 2^j r_j
  Fr ram_q;           // prod_{14<=j<b} (1 - r_j)
  Fr r16[16];         // r_j for j < min(b, 16)
  Fr pow2_b;          // 2^b
};

// y_j of the point (r_0..r_{b-1}, X, bits of i) for j < 16, at X in {0, 1}.
__device__ __forceinline__ Fr point_coord(const VirtualRound& V, uint64_t i, int j, int X) {
  if (j >= V.nvars) return fe_zero<FrConsts>();
  if (j < V.bound) return V.r16[j];
  if (j == V.bound) return X ? fe_one<FrConsts>() : fe_zero<FrConsts>();
  return ((i >> (j - V.bound - 1)) & 1) ? fe_one<FrConsts>() : fe_zero<FrConsts>();
}

__device__ __forceinline__ Fr xor8_at(const VirtualRound& V, int kind, uint64_t i, int X) {
  Fr acc = fe_zero<FrConsts>();
  for (int j = 7; j >= 0; --j) {
    acc = fe_dbl(acc);
    Fr y = point_coord(V, i, j, X), z = point_coord(V, i, j + 8, X);
    if (kind == V_XOR8A) acc = fe_add(acc, y);
    else if (kind == V_XOR8B) acc = fe_add(acc, z);
    else {
      Fr yz = fe_mul(y, z);
      acc = fe_sub(fe_add(acc, fe_add(y, z)), fe_dbl(yz));
    }
  }
  return acc;
}

// The line lo + X * step of a virtual table over pair i after b bound rounds.
__device__ __forceinline__ void virtual_line_dev(const VirtualRound& V, int kind, uint64_t i, Fr& lo, Fr& step) {
  const int b = V.bound;
  switch (kind) {
    case V_ROW:
      lo = fe_add(V.row_prefix, fr_u64(i << (b + 1)));
      step = V.pow2_b;
      return;
    case V_RANGE19:
    case V_RANGE16: {
      const int bits = kind == V_RANGE19 ? 19 : 16;
      const Fr pre = kind == V_RANGE19 ? V.range19_prefix : V.range16_prefix;
      if (b < bits) {
        uint64_t low = (bits - b - 1) >= 63 ? i : (i & ((1ull << (bits - b - 1)) - 1));
        lo = fe_add(pre, fr_u64(low << (b + 1)));
        step = V.pow2_b;
      } else {
        lo = pre;
        step = fe_zero<FrConsts>();
      }
      return;
    }
    case V_RAM_LIVE: {
      const int sh = b >= 13 ? 0 : 13 - b;
      const bool high_bit = (i >> sh) != 0;
      if (high_bit) {
        lo = fe_one<FrConsts>();
        step = fe_zero<FrConsts>();
      } else if (b >= 14) {
        lo = fe_sub(fe_one<FrConsts>(), V.ram_q);
        step = V.ram_q;
      } else {
        lo = fe_zero<FrConsts>();
        step = fe_zero<FrConsts>();
      }
      return;
    }
    default: {
      lo = xor8_at(V, kind, i, 0);
      step = fe_sub(xor8_at(V, kind, i, 1), lo);
      return;
    }
  }
}

}  // namespace apg
