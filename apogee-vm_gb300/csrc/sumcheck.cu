// The sumcheck prover on the device: one fused kernel per round folds every
// table with the previous round's challenge and sums the summand over the
// hypercube at the nodes the round needs; the host rebuilds the round's cubic
// and draws the next challenge.
//
// Restates crates/sumcheck/src/lib.rs (prove_zerocheck :359-408,
// round_evaluations :324-349) and crates/gkr/src/lib.rs (prove_sumcheck
// :792-899): per pair (2i, 2i+1) of every table the line lo + X*(hi - lo),
// the summand at X = 0..3 weighted by eq, SUMCHECK_ROUND then
// SUMCHECK_CHALLENGE, and the bind f'(i) = f(2i) + r*(f(2i+1) - f(2i))
// (crates/poly/src/lib.rs:156-185). The cubic factors as eq_r(X) q(X) with q
// quadratic, so the device sums q at X = 0 and 2 (and 1 in the first round)
// and the host derives the rest (run_sumcheck). Round r's kernel reads the
// level-(r-1) tables once, writes the level-r tables once and never re-reads
// them.
#include <algorithm>
#include <chrono>
#include <map>
#include <tuple>

#include "sumcheck.cuh"

namespace apg {

namespace {

constexpr int kRoundThreads = 128;
constexpr int kWarpModeGates = 16;  // weighted gates from which a list goes one pair per warp

struct RoundArgs {
  int nd;                    // data tables (eq is separate)
  int nv;                    // virtual tables
  uint8_t vkinds[8];
  const Fr* const* src;      // round-0 tables (nd data, then eq), device pointers
  const Fr* in_base;         // previous level (when !in_is_src): table k at in_base + k * in_len
  size_t in_len;
  int in_is_src;
  int bind;                  // fold the previous level with c first
  Fr c;
  Fr* out_base;              // this level (when bind): table k at out_base + k * (in_len / 2)
  size_t npairs;
  int slots_step0;           // first step slot
  int n_val_slots;           // nd + nv
  unsigned* done;            // blocks finished this round (zero between rounds)
  Fr* out;                   // the round's 4 sums, written by the last block
  int xsplit;                // one thread per (pair, node X) instead of per pair
  const uint8_t* src_bits;   // stored width of each src table (null: all Fr)
  int nodes;                 // bit X set: evaluate the summand at node X (0..2)
};

__device__ __forceinline__ const Fr* table_in(const RoundArgs& A, int k) {
  return A.in_is_src ? A.src[k] : A.in_base + (size_t)k * A.in_len;
}

// Pair i of table k: (lo, hi) = entries (2i, 2i + 1) of this round's level,
// folded from the previous level with c first when the round binds (the
// folded pair is stored when `store` is set). OUTLINE: the fold's two
// products are one call of the shared out-of-line rmul2 instead of two
// inlined multiplies, for the kernels of small rounds, where a launch runs its
// code once and fetching inlined copies of the multiply costs more than the
// call (APG_SMALL_OUTLINE; 0 inlines them everywhere).
#ifndef APG_SMALL_OUTLINE
#define APG_SMALL_OUTLINE 1
#endif
#ifndef APG_SMALL_WARP
#define APG_SMALL_WARP 1
#endif
template <bool OUTLINE = false>
__device__ __forceinline__ void load_line(const RoundArgs& A, int k, size_t i, Fr& lo, Fr& hi, bool store = true) {
  const Fr* t = table_in(A, k);
  const int bits = A.in_is_src && A.src_bits ? A.src_bits[k] : 0;
  if (!A.bind) {
    lo = bits ? narrow_entry(t, bits, 2 * i) : ld_fe(&t[2 * i]);
    hi = bits ? narrow_entry(t, bits, 2 * i + 1) : ld_fe(&t[2 * i + 1]);
    return;
  }
  Fr a0, a1, a2, a3;
  if (bits) {
    a0 = narrow_entry(t, bits, 4 * i);
    a1 = narrow_entry(t, bits, 4 * i + 1);
    a2 = narrow_entry(t, bits, 4 * i + 2);
    a3 = narrow_entry(t, bits, 4 * i + 3);
  } else {
    a0 = ld_fe(&t[4 * i]);
    a1 = ld_fe(&t[4 * i + 1]);
    a2 = ld_fe(&t[4 * i + 2]);
    a3 = ld_fe(&t[4 * i + 3]);
  }
  if (OUTLINE) {
    const FrPair f = rmul2(A.c, fe_sub(a1, a0), A.c, fe_sub(a3, a2));
    lo = fe_add(a0, f.a);
    hi = fe_add(a2, f.b);
  } else {
    lo = fe_add(a0, fe_mul(A.c, fe_sub(a1, a0)));
    hi = fe_add(a2, fe_mul(A.c, fe_sub(a3, a2)));
  }
  if (!store) return;
  Fr* o = A.out_base + (size_t)k * (A.in_len / 2);
  st_fe(&o[2 * i], lo);
  st_fe(&o[2 * i + 1], hi);
}

// lo + x * (hi - lo) for a node x in 0..2.
__device__ __forceinline__ Fr at_node(const Fr& lo, const Fr& step, int x) {
  Fr v = lo;
  for (int j = 0; j < x; ++j) v = fe_add(v, step);
  return v;
}

// After every block has published its 4 partial sums: the last block to
// finish (it takes the last ticket) adds them all into A.out and re-arms the
// counter for the next round.
__device__ __forceinline__ void round_total(const RoundArgs& A, const Fr* partials, Fr* red) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(A.done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int x = 0; x < 4; ++x) {
    Fr a = fe_zero<FrConsts>();
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
      const uint4* q = reinterpret_cast<const uint4*>(&partials[(size_t)b * 4 + x]);
      const uint4 u0 = __ldcg(q), u1 = __ldcg(q + 1);
      Fr v;
      v.v[0] = u0.x, v.v[1] = u0.y, v.v[2] = u0.z, v.v[3] = u0.w;
      v.v[4] = u1.x, v.v[5] = u1.y, v.v[6] = u1.z, v.v[7] = u1.w;
      a = fe_add(a, v);
    }
    red[threadIdx.x] = a;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
      if (threadIdx.x < (unsigned)off) red[threadIdx.x] = fe_add(red[threadIdx.x], red[threadIdx.x + off]);
      __syncthreads();
    }
    if (threadIdx.x == 0) st_fe(&A.out[x], red[0]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *A.done = 0;
}

// Resident blocks a SM k_round is compiled for (1: the compiler's choice).
#ifndef APG_ROUND_MIN_BLOCKS
#define APG_ROUND_MIN_BLOCKS 1
#endif
__global__ void __launch_bounds__(kRoundThreads, APG_ROUND_MIN_BLOCKS)
    k_round(RoundArgs A, DevProgram P, VirtualRound V, Fr* partials) {
  extern __shared__ uint32_t sm_raw[];
  const Slots sm = thread_slots(sm_raw);
  __shared__ Fr red[kRoundThreads];
  Fr acc[4];
#pragma unroll
  for (int x = 0; x < 4; ++x) acc[x] = fe_zero<FrConsts>();
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  if (A.xsplit) {
    // Small rounds: thread t evaluates pair t / 4 at node X = t % 4 alone
    // (X = 3 and, after the first round, X = 1 stay idle), so the evaluations
    // of a pair run side by side (latency, not work, is what bounds a round
    // with few pairs). Threads 4j..4j+3 of a block share a pair; the X = 0
    // thread stores the folded level.
    const int x = threadIdx.x & 3;
    // The X = 0 thread also stores the folded level, so it always runs.
    const bool on = x == 0 || ((A.nodes >> x) & 1);
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; on && t / 4 < A.npairs; t += stride) {
      const size_t i = t / 4;
      Fr lo, hi;
      for (int k = 0; k < A.nd; ++k) {
        load_line(A, k, i, lo, hi, x == 0);
        sm_st(sm, k, at_node(lo, fe_sub(hi, lo), x));
      }
      for (int v = 0; v < A.nv; ++v) {
        virtual_line_dev(V, A.vkinds[v], i, lo, hi);  // hi is the step here
        sm_st(sm, A.nd + v, at_node(lo, hi, x));
      }
      Fr e_lo, e_hi;
      load_line(A, A.nd, i, e_lo, e_hi, x == 0);
      acc[0] = fe_add(acc[0], fe_mul(fe_add(e_lo, e_hi), eval_summand(P, sm)));
    }
    // Reduce over threads of the same node: strides that are multiples of 4.
    red[threadIdx.x] = acc[0];
    __syncthreads();
    for (int off = blockDim.x / 2; off >= 4; off >>= 1) {
      if (threadIdx.x < (unsigned)off) red[threadIdx.x] = fe_add(red[threadIdx.x], red[threadIdx.x + off]);
      __syncthreads();
    }
    if (threadIdx.x < 4) st_fe(&partials[(size_t)blockIdx.x * 4 + threadIdx.x], red[threadIdx.x]);
    __syncthreads();
  } else {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < A.npairs; i += stride) {
    Fr lo, hi;
    for (int k = 0; k < A.nd; ++k) {
      load_line(A, k, i, lo, hi);
      sm_st(sm, k, lo);
      sm_st(sm, A.slots_step0 + k, fe_sub(hi, lo));
    }
    Fr e_lo, e_hi;
    load_line(A, A.nd, i, e_lo, e_hi);
    const Fr w = fe_add(e_lo, e_hi);  // the pair's eq weight without the current variable's factor
    for (int v = 0; v < A.nv; ++v) {
      virtual_line_dev(V, A.vkinds[v], i, lo, hi);
      sm_st(sm, A.nd + v, lo);
      sm_st(sm, A.slots_step0 + A.nd + v, hi);
    }
    for (int x = 0; x < 3; ++x) {
      if ((A.nodes >> x) & 1) {
        Fr s = eval_summand(P, sm);
        acc[x] = fe_add(acc[x], fe_mul(w, s));
      }
      if (x == 0 && !((A.nodes >> 1) & 1)) {  // straight to node 2: lo + 2 step
        for (int k = 0; k < A.n_val_slots; ++k) {
          const Fr st = sm_ld(sm, A.slots_step0 + k);
          sm_st(sm, k, fe_add(sm_ld(sm, k), fe_add(st, st)));
        }
        ++x;
      } else if (x < 2) {
        for (int k = 0; k < A.n_val_slots; ++k) sm_st(sm, k, fe_add(sm_ld(sm, k), sm_ld(sm, A.slots_step0 + k)));
      }
    }
  }
  // Block reduction, one node at a time through shared memory.
  for (int x = 0; x < 4; ++x) {
    red[threadIdx.x] = acc[x];
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
      if (threadIdx.x < (unsigned)off) red[threadIdx.x] = fe_add(red[threadIdx.x], red[threadIdx.x + off]);
      __syncthreads();
    }
    if (threadIdx.x == 0) st_fe(&partials[(size_t)blockIdx.x * 4 + x], red[0]);
    __syncthreads();
  }
  }
  round_total(A, partials, red);
}

// A summand S = sum_j c_j T_{a_j} T_{b_j} over data tables only (halving
// lists of tree gates, a zerocheck's product gate): thread per pair, each
// term's two lines read (and folded with the previous challenge) straight
// into registers and multiplied at the round's nodes, with no operand slots
// and no interpreter. Tables no term reads are folded too, so every table
// is bound each round as the generic kernel binds it.
struct PairTerms {
  const uint16_t* a;
  const uint16_t* b;
  const Fr* c;
  const uint8_t* unit;  // c_j == 1: its product is skipped
  const uint16_t* rest;
  int n, nrest;
};

// Four resident blocks a SM (128 registers a thread, no spills): the
// two-table zerocheck's rounds take 16 % less time than at the compiler's
// choice (166 registers, three blocks); five and six spill. The products are
// the interpreter's out-of-line rmul: inlined, the rounds took 15 % longer.
#ifndef APG_PAIRS_MIN_BLOCKS
#define APG_PAIRS_MIN_BLOCKS 4
#endif
__global__ void __launch_bounds__(kRoundThreads, APG_PAIRS_MIN_BLOCKS) k_round_pairs(RoundArgs A, PairTerms T, Fr* partials) {
  __shared__ Fr red[kRoundThreads];
  const bool n1 = (A.nodes >> 1) & 1;
  Fr acc0 = fe_zero<FrConsts>(), acc1 = fe_zero<FrConsts>(), acc2 = fe_zero<FrConsts>();
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < A.npairs; i += stride) {
    Fr lo, hi;
    for (int r = 0; r < T.nrest; ++r) load_line(A, T.rest[r], i, lo, hi);
    Fr s0 = fe_zero<FrConsts>(), s1 = fe_zero<FrConsts>(), s2 = fe_zero<FrConsts>();
    for (int j = 0; j < T.n; ++j) {
      Fr alo, ahi, blo, bhi;
      load_line(A, T.a[j], i, alo, ahi);
      load_line(A, T.b[j], i, blo, bhi);
      Fr p0 = rmul(alo, blo);
      Fr p2 = rmul(fe_sub(fe_add(ahi, ahi), alo), fe_sub(fe_add(bhi, bhi), blo));  // the lines at X = 2
      Fr p1 = n1 ? rmul(ahi, bhi) : fe_zero<FrConsts>();
      if (!T.unit[j]) {
        const Fr cj = ld_fe(&T.c[j]);
        p0 = rmul(cj, p0);
        p2 = rmul(cj, p2);
        if (n1) p1 = rmul(cj, p1);
      }
      s0 = fe_add(s0, p0);
      s2 = fe_add(s2, p2);
      if (n1) s1 = fe_add(s1, p1);
    }
    Fr e_lo, e_hi;
    load_line(A, A.nd, i, e_lo, e_hi);
    const Fr w = fe_add(e_lo, e_hi);  // the pair's eq weight without the current variable's factor
    acc0 = fe_add(acc0, rmul(w, s0));
    acc2 = fe_add(acc2, rmul(w, s2));
    if (n1) acc1 = fe_add(acc1, rmul(w, s1));
  }
  const Fr accs[4] = {acc0, acc1, acc2, fe_zero<FrConsts>()};
  for (int x = 0; x < 4; ++x) {
    red[threadIdx.x] = accs[x];
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
      if (threadIdx.x < (unsigned)off) red[threadIdx.x] = fe_add(red[threadIdx.x], red[threadIdx.x + off]);
      __syncthreads();
    }
    if (threadIdx.x == 0) st_fe(&partials[(size_t)blockIdx.x * 4 + x], red[0]);
    __syncthreads();
  }
  round_total(A, partials, red);
}

// The same summand in rounds with few pairs (the tops of halving lists): one
// thread per (pair, term), or per (pair, table no term reads), which only
// folds, so a pair's folds and products run side by side instead of as one
// thread's chain of a hundred products. Each term thread weighs its own term
// by c_j and the pair's eq weight; the block sums them all. The pair's eq
// line is stored by its first term's thread; a table two terms share is
// stored twice with the same value.
__global__ void __launch_bounds__(kRoundThreads) k_round_pairs_small(RoundArgs A, PairTerms T, Fr* partials) {
  __shared__ Fr red[kRoundThreads];
  const bool n1 = (A.nodes >> 1) & 1;
  const size_t per = (size_t)T.n + T.nrest;
  Fr acc0 = fe_zero<FrConsts>(), acc1 = fe_zero<FrConsts>(), acc2 = fe_zero<FrConsts>();
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < A.npairs * per; t += stride) {
    const size_t i = t / per;
    const int j = (int)(t - i * per);
    if (j >= T.n) {
      Fr lo, hi;
      load_line<APG_SMALL_OUTLINE>(A, T.rest[j - T.n], i, lo, hi);
      continue;
    }
    Fr alo, ahi, blo, bhi, e_lo, e_hi;
    load_line<APG_SMALL_OUTLINE>(A, T.a[j], i, alo, ahi);
    load_line<APG_SMALL_OUTLINE>(A, T.b[j], i, blo, bhi);
    load_line<APG_SMALL_OUTLINE>(A, A.nd, i, e_lo, e_hi, j == 0);
    Fr cw = fe_add(e_lo, e_hi);  // the pair's eq weight without the current variable's factor
    // The term's products at X = 0 and 2 (the lines at X = 2 are 2 hi - lo)
    // and its weight, two at a time.
    const FrPair p = rmul2(alo, blo, fe_sub(fe_add(ahi, ahi), alo), fe_sub(fe_add(bhi, bhi), blo));
    if (!T.unit[j]) cw = rmul(ld_fe(&T.c[j]), cw);
    const FrPair wp = rmul2(cw, p.a, cw, p.b);
    acc0 = fe_add(acc0, wp.a);
    acc2 = fe_add(acc2, wp.b);
    if (n1) acc1 = fe_add(acc1, rmul(cw, rmul(ahi, bhi)));
  }
  const Fr accs[4] = {acc0, acc1, acc2, fe_zero<FrConsts>()};
  for (int x = 0; x < 4; ++x) {
    red[threadIdx.x] = accs[x];
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
      if (threadIdx.x < (unsigned)off) red[threadIdx.x] = fe_add(red[threadIdx.x], red[threadIdx.x + off]);
      __syncthreads();
    }
    if (threadIdx.x == 0) st_fe(&partials[(size_t)blockIdx.x * 4 + x], red[0]);
    __syncthreads();
  }
  round_total(A, partials, red);
}

// Wide gate lists (many gates, many tables): one warp per pair. The pair's
// tables sit once in the warp's shared slots (values, then cached entries,
// then steps, then eq's value and step), written lane-parallel; at each node
// the lanes split the gates and the warp adds their weighted values.
// Five resident blocks a SM (96 registers, no spills) measured about 1 %
// faster than the unconstrained allocation (128 registers, four blocks).
#ifndef APG_ROUND_WARP_MIN_BLOCKS
#define APG_ROUND_WARP_MIN_BLOCKS 5
#endif
template <bool OUTLINE>
__global__ void __launch_bounds__(kRoundThreads, APG_ROUND_WARP_MIN_BLOCKS) k_round_warp(RoundArgs A, DevProgram P, VirtualRound V,
                                                              Fr* partials) {
  extern __shared__ uint32_t sm_raw[];
  __shared__ Fr red[kRoundThreads];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int per_warp = A.slots_step0 + A.n_val_slots + 2;
  const Slots S = warp_slots(sm_raw + (size_t)warp * per_warp * 8, per_warp);
  const int eq_slot = per_warp - 2;
  Fr acc[4];
#pragma unroll
  for (int x = 0; x < 4; ++x) acc[x] = fe_zero<FrConsts>();
  const size_t wstride = (size_t)gridDim.x * nwarps;
  for (size_t i = (size_t)blockIdx.x * nwarps + warp; i < A.npairs; i += wstride) {
    Fr lo, hi;
    for (int k = lane; k <= A.nd; k += 32) {
      load_line<OUTLINE>(A, k, i, lo, hi);
      if (k < A.nd) {
        sm_st(S, k, lo);
        sm_st(S, A.slots_step0 + k, fe_sub(hi, lo));
      } else {
        sm_st(S, eq_slot, fe_add(lo, hi));  // the pair's eq weight without the current variable's factor
      }
    }
    for (int v = lane; v < A.nv; v += 32) {
      virtual_line_dev(V, A.vkinds[v], i, lo, hi);  // hi is the step here
      sm_st(S, A.nd + v, lo);
      sm_st(S, A.slots_step0 + A.nd + v, hi);
    }
    __syncwarp();
    for (int x = 0; x < 3; ++x) {
      if ((A.nodes >> x) & 1) {  // uniform across the warp
        if (lane == 0)
          for (int g = 0; g < P.n_cached; ++g) sm_st(S, P.cached_slot0 + g, eval_gate_dev(P, g, S));
        __syncwarp();
        Fr part = fe_zero<FrConsts>();
        for (int j = lane; j < P.n_weighted; j += 32)
          part = fe_add(part, weigh(P, j, eval_gate_dev(P, P.n_cached + j, S)));
        for (int off = 16; off > 0; off >>= 1) {
          Fr o;
#pragma unroll
          for (int w = 0; w < 8; ++w) o.v[w] = __shfl_xor_sync(0xffffffffu, part.v[w], off);
          part = fe_add(part, o);
        }
        if (lane == 0) acc[x] = fe_add(acc[x], OUTLINE ? rmul(sm_ld(S, eq_slot), part) : fe_mul(sm_ld(S, eq_slot), part));
      }
      __syncwarp();
      if (x == 0 && !((A.nodes >> 1) & 1)) {  // straight to node 2: lo + 2 step
        for (int k = lane; k < A.n_val_slots; k += 32) {
          const Fr st = sm_ld(S, A.slots_step0 + k);
          sm_st(S, k, fe_add(sm_ld(S, k), fe_add(st, st)));
        }
        ++x;
      } else if (x < 2) {
        for (int k = lane; k < A.n_val_slots; k += 32) sm_st(S, k, fe_add(sm_ld(S, k), sm_ld(S, A.slots_step0 + k)));
      }
      __syncwarp();
    }
  }
  // Per node: the block's warps' sums (lane 0 of each), then the cross-block total.
  for (int x = 0; x < 4; ++x) {
    red[threadIdx.x] = lane == 0 ? acc[x] : fe_zero<FrConsts>();
    __syncthreads();
    if (threadIdx.x == 0) {
      Fr a = fe_zero<FrConsts>();
      for (int w = 0; w < nwarps; ++w) a = fe_add(a, red[32 * w]);
      st_fe(&partials[(size_t)blockIdx.x * 4 + x], a);
    }
    __syncthreads();
  }
  round_total(A, partials, red);
}

// Tables of length 2 -> their bound value (the last round's fold).
// With no rounds at all (a one-entry table) c is ignored and the entry itself
// is the value.
__global__ void k_final_bind(const Fr* const* src, const uint8_t* src_bits, const Fr* in_base, size_t in_len,
                             int in_is_src, int nt, Fr c, int no_rounds, Fr* out) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  const Fr* t = in_is_src ? src[k] : in_base + (size_t)k * in_len;
  const int bits = in_is_src && src_bits ? src_bits[k] : 0;
  const Fr a0 = bits ? narrow_entry(t, bits, 0) : ld_fe(&t[0]);
  if (no_rounds) {
    st_fe(&out[k], a0);
    return;
  }
  const Fr a1 = bits ? narrow_entry(t, bits, 1) : ld_fe(&t[1]);
  st_fe(&out[k], fe_add(a0, fe_mul(c, fe_sub(a1, a0))));
}

__global__ void k_lift(const void* p, int bits, size_t n, Fr* out) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) st_fe(&out[i], narrow_entry(p, bits, i));
}

// eq(r, y) for every y < 2^n: prod_j (y_j ? r_j : 1 - r_j).
__global__ void k_eq_table(const Fr* r, int n, size_t len, Fr* out) {
  size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (y >= len) return;
  Fr acc = fe_one<FrConsts>();
  for (int j = 0; j < n; ++j) {
    Fr rj = ld_fe(&r[j]);
    acc = fe_mul(acc, ((y >> j) & 1) ? rj : fe_sub(fe_one<FrConsts>(), rj));
  }
  st_fe(&out[y], acc);
}

// out[y] = lo[y mod 2^nlo] * hi[y >> nlo]: eq(r, y) split at bit nlo.
__global__ void k_eq_combine(const Fr* lo, const Fr* hi, int nlo, size_t len, Fr* out) {
  size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (y >= len) return;
  st_fe(&out[y], fe_mul(ld_fe(&lo[y & (((size_t)1 << nlo) - 1)]), ld_fe(&hi[y >> nlo])));
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

using host::F;

static Fr to_dev(const F& a) {
  Fr r;
  memcpy(r.v, a.w, 32);
  return r;
}

// eq(r, y) for every y < 2^|r|. Up to 12 variables each entry is its own
// product of |r| factors; beyond, the two halves' tables (2^(n/2) entries
// each) are built that way and every entry is one product of the two.
void lift_column(Ctx& c, const void* p, int bits, size_t n, Fr* out) {
  if (n) launch(c, k_lift, (unsigned)((n + 255) / 256), 256, 0, p, bits, n, out);
}

void build_eq_table(Ctx& c, const std::vector<F>& r, Fr* out) {
  const int n = (int)r.size();
  const size_t len = (size_t)1 << n;
  const int nlo = n / 2, nhi = n - nlo;
  const bool split = n > 12;
  const size_t lo_len = (size_t)1 << nlo, hi_len = (size_t)1 << nhi;
  Fr* d_r = c.scratch[S_TMP4].as<Fr>(std::max<size_t>(n, 1) + (split ? lo_len + hi_len : 0));
  if (n) APG_CUDA(cudaMemcpyAsync(d_r, r.data(), 32 * (size_t)n, cudaMemcpyHostToDevice, c.stream));
  if (!split) {
    launch(c, k_eq_table, (unsigned)((len + 255) / 256), 256, 0, (const Fr*)d_r, n, len, out);
    return;
  }
  Fr* lo = d_r + n;
  Fr* hi = lo + lo_len;
  launch(c, k_eq_table, (unsigned)((lo_len + 255) / 256), 256, 0, (const Fr*)d_r, nlo, lo_len, lo);
  launch(c, k_eq_table, (unsigned)((hi_len + 255) / 256), 256, 0, (const Fr*)(d_r + nlo), nhi, hi_len, hi);
  launch(c, k_eq_combine, (unsigned)((len + 255) / 256), 256, 0, (const Fr*)lo, (const Fr*)hi, nlo, len, out);
}

static VirtualRound virtual_round(const std::vector<F>& point, int nvars) {
  using namespace host;
  VirtualRound V;
  memset(&V, 0, sizeof(V));
  const int b = (int)point.size();
  V.bound = b;
  V.nvars = nvars;
  F row = fzero(), r19 = fzero(), r16 = fzero(), q = fone(), pw = fone();
  for (int j = 0; j < b; ++j) {
    F t = fmul(point[j], pw);
    row = fadd(row, t);
    if (j < 19) r19 = fadd(r19, t);
    if (j < 16) r16 = fadd(r16, t);
    if (j >= 14) q = fmul(q, fsub(fone(), point[j]));
    if (j < 16) V.r16[j] = to_dev(point[j]);
    pw = fadd(pw, pw);
  }
  V.row_prefix = to_dev(row);
  V.range19_prefix = to_dev(r19);
  V.range16_prefix = to_dev(r16);
  V.ram_q = to_dev(q);
  V.pow2_b = to_dev(pw);
  return V;
}

void run_sumcheck(Ctx& c, const DevProgram& prog, int nd, const std::vector<uint8_t>& vkinds, int n_cached,
                  const std::vector<const Fr*>& src, const std::vector<F>& eq_point, host::Transcript& tr,
                  std::vector<std::array<F, 4>>& rounds, std::vector<F>& point, std::vector<F>& finals,
                  const std::vector<uint8_t>& src_bits, const HostPairTerms* pairs) {
  const int n = (int)eq_point.size();
  const int nt = nd + 1;  // with eq
  if (vkinds.size() > 8) throw Error(APG_ERR_BAD_CIRCUIT, "more than 8 virtual tables");
  rounds.clear();
  point.clear();
  finals.assign(nd, host::fzero());

  // Round-0 sources: the data tables, then eq built from the eq point.
  const size_t len0 = (size_t)1 << n;
  Fr* eq = c.scratch[S_TMP3].as<Fr>(len0);
  build_eq_table(c, eq_point, eq);
  std::vector<const Fr*> srcs(src);
  srcs.push_back(eq);
  const Fr** d_src = c.scratch[S_TMP5].as<const Fr*>(nt);
  APG_CUDA(cudaMemcpyAsync(d_src, srcs.data(), sizeof(Fr*) * nt, cudaMemcpyHostToDevice, c.stream));
  // Stored widths of the data tables, when any is narrow (eq is Fr).
  const uint8_t* d_bits = nullptr;
  bool narrow = false;
  for (uint8_t b : src_bits) narrow |= b != 0;
  if (narrow) {
    if ((int)src_bits.size() != nd) throw Error(APG_ERR_INTERNAL, "one width per data table");
    std::vector<uint8_t> bits(src_bits);
    bits.push_back(0);
    uint8_t* db = c.scratch[S_ENTRIES].as<uint8_t>(nt);
    APG_CUDA(cudaMemcpyAsync(db, bits.data(), nt, cudaMemcpyHostToDevice, c.stream));
    APG_CUDA(cudaStreamSynchronize(c.stream));  // `bits` is a host temporary
    d_bits = db;
  }

  // Level buffers: level r (r >= 1) holds nt tables of 2^(n-r) entries.
  Fr* lvl[2] = {nullptr, nullptr};
  if (n >= 2) {
    lvl[1] = c.scratch[S_LEVEL_A].as<Fr>((size_t)nt * (len0 / 2));
    lvl[0] = c.scratch[S_LEVEL_B].as<Fr>((size_t)nt * (len0 / 4 > 0 ? len0 / 4 : 1));
  }
  const int n_val = nd + (int)vkinds.size();
  const int slots = 2 * n_val + n_cached;
  // Wide gate lists get narrower blocks (a power of two, for the reduction
  // tree) so that every thread's slots still fit in shared memory.
  // (Down to 8 threads a block for the widest lists, e.g. 130-column ones.)
  int threads = kRoundThreads;
  while (threads > 8 && (size_t)std::max(slots, 1) * 32 * threads > 200 * 1024) threads /= 2;
  const size_t smem = (size_t)std::max(slots, 1) * 32 * threads;
  // Lists of many gates go one pair per warp (k_round_warp): the pair's
  // tables are stored once for the warp instead of once per thread.
  const bool warp_mode = prog.n_weighted >= kWarpModeGates;
  if (!warp_mode && smem > 200 * 1024) throw Error(APG_ERR_BAD_CIRCUIT, "gate list too wide for one thread block");
  APG_CUDA(cudaFuncSetAttribute(k_round, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  const int max_blocks = c.sm_count * 8 * (kRoundThreads / threads);  // the same thread count in smaller blocks
  const int warp_slots = n_val + n_cached + n_val + 2;
  const size_t warp_smem = (size_t)(kRoundThreads / 32) * warp_slots * 32;
  if (warp_mode && warp_smem > 200 * 1024) throw Error(APG_ERR_BAD_CIRCUIT, "gate list too wide for one thread block");
  if (warp_mode) APG_CUDA(cudaFuncSetAttribute(k_round_warp<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  // Rounds with few enough pairs for one warp each in a single wave run one
  // pair per warp whatever the list's width (APG_SMALL_WARP): the lanes fold
  // the tables and evaluate the gates side by side, so a round's latency is a
  // fold and a gate, not one thread's chain through every fold and gate.
  const bool small_warp_ok = APG_SMALL_WARP && warp_smem <= 200 * 1024;
  if (small_warp_ok)
    APG_CUDA(cudaFuncSetAttribute(k_round_warp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  const int warp_max_blocks = c.sm_count * 16;
  Fr* partials = c.scratch[S_TMP6].as<Fr>((size_t)std::max(max_blocks, warp_max_blocks) * 4);
  Fr* d_out = c.scratch[S_RESULT].as<Fr>(4);
  unsigned* done = c.scratch[S_ROUND].as<unsigned>(1);
  APG_CUDA(cudaMemsetAsync(done, 0, sizeof(unsigned), c.stream));
  F* sums = reinterpret_cast<F*>(c.host_pinned());
  DevProgram P = prog;
  P.cached_slot0 = n_val;
  // The pair-term kernel's tables on the device (when the summand has that form).
  PairTerms PT;
  memset(&PT, 0, sizeof(PT));
  const bool use_pairs = pairs && vkinds.empty() && n_cached == 0 && !pairs->a.empty();
  if (use_pairs) {
    const size_t nt_ = pairs->a.size(), nr = pairs->rest.size();
    const size_t cb = 32 * nt_, ab = 2 * nt_, rb = 2 * std::max<size_t>(nr, 1), ub = nt_;
    const size_t total = cb + 2 * ab + rb + ub + 4 * 32;
    uint8_t* d = c.scratch[S_PAIR_TERMS].as<uint8_t>(total);
    std::vector<uint8_t> h(total, 0);
    size_t off = 0;
    auto put = [&](const void* p, size_t n) {
      const size_t at = (off + 31) & ~(size_t)31;
      if (n) memcpy(h.data() + at, p, n);
      off = at + n;
      return d + at;
    };
    std::vector<uint8_t> unit(nt_);
    for (size_t j = 0; j < nt_; ++j) unit[j] = pairs->c[j] == host::fone() ? 1 : 0;
    PT.c = reinterpret_cast<const Fr*>(put(pairs->c.data(), cb));
    PT.a = reinterpret_cast<const uint16_t*>(put(pairs->a.data(), ab));
    PT.b = reinterpret_cast<const uint16_t*>(put(pairs->b.data(), ab));
    PT.rest = reinterpret_cast<const uint16_t*>(put(pairs->rest.data(), 2 * nr));
    PT.unit = put(unit.data(), ub);
    PT.n = (int)nt_;
    PT.nrest = (int)nr;
    APG_CUDA(cudaMemcpyAsync(d, h.data(), total, cudaMemcpyHostToDevice, c.stream));
    APG_CUDA(cudaStreamSynchronize(c.stream));  // `h` is a host temporary
  }

  // 1/r_j for every nonzero eq coordinate, from one inversion (Montgomery's
  // batch trick): the rounds divide by their coordinate.
  std::vector<F> inv_r(n, host::fzero());
  {
    std::vector<F> pre(n + 1, host::fone());
    for (int j = 0; j < n; ++j) pre[j + 1] = eq_point[j].zero() ? pre[j] : host::fmul(pre[j], eq_point[j]);
    F inv = host::finv(pre[n]);
    for (int j = n; j-- > 0;) {
      if (eq_point[j].zero()) continue;
      inv_r[j] = host::fmul(inv, pre[j]);
      inv = host::fmul(inv, eq_point[j]);
    }
  }
  F chal = host::fzero();
  for (int r = 0; r < n; ++r) {
    RoundArgs A;
    memset(&A, 0, sizeof(A));
    A.nd = nd;
    A.nv = (int)vkinds.size();
    for (size_t v = 0; v < vkinds.size(); ++v) A.vkinds[v] = vkinds[v];
    A.src = d_src;
    A.bind = r > 0;
    A.c = to_dev(chal);
    A.in_is_src = r <= 1;
    A.in_len = (size_t)1 << (n - r + (r > 0 ? 1 : 0));
    A.in_base = r >= 2 ? lvl[(r - 1) & 1] : nullptr;
    A.out_base = r >= 1 ? lvl[r & 1] : nullptr;
    A.npairs = (size_t)1 << (n - r - 1);
    A.slots_step0 = n_val + n_cached;
    A.n_val_slots = n_val;
    A.done = done;
    A.out = d_out;
    VirtualRound V = virtual_round(point, n);
    // Rounds too small to fill the device evaluate the nodes of a pair on
    // threads of their own.
    A.xsplit = A.npairs * 4 <= (size_t)threads * max_blocks ? 1 : 0;
    A.src_bits = d_bits;
    // The round polynomial factors as s(X) = eq_r(X) q(X): eq's factor for
    // this variable, eq_r(X) = (1 - r_r)(1 - X) + r_r X, is common to every
    // pair, and the rest of a pair's eq weight is e(2i) + e(2i + 1). The
    // device sums q at nodes 0 and 2 (q has degree 2); from the second round
    // on q(1) follows from s(0) + s(1) = s_{r-1}(c_{r-1}), which holds for any
    // tables because the bound tables are the lines at c. Round 0, and a round
    // whose eq coordinate is 0, evaluate node 1 as well.
    const F rr = eq_point[r];
    const bool need1 = r == 0 || rr.zero();
    A.nodes = need1 ? 7 : 5;
    const size_t work = A.xsplit ? A.npairs * 4 : A.npairs;
    const int blocks = warp_mode
                           ? (int)std::min<size_t>((A.npairs + kRoundThreads / 32 - 1) / (kRoundThreads / 32),
                                                   (size_t)warp_max_blocks)
                           : (int)std::min<size_t>((work + threads - 1) / threads, (size_t)max_blocks);
    cudaEvent_t t0 = c.timer_begin();
    if (use_pairs && !A.xsplit)
      launch(c, k_round_pairs, (int)std::min<size_t>((A.npairs + kRoundThreads - 1) / kRoundThreads,
                                                     (size_t)c.sm_count * 8),
             kRoundThreads, 0, A, PT, partials);
    else if (use_pairs && PT.n + PT.nrest >= 4)  // (one or two terms: the node-split generic rounds were faster)
      launch(c, k_round_pairs_small,
             (int)std::min<size_t>((A.npairs * (size_t)(PT.n + PT.nrest) + kRoundThreads - 1) / kRoundThreads,
                                   (size_t)c.sm_count * 8),
             kRoundThreads, 0, A, PT, partials);
    else if (small_warp_ok && A.npairs * 32 <= (size_t)kRoundThreads * c.sm_count * 4)
      launch(c, k_round_warp<true>, (int)((A.npairs + kRoundThreads / 32 - 1) / (kRoundThreads / 32)), kRoundThreads,
             warp_smem, A, P, V, partials);
    else if (warp_mode) launch(c, k_round_warp<false>, blocks, kRoundThreads, warp_smem, A, P, V, partials);
    else launch(c, k_round, blocks, threads, smem, A, P, V, partials);
    c.timer_end(APG_TIMER_SUMCHECK_ROUND, t0);
    APG_CUDA(cudaMemcpyAsync(sums, d_out, 128, cudaMemcpyDeviceToHost, c.stream));
    APG_CUDA(cudaStreamSynchronize(c.stream));
    const auto host0 = std::chrono::steady_clock::now();
    F q[4] = {sums[0], sums[1], sums[2], host::fzero()};
    const F one_m_r = host::fsub(host::fone(), rr);
    if (!need1) {
      const auto& gp = rounds.back();  // s_{r-1}(X), ascending coefficients
      const F claim = host::fadd(
          gp[0], host::fmul(chal, host::fadd(gp[1], host::fmul(chal, host::fadd(gp[2], host::fmul(chal, gp[3]))))));
      q[1] = host::fmul(host::fsub(claim, host::fmul(one_m_r, q[0])), inv_r[r]);
    }
    // q(3) = q(0) - 3 q(1) + 3 q(2); s(X) = eq_r(X) q(X) with eq_r(X) = 1 - r - X + 2 r X.
    const F three = host::from_u64(3);
    q[3] = host::fadd(q[0], host::fmul(three, host::fsub(q[2], q[1])));
    F sv[4];
    F eqx = one_m_r;                          // eq_r(0)
    const F step = host::fsub(host::fadd(rr, rr), host::fone());  // eq_r(X + 1) - eq_r(X) = 2r - 1
    for (int x = 0; x < 4; ++x) {
      sv[x] = host::fmul(eqx, q[x]);
      eqx = host::fadd(eqx, step);
    }
    auto g = host::cubic_through(sv);
    tr.absorb(host::T_SUMCHECK_ROUND, g.data(), 4);
    chal = tr.challenge(host::T_SUMCHECK_CHALLENGE);
    rounds.push_back(g);
    point.push_back(chal);
    if (c.timers.on) {  // the host's share of a round: interpolation and the transcript step
      c.timers.ms[APG_TIMER_HOST_ROUND] +=
          std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - host0).count();
      c.timers.count[APG_TIMER_HOST_ROUND] += 1;
    }
  }
  // The last fold: every table bound to the full point.
  Fr* d_fin = c.scratch[S_TMP7].as<Fr>(nt);
  if (nd > 0) {
    const Fr* base = n >= 2 ? lvl[(n - 1) & 1] : nullptr;
    launch(c, k_final_bind, (unsigned)((nd + 63) / 64), 64, 0, (const Fr* const*)d_src, d_bits, base, (size_t)2,
           n <= 1 ? 1 : 0, nd, to_dev(chal), n == 0 ? 1 : 0, d_fin);
    APG_CUDA(cudaMemcpyAsync(finals.data(), d_fin, 32 * (size_t)nd, cudaMemcpyDeviceToHost, c.stream));
  }
  APG_CUDA(cudaStreamSynchronize(c.stream));
}

// A device copy of a resolved gate list.
namespace {

// A summed gate list without cached entries is one quadratic form in its
// slots: S = sum_j w_j g_j = C + sum_i A_i x_i + sum_{a<=b} B_ab x_a x_b.
// Expanding every gate into those monomials (weights applied on the host)
// and merging equal monomials across gates needs fewer products per node
// than evaluating the gates one by one when the gates share operands (the
// reference's family circuits: about 30 % fewer). The form is emitted as
// quadratic gates of at most kLinChunk coefficients, weight 1, so the lanes
// of a warp still split the work and every coefficient is under the 0/1/-1
// masks. Exact field arithmetic: the sum is the same at every node.
constexpr int kLinChunk = 31;

bool linearize(HostProgram& hp) {
  if (!hp.summed || hp.n_cached != 0 || hp.n_weighted < kWarpModeGates) return false;
  const F one = host::fone(), zero = host::fzero(), minus_one = host::fneg(host::fone());
  auto triv = [&](const F& v) { return v == zero || v == one || v == minus_one; };
  F cst = zero;
  std::map<uint16_t, F> lin;
  std::map<std::pair<uint16_t, uint16_t>, F> quad;
  auto add_lin = [&](uint16_t a, const F& v) { lin[a] = host::fadd(lin.count(a) ? lin[a] : zero, v); };
  auto add_quad = [&](uint16_t a, uint16_t b, const F& v) {
    const auto k = a < b ? std::make_pair(a, b) : std::make_pair(b, a);
    quad[k] = host::fadd(quad.count(k) ? quad[k] : zero, v);
  };
  long now = 0;  // products a node as the gates stand
  for (int j = 0; j < hp.n_weighted; ++j) {
    const DevGate& g = hp.gates[j];
    const F w = j < (int)hp.weights.size() ? hp.weights[j] : one;
    const F* c = hp.coeffs.data() + g.cf_off;
    const uint16_t* o = hp.ops.data() + g.op_off;
    const int t = g.p1, u = g.p2;
    now += w == one ? 0 : 1;
    switch (g.kind) {
      case G_LINEAR:
        for (int i = 0; i < t; ++i) add_lin(o[i], host::fmul(w, c[i])), now += triv(c[i]) ? 0 : 1;
        cst = host::fadd(cst, host::fmul(w, c[t]));
        break;
      case G_PRODUCT:
        add_quad(o[0], o[1], host::fmul(w, c[0]));
        now += 1 + (triv(c[0]) ? 0 : 1);
        break;
      case G_MASK:  // x m + 1 - m
        add_quad(o[0], o[1], w);
        add_lin(o[1], host::fneg(w));
        cst = host::fadd(cst, w);
        now += 1;
        break;
      case G_AFFINE: {  // (sum l_i x_i + l_t)(sum r_k y_k + r_u)
        const F lt = c[t], ru = c[t + 1 + u];
        for (int i = 0; i < t; ++i) {
          for (int k = 0; k < u; ++k) add_quad(o[i], o[t + k], host::fmul(w, host::fmul(c[i], c[t + 1 + k])));
          add_lin(o[i], host::fmul(w, host::fmul(c[i], ru)));
          now += triv(c[i]) ? 0 : 1;
        }
        for (int k = 0; k < u; ++k) {
          add_lin(o[t + k], host::fmul(w, host::fmul(lt, c[t + 1 + k])));
          now += triv(c[t + 1 + k]) ? 0 : 1;
        }
        cst = host::fadd(cst, host::fmul(w, host::fmul(lt, ru)));
        now += 1;
        break;
      }
      case G_TREE_PRODUCT:
        add_quad(o[0], o[1], w);
        now += 1;
        break;
      case G_TREE_CROSS:
        add_quad(o[0], o[3], w);
        add_quad(o[1], o[2], w);
        now += 2;
        break;
      case G_QUADRATIC:
        cst = host::fadd(cst, host::fmul(w, c[0]));
        for (int i = 0; i < t; ++i) add_lin(o[i], host::fmul(w, c[1 + i])), now += triv(c[1 + i]) ? 0 : 1;
        for (int k = 0; k < u; ++k) {
          if (c[1 + t + k] == zero) continue;
          add_quad(o[t + 2 * k], o[t + 2 * k + 1], host::fmul(w, c[1 + t + k]));
          now += 1 + (triv(c[1 + t + k]) ? 0 : 1);
        }
        break;
      default:
        return false;
    }
  }
  std::vector<std::pair<uint16_t, F>> L;
  std::vector<std::pair<std::pair<uint16_t, uint16_t>, F>> Q;
  long lin_cost = 0;
  for (auto& e : lin)
    if (e.second != zero) L.push_back(e), lin_cost += triv(e.second) ? 0 : 1;
  for (auto& e : quad)
    if (e.second != zero) Q.push_back(e), lin_cost += 1 + (triv(e.second) ? 0 : 1);
  if (lin_cost >= now) return false;
  // Chunks of at most kLinChunk coefficients (the constant rides in chunk 0),
  // at least one a lane of the warp.
  const size_t terms = L.size() + Q.size();
// At least 96 chunks (about three a lane): measured 3-5 % faster than 32, 64,
// 128 or 192 on the reference's add_sub and shift_bitwise circuits.
#ifndef APG_LIN_MIN_CHUNKS
#define APG_LIN_MIN_CHUNKS 96
#endif
  const size_t chunks = std::max<size_t>((terms + kLinChunk - 2) / (kLinChunk - 1), APG_LIN_MIN_CHUNKS);
  const size_t per = std::max<size_t>(1, (terms + chunks - 1) / chunks);
  std::vector<DevGate> gates;
  std::vector<uint16_t> ops;
  std::vector<F> coeffs;
  size_t li = 0, qi = 0;
  bool first = true;
  while (first || li < L.size() || qi < Q.size()) {
    DevGate d;
    memset(&d, 0, sizeof(d));
    d.kind = G_QUADRATIC;
    d.op_off = (uint32_t)ops.size();
    d.cf_off = (uint32_t)coeffs.size();
    coeffs.push_back(first ? cst : zero);
    first = false;
    size_t take = per;
    int t = 0, u = 0;
    std::vector<F> qc;
    std::vector<uint16_t> qo;
    while (take && li < L.size()) {
      ops.push_back(L[li].first);
      coeffs.push_back(L[li].second);
      ++li, ++t, --take;
    }
    while (take && qi < Q.size()) {
      qo.push_back(Q[qi].first.first);
      qo.push_back(Q[qi].first.second);
      qc.push_back(Q[qi].second);
      ++qi, ++u, --take;
    }
    ops.insert(ops.end(), qo.begin(), qo.end());
    coeffs.insert(coeffs.end(), qc.begin(), qc.end());
    d.p1 = (uint16_t)t;
    d.p2 = (uint16_t)u;
    d.nops = (uint16_t)(t + 2 * u);
    gates.push_back(d);
  }
  hp.gates = gates;
  hp.ops = ops;
  hp.coeffs = coeffs;
  hp.n_weighted = (int)gates.size();
  hp.weights.assign(gates.size(), one);
  return true;
}

}  // namespace

bool pair_terms_of(const HostProgram& hp, int nd, HostPairTerms& out) {
  out = HostPairTerms();
  if (hp.n_cached != 0 || hp.n_weighted <= 0) return false;
  const F one = host::fone(), zero = host::fzero();
  // Terms over the same two tables merge (exact arithmetic: the sum is the
  // same at every node).
  std::map<std::pair<uint16_t, uint16_t>, F> merged;
  auto term = [&](uint16_t a, uint16_t b, const F& cf) {
    if (a >= nd || b >= nd) return false;
    const auto k = a < b ? std::make_pair(a, b) : std::make_pair(b, a);
    auto it = merged.find(k);
    if (it == merged.end()) merged.emplace(k, cf);
    else it->second = host::fadd(it->second, cf);
    return true;
  };
  for (int j = 0; j < hp.n_weighted; ++j) {
    const DevGate& g = hp.gates[j];
    const F W = j < (int)hp.weights.size() ? hp.weights[j] : one;
    const uint16_t* op = hp.ops.data() + g.op_off;
    const F* cf = hp.coeffs.data() + g.cf_off;
    bool ok = false;
    switch (g.kind) {
      case G_TREE_PRODUCT:  // v0 v1
        ok = g.nops == 2 && term(op[0], op[1], W);
        break;
      case G_PRODUCT:  // c v0 v1
        ok = g.nops == 2 && term(op[0], op[1], host::fmul(cf[0], W));
        break;
      case G_TREE_CROSS:  // v0 v3 + v1 v2
        ok = g.nops == 4 && term(op[0], op[3], W) && term(op[1], op[2], W);
        break;
      case G_QUADRATIC:  // c0 + linear + products: products only
        ok = g.p1 == 0 && cf[0] == zero && g.nops == 2 * g.p2;
        for (uint32_t u = 0; ok && u < g.p2; ++u) ok = term(op[2 * u], op[2 * u + 1], host::fmul(cf[1 + u], W));
        break;
      default:
        ok = false;
    }
    if (!ok) {
      out = HostPairTerms();
      return false;
    }
  }
  for (auto& kv : merged) {
    if (kv.second == zero) continue;
    out.a.push_back(kv.first.first);
    out.b.push_back(kv.first.second);
    out.c.push_back(kv.second);
  }
  if (out.a.empty() || out.a.size() > 4096) {
    out = HostPairTerms();
    return false;
  }
  std::vector<char> used(nd, 0);
  for (size_t j = 0; j < out.a.size(); ++j) used[out.a[j]] = used[out.b[j]] = 1;
  for (int k = 0; k < nd; ++k)
    if (!used[k]) out.rest.push_back((uint16_t)k);
  return true;
}

void upload_program(Ctx& c, const HostProgram& hp_in, DevProgram& P, int slot_cap) {
  (void)slot_cap;
  HostProgram hp = hp_in;
  linearize(hp);
  std::vector<DevGate> gates = hp.gates;
  const std::vector<F>& coeffs = hp.coeffs;
  std::vector<F> weights = hp.weights;
  // Weights equal to 1 (lambda^0, a zerocheck's gate) skip their product.
  // Folding the other weights into the gates' coefficients was measured and
  // was slower: it turns coefficients of 1 and -1, which cost nothing, into
  // products.
  for (auto& g : gates) g.flags = 0;
  for (size_t j = 0; j < weights.size() && hp.n_cached + j < gates.size(); ++j)
    if (weights[j] == host::fone()) gates[hp.n_cached + j].flags |= kGateUnitWeight;
  // Mark unit coefficients so the device skips their products.
  const host::F one = host::fone(), minus_one = host::fneg(host::fone()), zero = host::fzero();
  for (auto& g : gates) {
    g.ones = g.negs = g.zeros = 0;
    for (uint32_t i = 0; i < 32 && g.cf_off + i < coeffs.size(); ++i) {
      const host::F& v = coeffs[g.cf_off + i];
      if (v == one) g.ones |= 1u << i;
      else if (v == minus_one) g.negs |= 1u << i;
      else if (v == zero) g.zeros |= 1u << i;
    }
  }
  // The weighted sum does not depend on the order of its gates: group gates
  // of one shape together (with their weights), so the lanes of a warp that
  // evaluate consecutive gates take the same code path (measured: the add_sub
  // circuit's proof 17 % faster; sorting on the 0/1/-1 coefficient patterns
  // as well gained nothing more).
  if (hp.summed) {
    const int n0 = hp.n_cached, nw = hp.n_weighted;
    std::vector<int> perm(nw);
    for (int j = 0; j < nw; ++j) perm[j] = j;
    auto key = [&](int j) {
      const DevGate& g = gates[n0 + j];
      return std::make_tuple(g.kind, g.flags, g.p1, g.p2, g.nops);
    };
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return key(a) < key(b); });
    std::vector<DevGate> wg(nw);
    std::vector<F> ww(nw);
    for (int j = 0; j < nw; ++j) {
      wg[j] = gates[n0 + perm[j]];
      ww[j] = perm[j] < (int)weights.size() ? weights[perm[j]] : host::fone();
    }
    for (int j = 0; j < nw; ++j) gates[n0 + j] = wg[j];
    weights = ww;
  }
  const size_t gb = gates.size() * sizeof(DevGate);
  const size_t ob = hp.ops.size() * sizeof(uint16_t);
  const size_t cb = coeffs.size() * 32;
  const size_t wb = weights.size() * 32;
  const size_t total = gb + ob + cb + wb + 256;
  uint8_t* d = c.scratch[S_TMP2].as<uint8_t>(total);
  std::vector<uint8_t> h(total, 0);
  size_t off = 0;
  auto put = [&](const void* p, size_t n) {
    size_t at = (off + 31) & ~(size_t)31;
    if (n) memcpy(h.data() + at, p, n);
    off = at + n;
    return d + at;
  };
  P.gates = (const DevGate*)put(gates.data(), gb);
  P.ops = (const uint16_t*)put(hp.ops.data(), ob);
  P.coeffs = (const Fr*)put(coeffs.data(), cb);
  P.weights = (const Fr*)put(weights.data(), wb);
  P.n_cached = hp.n_cached;
  P.n_weighted = hp.n_weighted;
  APG_CUDA(cudaMemcpyAsync(d, h.data(), off, cudaMemcpyHostToDevice, c.stream));
}

}  // namespace apg
