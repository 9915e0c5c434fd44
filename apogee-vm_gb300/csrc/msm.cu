// Pippenger MSM on sm_103a (replaces crates/curve/src/msm.rs:48-311).
//
// Pipeline for a group of columns over the same bases, all on the context's
// stream (msm_group):
//  1. k_digits      one thread per scalar: Montgomery -> canonical, signed
//                   c-bit digits in [-2^(c-1), 2^(c-1)] (the reference's
//                   recoding rule, msm.rs:180-198) and a histogram of bucket
//                   occupancy with warp-aggregated atomics.
//  2. scan          exclusive scan of the histogram (bucket starts).
//  3. k_digits      the same digits again, each placed as a 4-byte reference
//                   at its bucket's cursor: a counting sort without an
//                   intermediate entry list.
//  4. k_bucket_acc  persistent, load-balanced bucket accumulation: one wave of
//                   threads, each folding an equal slice of the sorted list
//                   run by run into XYZZ accumulators with mixed adds; runs cut
//                   by a slice edge are stitched by k_fold_edges.
//  5. k_level/k_sum bucket reduction sum_k k*B_k as a tree of running sums,
//                   every column's bucket range at once.
//  6. k_finish_cols per column, combine windows (Horner) or, with a
//                   precomputed SRS window table, nothing: there every window
//                   shares one bucket set because the table already holds
//                   2^(c*w) * P_i; then the canonical affine encoding.
// The allocation-free variant at the end of this file keeps the first
// single-MSM form of the pipeline (k_recode, k_scatter, k_accumulate, k_finish).
#include "common.cuh"

namespace apg {

namespace {

constexpr int kLevelFan = 8;  // buckets folded per thread in one reduction level

__device__ __forceinline__ void raise_flag(uint32_t* flags, uint32_t f) { atomicOr(flags, f); }

__device__ __forceinline__ Fq fq_const_u32(uint32_t v) {
  Fq a = fe_zero<FqConsts>();
  a.v[0] = v;
  return fe_to_mont(a);
}

__device__ __forceinline__ Affine generator_affine() {
  Affine g;
  g.x = fe_one<FqConsts>();
  g.y = fq_const_u32(2);
  return g;
}

__device__ __forceinline__ bool on_curve(const Affine& p) {
  Fq rhs = fe_add(fe_mul(fe_sqr(p.x), p.x), fq_const_u32(3));
  return fe_eq(fe_sqr(p.y), rhs);
}

// ---- point conversion -------------------------------------------------------

__global__ void k_points_in(const uint4* raw, size_t n, Affine* dst, uint32_t* flags) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint4 q0 = raw[4 * i], q1 = raw[4 * i + 1], q2 = raw[4 * i + 2], q3 = raw[4 * i + 3];
  uint32_t w[16] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w,
                    q2.x, q2.y, q2.z, q2.w, q3.x, q3.y, q3.z, q3.w};
  uint32_t any = 0;
#pragma unroll
  for (int k = 0; k < 16; ++k) any |= w[k];
  Affine a;
  if (any == 0) {
    a.x = fe_zero<FqConsts>();
    a.y = fe_zero<FqConsts>();
  } else {
    if (!fe_lt_mod<FqConsts>(w) || !fe_lt_mod<FqConsts>(w + 8)) raise_flag(flags, DEV_NONCANONICAL);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      a.x.v[k] = w[k];
      a.y.v[k] = w[8 + k];
    }
    a.x = fe_to_mont(a.x);
    a.y = fe_to_mont(a.y);
    if (!on_curve(a)) raise_flag(flags, DEV_OFF_CURVE);
  }
  st_fe(&dst[i].x, a.x);
  st_fe(&dst[i].y, a.y);
}

__global__ void k_points_out(const Affine* src, size_t n, uint4* raw) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  Affine a = ld_affine(&src[i]);
  Fq x = fe_from_mont(a.x), y = fe_from_mont(a.y);
  raw[4 * i] = make_uint4(x.v[0], x.v[1], x.v[2], x.v[3]);
  raw[4 * i + 1] = make_uint4(x.v[4], x.v[5], x.v[6], x.v[7]);
  raw[4 * i + 2] = make_uint4(y.v[0], y.v[1], y.v[2], y.v[3]);
  raw[4 * i + 3] = make_uint4(y.v[4], y.v[5], y.v[6], y.v[7]);
}

}  // namespace

// Canonical Fr -> Montgomery in place, flagging values >= p.
__global__ void k_fr_to_mont(Fr* v, size_t n, uint32_t* flags) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  Fr a = ld_fe(&v[i]);
  if (!fe_lt_mod<FrConsts>(a.v)) atomicOr(flags, (uint32_t)DEV_NONCANONICAL);
  st_fe(&v[i], fe_to_mont(a));
}

namespace {

// [tau^i] G by double-and-add over the canonical bits of tau^i.
__global__ void k_srs_powers(Fr tau, size_t n, Affine* dst, uint32_t* flags) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  Fr s = fe_one<FrConsts>(), base = tau;
  for (size_t e = i; e; e >>= 1) {
    if (e & 1) s = fe_mul(s, base);
    base = fe_sqr(base);
  }
  Fr sc = fe_from_mont(s);
  const Affine g = generator_affine();
  Xyzz acc = xyzz_inf();
  for (int bit = 253; bit >= 0; --bit) {
    acc = xyzz_dbl(acc);
    if ((sc.v[bit >> 5] >> (bit & 31)) & 1) acc = xyzz_add_affine(acc, g);
  }
  Affine a = xyzz_to_affine(acc, flags);
  st_fe(&dst[i].x, a.x);
  st_fe(&dst[i].y, a.y);
}

// tab[w*n + i] = 2^(c*w) * base[i].
__global__ void k_window_table(const Affine* base, size_t n, int c, int windows, Affine* tab, uint32_t* flags) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  Affine cur = ld_affine(&base[i]);
  st_fe(&tab[i].x, cur.x);
  st_fe(&tab[i].y, cur.y);
  for (int w = 1; w < windows; ++w) {
    if (!aff_is_inf(cur)) {
      Xyzz acc = xyzz_from_affine(cur);
      for (int j = 0; j < c; ++j) acc = xyzz_dbl(acc);
      cur = xyzz_to_affine(acc, flags);
    }
    st_fe(&tab[(size_t)w * n + i].x, cur.x);
    st_fe(&tab[(size_t)w * n + i].y, cur.y);
  }
}

// ---- recode + histogram -------------------------------------------------------

// Entry layout: bits 63..32 bucket (space*K + |d|-1), bit 31 negate, bits 30..0
// base index. A zero digit writes kSkip and is not counted.
constexpr uint64_t kSkip = ~0ull;

template <bool SMALL>
__global__ void k_recode(const void* scalars, size_t n, int c, int windows, int precomp, size_t tab_n,
                         int canonical_in, uint64_t* entries, uint32_t* counts, uint32_t* flags) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t limbs[8];
  if (SMALL) {
    limbs[0] = reinterpret_cast<const uint32_t*>(scalars)[i];
#pragma unroll
    for (int k = 1; k < 8; ++k) limbs[k] = 0;
  } else {
    Fr s = ld_fe(reinterpret_cast<const Fr*>(scalars) + i);
    if (!fe_lt_mod<FrConsts>(s.v)) raise_flag(flags, DEV_NONCANONICAL);
    if (!canonical_in) s = fe_from_mont(s);
#pragma unroll
    for (int k = 0; k < 8; ++k) limbs[k] = s.v[k];
  }
  const uint32_t K = 1u << (c - 1);
  const uint32_t mask = (1u << c) - 1;
  uint32_t carry = 0;
  for (int w = 0; w < windows; ++w) {
    int off = w * c;
    uint32_t raw = 0;
    if (off < 256) {
      int limb = off >> 5, sh = off & 31;
      uint64_t v = limbs[limb] >> sh;
      if (limb + 1 < 8) v |= (uint64_t)limbs[limb + 1] << (32 - sh);
      raw = (uint32_t)v & mask;
    }
    uint32_t coef = raw + carry;
    uint32_t mag;
    uint32_t neg = 0;
    if (w == windows - 1 || coef < K) {
      mag = coef;
      carry = 0;
    } else {
      mag = (1u << c) - coef;  // digit coef - 2^c < 0
      neg = 1;
      carry = 1;
    }
    uint64_t e = kSkip;
    if (mag) {
      uint32_t space = precomp ? 0u : (uint32_t)w;
      uint32_t bucket = space * K + (mag - 1);
      uint64_t pidx = precomp ? (uint64_t)w * tab_n + i : i;
      e = ((uint64_t)bucket << 32) | ((uint64_t)neg << 31) | pidx;
      atomicAdd(&counts[bucket], 1u);
    }
    entries[(size_t)w * n + i] = e;
  }
}

// ---- exclusive scan (u32), three passes ------------------------------------

constexpr int kScanBlock = 1024;
constexpr int kScanItems = 4;  // per thread

__global__ void k_scan_local(uint32_t* data, size_t n, uint32_t* block_sums) {
  __shared__ uint32_t sh[kScanBlock];
  size_t base = (size_t)blockIdx.x * kScanBlock * kScanItems + (size_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < n) ? data[base + k] : 0;
    sum += v[k];
  }
  sh[threadIdx.x] = sum;
  __syncthreads();
  for (int off = 1; off < kScanBlock; off <<= 1) {
    uint32_t t = threadIdx.x >= (unsigned)off ? sh[threadIdx.x - off] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  uint32_t run = sh[threadIdx.x] - sum;  // exclusive prefix of this thread
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) data[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == kScanBlock - 1) block_sums[blockIdx.x] = sh[threadIdx.x];
}

// Exclusive scan of up to kScanBlock block sums in one block; total at [nb].
__global__ void k_scan_blocks(uint32_t* block_sums, int nb) {
  __shared__ uint32_t sh[kScanBlock];
  uint32_t v = threadIdx.x < (unsigned)nb ? block_sums[threadIdx.x] : 0;
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int off = 1; off < kScanBlock; off <<= 1) {
    uint32_t t = threadIdx.x >= (unsigned)off ? sh[threadIdx.x - off] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  if (threadIdx.x < (unsigned)nb) block_sums[threadIdx.x] = sh[threadIdx.x] - v;
  if (threadIdx.x == kScanBlock - 1) block_sums[nb] = sh[threadIdx.x];
}

__global__ void k_scan_add(uint32_t* data, size_t n, const uint32_t* block_sums, uint32_t* total_out) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) data[i] += block_sums[i / (kScanBlock * kScanItems)];
  if (i == 0) *total_out = block_sums[(n + kScanBlock * kScanItems - 1) / (kScanBlock * kScanItems)];
}

__global__ void k_scatter(const uint64_t* entries, size_t e_count, uint32_t* cursor, uint64_t* sorted) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= e_count) return;
  uint64_t e = entries[i];
  if (e == kSkip) return;
  uint32_t pos = atomicAdd(&cursor[e >> 32], 1u);
  sorted[pos] = e;
}

// ---- accumulation -----------------------------------------------------------

__device__ __forceinline__ Affine load_base(const Affine* bases, uint64_t e) {
  Affine a = ld_affine(&bases[e & 0x7fffffffu]);
  if ((e >> 31) & 1) a.y = fe_neg(a.y);
  return a;
}

// Runs of equal buckets are folded by fixed-length segments; a run that
// touches a segment edge is only partial and leaves the segment as an item
// (key, point, present) in slot 2s (the run the segment started inside) or
// 2s+1 (the run it ends inside). Absent slots carry the neighbouring key and
// the identity, so the item list stays sorted and gap-free; the next level
// folds it the same way until one segment holds everything. A run that
// starts and ends inside a segment is a whole bucket and is written directly,
// so every bucket is written exactly once however skewed the digits are.
constexpr uint32_t kNoKey = 0xffffffffu;

__device__ __forceinline__ void put_item(uint32_t* keys, Xyzz* pts, uint8_t* present, size_t slot, uint32_t key,
                                         const Xyzz* p) {
  keys[slot] = key;
  present[slot] = p ? 1 : 0;
  if (p) st_xyzz(&pts[slot], *p);
}

__global__ void __launch_bounds__(128) k_accumulate(const uint64_t* sorted, const uint32_t* total, int seg_len,
                                                    size_t nseg, const Affine* bases, Xyzz* buckets,
                                                    uint32_t* okeys, Xyzz* opts, uint8_t* opres) {
  size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const size_t E = *total;
  const size_t lo = s * (size_t)seg_len;
  if (lo >= E) {
    put_item(okeys, opts, opres, 2 * s, kNoKey, nullptr);
    put_item(okeys, opts, opres, 2 * s + 1, kNoKey, nullptr);
    return;
  }
  const size_t hi = min(lo + (size_t)seg_len, E);
  const uint32_t first = (uint32_t)(sorted[lo] >> 32);
  uint32_t cur = first;
  const bool starts_before = lo > 0 && (uint32_t)(sorted[lo - 1] >> 32) == cur;
  const bool continues = hi < E && (uint32_t)(sorted[hi] >> 32) == (uint32_t)(sorted[hi - 1] >> 32);
  bool first_run = true, head_written = false;
  Xyzz acc = xyzz_inf();
  for (size_t i = lo; i < hi; ++i) {
    uint64_t e = sorted[i];
    uint32_t b = (uint32_t)(e >> 32);
    if (b != cur) {
      if (first_run && starts_before) {
        put_item(okeys, opts, opres, 2 * s, cur, &acc);
        head_written = true;
      } else {
        st_xyzz(&buckets[cur], acc);
      }
      first_run = false;
      cur = b;
      acc = xyzz_inf();
    }
    Affine p = load_base(bases, e);
    if (!aff_is_inf(p)) acc = xyzz_add_affine(acc, p);
  }
  if (first_run && starts_before) {
    put_item(okeys, opts, opres, 2 * s, cur, &acc);
    head_written = true;
    put_item(okeys, opts, opres, 2 * s + 1, cur, nullptr);
  } else {
    if (continues) put_item(okeys, opts, opres, 2 * s + 1, cur, &acc);
    else {
      st_xyzz(&buckets[cur], acc);
      put_item(okeys, opts, opres, 2 * s + 1, cur, nullptr);
    }
  }
  if (!head_written) put_item(okeys, opts, opres, 2 * s, first, nullptr);
}

// One level of the edge-run folding over items (see k_accumulate).
__global__ void __launch_bounds__(128) k_fold_edges(const uint32_t* keys, const Xyzz* pts, const uint8_t* pres,
                                                    size_t len, int seg_len, size_t nseg, Xyzz* buckets,
                                                    uint32_t* okeys, Xyzz* opts, uint8_t* opres) {
  size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const size_t lo = s * (size_t)seg_len;
  if (lo >= len) {
    put_item(okeys, opts, opres, 2 * s, kNoKey, nullptr);
    put_item(okeys, opts, opres, 2 * s + 1, kNoKey, nullptr);
    return;
  }
  const size_t hi = min(lo + (size_t)seg_len, len);
  const uint32_t first = keys[lo];
  uint32_t cur = first;
  const bool starts_before = lo > 0 && keys[lo - 1] == cur;
  const bool continues = hi < len && keys[hi] == keys[hi - 1];
  bool first_run = true, head_written = false, any = false;
  Xyzz acc = xyzz_inf();
  for (size_t i = lo; i < hi; ++i) {
    uint32_t b = keys[i];
    if (b != cur) {
      if (first_run && starts_before) {
        put_item(okeys, opts, opres, 2 * s, cur, any ? &acc : nullptr);
        head_written = true;
      } else if (any && cur != kNoKey) {
        st_xyzz(&buckets[cur], acc);
      }
      first_run = false;
      cur = b;
      acc = xyzz_inf();
      any = false;
    }
    if (pres[i]) {
      acc = any ? xyzz_add(acc, ld_xyzz(&pts[i])) : ld_xyzz(&pts[i]);
      any = true;
    }
  }
  if (first_run && starts_before) {
    put_item(okeys, opts, opres, 2 * s, cur, any ? &acc : nullptr);
    head_written = true;
    put_item(okeys, opts, opres, 2 * s + 1, cur, nullptr);
  } else {
    if (continues) put_item(okeys, opts, opres, 2 * s + 1, cur, any ? &acc : nullptr);
    else {
      if (any && cur != kNoKey) st_xyzz(&buckets[cur], acc);
      put_item(okeys, opts, opres, 2 * s + 1, cur, nullptr);
    }
  }
  if (!head_written) put_item(okeys, opts, opres, 2 * s, first, nullptr);
}

// ---- bucket reduction -------------------------------------------------------

// in[space*M + k] has weight k+1. Group g of `fan` buckets yields
// T_g = sum_j (j+1) in[g*fan + j] and R_g = sum_j in[g*fan + j]; the next
// level takes R_1..R_{G-1} (weights 1..G-1) and an identity pad at weight G:
//   sum_k k B_k = sum_g T_g + fan * sum_g g R_g.
__global__ void k_level(const Xyzz* in, int M, int spaces, int fan, Xyzz* outT, Xyzz* outR) {
  int G = (M + fan - 1) / fan;
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= spaces * G) return;
  int sp = idx / G, g = idx % G;
  int lo = g * fan, hi = min(lo + fan, M);
  Xyzz run = xyzz_inf(), tot = xyzz_inf();
  for (int k = hi - 1; k >= lo; --k) {
    run = xyzz_add(run, ld_xyzz(&in[(size_t)sp * M + k]));
    tot = xyzz_add(tot, run);
  }
  st_xyzz(&outT[(size_t)sp * G + g], tot);
  if (g > 0) st_xyzz(&outR[(size_t)sp * G + g - 1], run);
  else st_xyzz(&outR[(size_t)sp * G + G - 1], xyzz_inf());
}

// out[space] = sum of in[space*M .. space*M + M).
__global__ void k_sum(const Xyzz* in, int M, Xyzz* out) {
  __shared__ Xyzz sh[128];
  int sp = blockIdx.x;
  Xyzz acc = xyzz_inf();
  for (int k = threadIdx.x; k < M; k += blockDim.x) acc = xyzz_add(acc, ld_xyzz(&in[(size_t)sp * M + k]));
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if (threadIdx.x < (unsigned)off) sh[threadIdx.x] = xyzz_add(sh[threadIdx.x], sh[threadIdx.x + off]);
    __syncthreads();
  }
  if (threadIdx.x == 0) st_xyzz(&out[sp], sh[0]);
}

// First stage of a wide sum: block b of space sp folds in[sp*M + b*256 ..
// +256) into part[sp*gridDim.x + b], two points a thread then a tree.
__global__ void k_sum_blocks(const Xyzz* in, int M, Xyzz* part) {
  __shared__ Xyzz sh[128];
  const int sp = blockIdx.y, b = blockIdx.x;
  const int k0 = b * 256 + threadIdx.x, k1 = k0 + 128;
  Xyzz acc = k0 < M ? ld_xyzz(&in[(size_t)sp * M + k0]) : xyzz_inf();
  if (k1 < M) acc = xyzz_add(acc, ld_xyzz(&in[(size_t)sp * M + k1]));
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int off = 64; off > 0; off >>= 1) {
    if (threadIdx.x < (unsigned)off) sh[threadIdx.x] = xyzz_add(sh[threadIdx.x], sh[threadIdx.x + off]);
    __syncthreads();
  }
  if (threadIdx.x == 0) st_xyzz(&part[(size_t)sp * gridDim.x + b], sh[0]);
}

// tsum[level*spaces + sp] holds level sums; combine by Horner in `fan`, then
// combine spaces (windows) by Horner in 2^c, normalise and write 64 bytes.
__global__ void k_finish(const Xyzz* tsum, int levels, int spaces, int fan_log, int c, uint32_t* out64,
                         uint32_t* flags) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  Xyzz total = xyzz_inf();
  for (int sp = spaces - 1; sp >= 0; --sp) {
    for (int j = 0; j < c && sp != spaces - 1; ++j) total = xyzz_dbl(total);
    Xyzz s = xyzz_inf();
    for (int l = levels - 1; l >= 0; --l) {
      for (int j = 0; j < fan_log && l != levels - 1; ++j) s = xyzz_dbl(s);
      s = xyzz_add(s, ld_xyzz(&tsum[(size_t)l * spaces + sp]));
    }
    total = xyzz_add(total, s);
  }
  Affine a = xyzz_to_affine(total, flags);
  Fq x = fe_from_mont(a.x), y = fe_from_mont(a.y);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    out64[k] = x.v[k];
    out64[8 + k] = y.v[k];
  }
}

// ---- the grouped pipeline -----------------------------------------------------
//
// A group is up to kMaxCols scalar columns against one set of bases (an SRS
// window table or generic bases). Bucket keys are (col * spaces + space) * K +
// |d| - 1, with spaces = 1 over a window table and one space per window
// otherwise, so every column owns a key range and one counting sort, one
// accumulation and one bucket reduction serve the whole group: the
// latency-bound reduction is paid once per group instead of once per column.
// The sorted list holds 4-byte references (bit 31 negate, bits 30..0 base
// index); after the scatter the cursor array holds every bucket's end, which
// is all the accumulation needs to find its runs.

constexpr int kMaxCols = 32;

struct MsmCols {
  const void* s[kMaxCols];
  uint32_t len[kMaxCols];
  uint32_t off[kMaxCols];  // first base of the column (a stack's slot j starts at j * 2^n)
  int shared;              // 1: every column feeds one bucket set (one result, the sum)
  int bits;                // small scalars: 32, 16, 8 or 1 (bit-packed in u64 limbs)
};

// Scalar i of a small-scalar column of the given width.
__device__ __forceinline__ uint32_t small_scalar(const void* col, uint32_t i, int bits) {
  switch (bits) {
    case 1:
      return (uint32_t)((reinterpret_cast<const uint64_t*>(col)[i >> 6] >> (i & 63)) & 1u);
    case 8:
      return reinterpret_cast<const uint8_t*>(col)[i];
    case 16:
      return reinterpret_cast<const uint16_t*>(col)[i];
    default:
      return reinterpret_cast<const uint32_t*>(col)[i];
  }
}

// Digits of one scalar, counted (SCATTER = false) or placed (SCATTER = true).
// Lanes of a warp that hit the same bucket share one atomic: the leader adds
// the group's size and hands each peer its rank, so a bucket that a large
// share of the scalars hit (digit 1 from {0,1} columns and from the carries of
// 32-bit values) costs one atomic per warp, not one per scalar. Measured and
// not kept: aggregating only the lanes that share the first active lane's
// bucket, with plain atomics for the rest (13 % slower on mixed columns), and
// the window width compiled in with the window loop unrolled and every
// window's atomic issued before the first result is awaited (no change in
// either pass at 2^22).
template <bool SMALL, bool SCATTER>
__global__ void __launch_bounds__(256) k_digits(MsmCols cols, int c, int windows, int precomp, uint32_t tab_n,
                                                int canonical_in, uint32_t* cursor, uint32_t* sorted,
                                                uint32_t* flags) {
  const uint32_t col = blockIdx.y;
  const uint32_t n = cols.len[col];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31u;
  if (i - lane >= n) return;  // the whole warp lies past the column's end
  const bool live = i < n;
  uint32_t limbs[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) limbs[k] = 0;
  if (live) {
    if (SMALL) {
      limbs[0] = small_scalar(cols.s[col], i, cols.bits);
    } else {
      Fr s = ld_fe(reinterpret_cast<const Fr*>(cols.s[col]) + i);
      if (!SCATTER && !fe_lt_mod<FrConsts>(s.v)) raise_flag(flags, DEV_NONCANONICAL);
      if (!canonical_in) s = fe_from_mont(s);
#pragma unroll
      for (int k = 0; k < 8; ++k) limbs[k] = s.v[k];
    }
  }
  const uint32_t K = 1u << (c - 1);
  const uint32_t mask = (1u << c) - 1;
  const uint32_t spaces = precomp ? 1u : (uint32_t)windows;
  const uint32_t key0 = cols.shared ? 0u : col * spaces * K;
  const uint32_t base_i = cols.off[col] + i;
  uint32_t carry = 0;
  for (int w = 0; w < windows; ++w) {
    const int off = w * c;
    uint32_t raw = 0;
    if (off < 256) {
      const int limb = off >> 5, sh = off & 31;
      uint64_t v = limbs[limb] >> sh;
      if (limb + 1 < 8) v |= (uint64_t)limbs[limb + 1] << (32 - sh);
      raw = (uint32_t)v & mask;
    }
    const uint32_t coef = raw + carry;
    uint32_t mag, neg = 0;
    if (w == windows - 1 || coef < K) {
      mag = coef;
      carry = 0;
    } else {
      mag = (1u << c) - coef;  // digit coef - 2^c < 0
      neg = 1;
      carry = 1;
    }
    if (!live) mag = 0;
    if (mag > K) {  // unreachable for values below r; never index past the bucket range
      if (!SCATTER) raise_flag(flags, DEV_NONCANONICAL);
      mag = 0;
    }
    const unsigned active = __ballot_sync(0xffffffffu, mag != 0);
    if (mag) {
      const uint32_t key = key0 + (precomp ? 0u : (uint32_t)w * K) + mag - 1;
      const unsigned peers = __match_any_sync(active, key);
      const int leader = __ffs(peers) - 1;
      if (SCATTER) {
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(&cursor[key], (uint32_t)__popc(peers));
        base = __shfl_sync(peers, base, leader);
        const uint32_t idx = precomp ? (uint32_t)w * tab_n + base_i : base_i;
        sorted[base + (uint32_t)__popc(peers & ((1u << lane) - 1u))] = (neg << 31) | idx;
      } else if ((int)lane == leader) {
        atomicAdd(&cursor[key], (uint32_t)__popc(peers));
      }
    }
  }
}

// Persistent bucket accumulation: the grid is one wave of resident threads
// and thread s folds the s-th of nseg equal slices of the sorted list, so the
// work is balanced however the digits are distributed. Runs are found from
// the bucket ends; a run cut by a slice edge leaves as an item for
// k_fold_edges exactly as in k_accumulate.
// Four resident blocks per SM (128 registers a thread): measured 2-3 % faster
// than the three that the unconstrained allocation (144) leaves room for.
#ifndef APG_ACC_MIN_BLOCKS
#define APG_ACC_MIN_BLOCKS 4
#endif
// After affine pair rounds (`mode` non-null and *mode == 0) the input is the
// last round's explicit point list, position i holding point i, with its own
// bucket ends and total; otherwise references into `bases`.
__global__ void __launch_bounds__(128, APG_ACC_MIN_BLOCKS) k_bucket_acc(const uint32_t* sorted, const uint32_t* ends, uint32_t nbins,
                                                    const uint32_t* total, size_t nseg, const Affine* bases,
                                                    Xyzz* buckets, uint32_t* okeys, Xyzz* opts, uint8_t* opres,
                                                    const uint32_t* mode, const uint32_t* pair_ends,
                                                    const Affine* pair_pts) {
  const size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const bool direct = mode && *mode == 0;
  if (direct) {
    ends = pair_ends;
    total = pair_ends + nbins - 1;
    bases = pair_pts;
  }
  const size_t E = *total;
  const size_t seg = (E + nseg - 1) / nseg;
  const size_t lo = s * seg;
  if (lo >= E) {
    put_item(okeys, opts, opres, 2 * s, kNoKey, nullptr);
    put_item(okeys, opts, opres, 2 * s + 1, kNoKey, nullptr);
    return;
  }
  const size_t hi = min(lo + seg, E);
  // The bucket holding position lo: the first key whose end lies past it.
  uint32_t a = 0, b = nbins - 1;
  while (a < b) {
    const uint32_t m = (a + b) >> 1;
    if (ends[m] > lo) b = m;
    else a = m + 1;
  }
  uint32_t cur = a;
  size_t run_end = ends[cur];
  const bool starts_before = lo > (cur ? (size_t)ends[cur - 1] : 0);
  const uint32_t first = cur;
  bool first_run = true, head_written = false;
  Xyzz acc = xyzz_inf();
  for (size_t i = lo; i < hi; ++i) {
    if (i == run_end) {
      if (first_run && starts_before) {
        put_item(okeys, opts, opres, 2 * s, cur, &acc);
        head_written = true;
      } else {
        st_xyzz(&buckets[cur], acc);
      }
      first_run = false;
      do {
        run_end = ends[++cur];
      } while (run_end <= i);
      acc = xyzz_inf();
    }
    const uint32_t e = direct ? (uint32_t)i : sorted[i];
    Affine p = ld_affine(&bases[e & 0x7fffffffu]);
    if (!direct && (e >> 31)) p.y = fe_neg(p.y);
    if (!aff_is_inf(p)) acc = xyzz_add_affine(acc, p);
  }
  const bool continues = hi < run_end;
  if (first_run && starts_before) {
    put_item(okeys, opts, opres, 2 * s, cur, &acc);
    head_written = true;
    put_item(okeys, opts, opres, 2 * s + 1, cur, nullptr);
  } else {
    if (continues) {
      put_item(okeys, opts, opres, 2 * s + 1, cur, &acc);
    } else {
      st_xyzz(&buckets[cur], acc);
      put_item(okeys, opts, opres, 2 * s + 1, cur, nullptr);
    }
  }
  if (!head_written) put_item(okeys, opts, opres, 2 * s, first, nullptr);
}

// ---- affine pair rounds ------------------------------------------------------
//
// Before the XYZZ accumulation, a few rounds halve every bucket's run by adding
// its points in adjacent pairs in affine coordinates. All the pairs one thread
// owns share one field inversion (Montgomery's batch trick: the running product
// of the denominators going forward, one inversion, then each pair's inverse at
// two products going backward), so a pair sum costs 5M + 1S plus a share of one
// inversion, against 8M + 2S for each mixed XYZZ addition it replaces. Equal x
// (a doubling, or P + (-P)) and infinity are classified per pair, so no zero
// ever enters the product.
//
// Round r reads a list with bucket ends `ends_in` and writes the list of
// ceil(len/2) points per bucket at the exclusive-scan offsets `start_out`
// (nbins + 1 entries, the total last). Round 0 reads sorted references into
// the bases; later rounds read the previous round's points. A round 0 whose
// output would not fit the scratch sets *mode = 1 and every later step takes
// the references instead.

// Four rounds (a bucket's run cut to a sixteenth before the XYZZ tail):
// measured 1.2 % faster on the 2^22 commit than three; the fourth round's
// lists are short, but its pair sums still replace XYZZ additions.
#ifndef APG_PAIR_ROUNDS
#define APG_PAIR_ROUNDS 4
#endif
constexpr int kPairRounds = APG_PAIR_ROUNDS;
// Lists shorter than this per group are left to the XYZZ kernel alone (the
// extra launches would cost more than the products saved).
constexpr size_t kPairMinEntries = (size_t)1 << 21;
// Round 0's output list is held to this many points (64 bytes each).
constexpr size_t kPairMaxPoints = (size_t)48 << 20;

__global__ void k_halve_counts(const uint32_t* ends_in, uint32_t nbins, uint32_t* cnt) {
  const size_t b = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (b > nbins) return;
  if (b == nbins) {
    cnt[b] = 0;
    return;
  }
  const uint32_t len = ends_in[b] - (b ? ends_in[b - 1] : 0u);
  cnt[b] = (len + 1) / 2;
}

template <bool REFS>
__device__ __forceinline__ Affine pair_point(const uint32_t* refs, const Affine* src, uint32_t i) {
  if (REFS) {
    const uint32_t e = refs[i];
    Affine p = ld_affine(&src[e & 0x7fffffffu]);
    if (e >> 31) p.y = fe_neg(p.y);
    return p;
  }
  return ld_affine(&src[i]);
}

enum : int { kPairFirst = 0, kPairSecond = 1, kPairInf = 2, kPairAdd = 3, kPairDbl = 4 };

// The pair rounds' products are inlined (unlike the XYZZ formulas, whose ten
// inlined products a step overflowed the instruction cache): the compiler
// interleaves the independent ones, measured 2 % faster than calls.
// APG_PAIR_CALLS=1 makes them out-of-line calls instead (a build knob for
// measurement).
#ifndef APG_PAIR_CALLS
#define APG_PAIR_CALLS 0
#endif
__device__ __forceinline__ Fq pmul(const Fq& a, const Fq& b) { return APG_PAIR_CALLS ? cmul(a, b) : fe_mul(a, b); }
__device__ __forceinline__ Fq psqr(const Fq& a) { return APG_PAIR_CALLS ? csqr(a) : fe_sqr(a); }
__device__ __forceinline__ Fq2 pmul2(const Fq& a, const Fq& b, const Fq& c, const Fq& d) {
  if (APG_PAIR_CALLS) return cmul2(a, b, c, d);
  Fq2 r;
  r.a = fe_mul(a, b);
  r.b = fe_mul(c, d);
  return r;
}

// What the pair (p0, p1) sums to: p0 or p1 when the other is infinity, the
// point at infinity for P + (-P), else an addition or a doubling.
__device__ __forceinline__ int pair_kind(const Affine& p0, const Affine& p1) {
  if (aff_is_inf(p1)) return kPairFirst;
  if (aff_is_inf(p0)) return kPairSecond;
  if (!fe_eq(p0.x, p1.x)) return kPairAdd;
  return fe_eq(p0.y, p1.y) ? kPairDbl : kPairInf;
}

// The forward pass needs only the x coordinates (and y where x decides nothing).
template <bool REFS>
__device__ __forceinline__ bool pair_denominator(const uint32_t* refs, const Affine* src, uint32_t i0, Fq& d) {
  uint32_t j0 = i0, j1 = i0 + 1;
  bool n0 = false, n1 = false;
  if (REFS) {
    const uint32_t e0 = refs[i0], e1 = refs[i0 + 1];
    j0 = e0 & 0x7fffffffu;
    j1 = e1 & 0x7fffffffu;
    n0 = e0 >> 31;
    n1 = e1 >> 31;
  }
  const Fq x0 = ld_fe(&src[j0].x), x1 = ld_fe(&src[j1].x);
  if (!fe_eq(x0, x1)) {
    if (fe_is_zero(x0) && fe_is_zero(ld_fe(&src[j0].y))) return false;
    if (fe_is_zero(x1) && fe_is_zero(ld_fe(&src[j1].y))) return false;
    d = fe_sub(x1, x0);
    return true;
  }
  Fq y0 = ld_fe(&src[j0].y), y1 = ld_fe(&src[j1].y);
  if (n0) y0 = fe_neg(y0);
  if (n1) y1 = fe_neg(y1);
  if (fe_is_zero(x0) && (fe_is_zero(y0) || fe_is_zero(y1))) return false;  // an infinity
  if (!fe_eq(y0, y1)) return false;                                        // P + (-P)
  d = fe_add(y0, y0);
  return true;
}

// Field element shuffles across a full warp.
__device__ __forceinline__ Fq shfl_up_fq(const Fq& a, int off) {
  Fq r;
#pragma unroll
  for (int w = 0; w < 8; ++w) r.v[w] = __shfl_up_sync(0xffffffffu, a.v[w], off);
  return r;
}
__device__ __forceinline__ Fq shfl_down_fq(const Fq& a, int off) {
  Fq r;
#pragma unroll
  for (int w = 0; w < 8; ++w) r.v[w] = __shfl_down_sync(0xffffffffu, a.v[w], off);
  return r;
}
__device__ __forceinline__ Fq shfl_fq(const Fq& a, int lane) {
  Fq r;
#pragma unroll
  for (int w = 0; w < 8; ++w) r.v[w] = __shfl_sync(0xffffffffu, a.v[w], lane);
  return r;
}

// Each thread's 1/v (v != 0) from one inversion a block of kPairThreads:
// per warp the inclusive prefix and suffix products across the lanes give
// the warp's total and each lane's product of the others; warp 0 inverts the
// product of the warps' totals (the binary Euclid costs as many instructions
// as a lane's work in a late pair round, so one a block instead of one a warp
// is a quarter of that) and hands each warp the inverse of its total; then
// 1/v_i = (1/total_w) * (lanes before i) * (lanes after i). All threads of the
// block must call it.
constexpr int kPairThreads = 128;
constexpr int kPairWarps = kPairThreads / 32;

__device__ __forceinline__ Fq block_inverse(const Fq& v, uint32_t* flags) {
  __shared__ Fq tot[kPairWarps], tinv[kPairWarps];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  Fq pre = v, suf = v;
#pragma unroll 1
  for (int off = 1; off < 32; off <<= 1) {
    const Fq a = shfl_up_fq(pre, off), b = shfl_down_fq(suf, off);
    const Fq2 q = cmul2(pre, a, suf, b);
    if (lane >= off) pre = q.a;
    if (lane + off < 32) suf = q.b;
  }
  if (lane == 31) tot[w] = pre;
  Fq ex = shfl_up_fq(pre, 1), sx = shfl_down_fq(suf, 1);
  if (lane == 0) ex = fe_one<FqConsts>();
  if (lane == 31) sx = fe_one<FqConsts>();
  const Fq others = cmul(ex, sx);
  __syncthreads();
  if (w == 0) {
    Fq all = tot[0];
#pragma unroll 1
    for (int i = 1; i < kPairWarps; ++i) all = cmul(all, tot[i]);
    Fq o = fe_inverse(all, flags);  // every lane of warp 0 inverts the same value
#pragma unroll 1
    for (int i = 0; i < kPairWarps; ++i)
      if (i != lane) o = cmul(o, tot[i]);
    if (lane < kPairWarps) tinv[lane] = o;
  }
  __syncthreads();
  return cmul(tinv[w], others);
}

// The first bucket whose output reaches past slot o (o below the total).
__device__ __forceinline__ uint32_t pair_bucket(const uint32_t* start_out, uint32_t nbins, size_t o) {
  uint32_t a = 0, b = nbins - 1;
  while (a < b) {
    const uint32_t mid = (a + b) >> 1;
    if (start_out[mid + 1] > o) b = mid;
    else a = mid + 1;
  }
  return a;
}

// The bucket holding output slot o, from the bucket b of an earlier (seek_up)
// or later (seek_down) slot of the same lane. A lane's slots are 32 apart, so
// where most buckets are empty (a short column grouped with a long one) the
// cursor may pass many buckets in one step: it gallops (1, 2, 4, ... buckets)
// and then bisects, one comparison where buckets are dense.
__device__ __forceinline__ uint32_t pair_seek_up(const uint32_t* start_out, uint32_t nbins, uint32_t b, size_t o) {
  if (start_out[b + 1] > o) return b;
  uint32_t lo = b + 1, hi, step = 1;  // start_out[lo] <= o: the bucket is at or past lo
  for (;;) {
    hi = lo + step;
    if (hi >= nbins - 1 || start_out[hi + 1] > o) break;
    lo = hi + 1;
    step <<= 1;
  }
  hi = min(hi, nbins - 1);
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (start_out[mid + 1] > o) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

__device__ __forceinline__ uint32_t pair_seek_down(const uint32_t* start_out, uint32_t b, size_t o) {
  if (start_out[b] <= o) return b;
  uint32_t hi = b - 1, lo, step = 1;  // the bucket is at or before hi
  for (;;) {
    if (hi < step) {
      lo = 0;
      break;
    }
    lo = hi - step;
    if (start_out[lo] <= o) break;
    hi = lo - 1;
    step <<= 1;
  }
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (start_out[mid] <= o) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Slot o of bucket b reads input i0 and, when `two`, i0 + 1.
__device__ __forceinline__ uint32_t pair_input(const uint32_t* ends_in, const uint32_t* start_out, uint32_t b,
                                               size_t o, bool& two) {
  const uint32_t i0 = (b ? ends_in[b - 1] : 0u) + 2u * (uint32_t)(o - start_out[b]);
  two = i0 + 1 < ends_in[b];
  return i0;
}

// One output slot of the backward pass: what it needs of its inputs (x0, y0,
// x1), its kind, and the denominator and numerator of the slope when it has
// one (1 and 0 otherwise, which leave the running inverse unchanged).
struct PairSlot {
  Fq x0, y0, x1, d, num;
  uint32_t i0;
  int kind;
};

template <bool REFS>
__device__ __forceinline__ void pair_load(const uint32_t* refs, const Affine* src, uint32_t i0, bool two,
                                          PairSlot& t) {
  const Affine p0 = pair_point<REFS>(refs, src, i0);
  Affine p1 = p0;
  t.i0 = i0;
  t.kind = kPairFirst;
  if (two) {
    p1 = pair_point<REFS>(refs, src, i0 + 1);
    t.kind = pair_kind(p0, p1);
  }
  t.x0 = p0.x;
  t.y0 = p0.y;
  t.x1 = p1.x;
  t.d = fe_one<FqConsts>();
  t.num = fe_zero<FqConsts>();
  if (t.kind == kPairAdd) {
    t.d = fe_sub(p1.x, p0.x);
    t.num = fe_sub(p1.y, p0.y);
  } else if (t.kind == kPairDbl) {
    t.d = fe_add(p0.y, p0.y);
    const Fq q = psqr(p0.x);
    t.num = fe_add(q, fe_add(q, q));
  }
}

// The slot's sum, given the slope lam when it has one.
template <bool REFS>
__device__ __forceinline__ void pair_store(const uint32_t* refs, const Affine* src, const PairSlot& t,
                                           const Fq& lam, const Fq& l2, Affine* dst) {
  Fq x = t.x0, y = t.y0;
  if (t.kind == kPairSecond) {
    const Affine p1 = pair_point<REFS>(refs, src, t.i0 + 1);
    x = p1.x;
    y = p1.y;
  } else if (t.kind == kPairInf) {
    x = fe_zero<FqConsts>();
    y = fe_zero<FqConsts>();
  } else if (t.kind != kPairFirst) {
    x = fe_sub(fe_sub(l2, t.x0), t.x1);
    y = fe_sub(pmul(lam, fe_sub(t.x0, x)), t.y0);
  }
  st_fe(&dst->x, x);
  st_fe(&dst->y, y);
}

// Resident blocks a SM for the backward half of a round (it holds a slot's two
// points, its running inverse and the slope): six blocks cap it at 80
// registers with a few bytes spilled, measured 1 % faster on the headline
// step than five at 92 registers; seven (72 registers) spilled more and was
// slower.
#ifndef APG_PAIR_MIN_BLOCKS
#define APG_PAIR_MIN_BLOCKS 6
#endif
// The slots of a pair round. A warp owns 32 * m consecutive output slots and
// lane l takes slots base + 32 j + l, so the lanes' references, explicit input
// points, running products and outputs move in coalesced rows. Both halves of
// a round derive the same assignment from (E, T).
struct PairLane {
  size_t o0, steps;
};

__device__ __forceinline__ PairLane pair_lane(size_t s, size_t E, size_t T) {
  PairLane l;
  const size_t m = (E + T - 1) / T;
  l.o0 = (s / 32) * 32 * m + (s & 31);
  l.steps = l.o0 < E ? min(m, (E - l.o0 + 31) / 32) : 0;
  return l;
}

// Forward half: lane s multiplies up the slope denominators of its slots,
// leaving the running product before slot j in pp[j * T + s] and the lane's
// total in tot[s]. No barrier: the lanes of a block finish independently.
// A round 0 whose output would not fit the scratch (E > cap) sets *mode = 1,
// and every later step takes the references instead.
// Slot inputs handed from the forward to the backward half (`idx`, one word a
// slot in the same j * T + s layout as the running products): the first
// input's position, and bit 31 when the slot has a second input. With it the
// backward half neither searches the bucket offsets nor waits on them, and
// issues a slot's reference loads one slot ahead and its word loads two
// ahead (k_pair_bwd_pf). APG_PAIR_PF=0 keeps the searching k_pair_bwd (a
// build knob for measurement). Measured on a GB300 (uniform 2^22
// accumulation / mixed 16 x 2^22 commit): searching 11.86 / 56.6 ms; words
// and references ahead 11.36 / 54.8 ms at five blocks an SM (11.23 / 56.1 at
// four); also the points and running product one slot ahead (128 registers,
// three or four blocks) 11.8-12.0 / 56.7-59.0; the x coordinates one slot
// ahead with the slope's inverse started on x alone 11.35 / 56.0 at four
// blocks, 12.1 / 57.7 at five.
#ifndef APG_PAIR_PF
#define APG_PAIR_PF 1
#endif
constexpr uint32_t kPairTwo = 0x80000000u;
// APG_PAIR_FWD_AHEAD: the forward half also loads the next slot's word and
// references while the current slot's x coordinates are in flight.
#ifndef APG_PAIR_FWD_AHEAD
#define APG_PAIR_FWD_AHEAD 1
#endif

// A slot word's references: table references in round 0, list positions
// after it (a one-input slot repeats its first).
template <bool REFS>
__device__ __forceinline__ void pair_refs(const uint32_t* refs, uint32_t w, uint32_t& e0, uint32_t& e1) {
  const uint32_t i0 = w & ~kPairTwo;
  const bool two = (w & kPairTwo) != 0;
  if (REFS) {
    e0 = refs[i0];
    e1 = two ? refs[i0 + 1] : e0;
  } else {
    e0 = i0;
    e1 = two ? i0 + 1 : i0;
  }
}

// pair_denominator with the two x coordinates already loaded.
template <bool REFS>
__device__ __forceinline__ bool pair_denominator_x(const Affine* src, uint32_t e0, uint32_t e1, const Fq& x0,
                                                   const Fq& x1, Fq& d) {
  const uint32_t j0 = REFS ? (e0 & 0x7fffffffu) : e0, j1 = REFS ? (e1 & 0x7fffffffu) : e1;
  if (!fe_eq(x0, x1)) {
    if (fe_is_zero(x0) && fe_is_zero(ld_fe(&src[j0].y))) return false;
    if (fe_is_zero(x1) && fe_is_zero(ld_fe(&src[j1].y))) return false;
    d = fe_sub(x1, x0);
    return true;
  }
  Fq y0 = ld_fe(&src[j0].y), y1 = ld_fe(&src[j1].y);
  if (REFS && (e0 >> 31)) y0 = fe_neg(y0);
  if (REFS && (e1 >> 31)) y1 = fe_neg(y1);
  if (fe_is_zero(x0) && (fe_is_zero(y0) || fe_is_zero(y1))) return false;  // an infinity
  if (!fe_eq(y0, y1)) return false;                                        // P + (-P)
  d = fe_add(y0, y0);
  return true;
}

template <bool REFS>
__global__ void __launch_bounds__(kPairThreads)
    k_pair_fwd(const uint32_t* refs, const Affine* src, const uint32_t* ends_in, const uint32_t* start_out,
               uint32_t nbins, size_t cap, uint32_t* mode, size_t T, Fq* pp, Fq* tot, uint32_t* idx) {
  const size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (s >= T || *mode) return;
  const size_t E = start_out[nbins];
  if (E > cap) {
    if (s == 0) *mode = 1;
    return;
  }
  const PairLane L = pair_lane(s, E, T);
  uint32_t b = L.steps ? pair_bucket(start_out, nbins, L.o0) : 0u;
  Fq acc = fe_one<FqConsts>();
  if (APG_PAIR_PF && APG_PAIR_FWD_AHEAD) {
    // The next slot's bucket search, word and references are issued while
    // this slot's x coordinates are in flight.
    uint32_t wa = 0, ea0 = 0, ea1 = 0;
    if (L.steps) {
      bool two;
      wa = pair_input(ends_in, start_out, b, L.o0, two);
      wa |= two ? kPairTwo : 0u;
      pair_refs<REFS>(refs, wa, ea0, ea1);
    }
    for (size_t j = 0; j < L.steps; ++j) {
      const Fq x0 = ld_fe(&src[REFS ? (ea0 & 0x7fffffffu) : ea0].x);
      const Fq x1 = ld_fe(&src[REFS ? (ea1 & 0x7fffffffu) : ea1].x);
      uint32_t wb = 0, eb0 = 0, eb1 = 0;
      if (j + 1 < L.steps) {
        const size_t o = L.o0 + 32 * (j + 1);
        b = pair_seek_up(start_out, nbins, b, o);
        bool two;
        wb = pair_input(ends_in, start_out, b, o, two);
        wb |= two ? kPairTwo : 0u;
        pair_refs<REFS>(refs, wb, eb0, eb1);
      }
      idx[j * T + s] = wa;
      Fq d;
      if ((wa & kPairTwo) && pair_denominator_x<REFS>(src, ea0, ea1, x0, x1, d)) {
        st_fe(&pp[j * T + s], acc);
        acc = fe_mul(acc, d);
      }
      wa = wb;
      ea0 = eb0;
      ea1 = eb1;
    }
    st_fe(&tot[s], acc);
    return;
  }
  for (size_t j = 0; j < L.steps; ++j) {
    const size_t o = L.o0 + 32 * j;
    b = pair_seek_up(start_out, nbins, b, o);
    bool two;
    const uint32_t i0 = pair_input(ends_in, start_out, b, o, two);
    if (APG_PAIR_PF) idx[j * T + s] = i0 | (two ? kPairTwo : 0u);
    Fq d;
    if (!two || !pair_denominator<REFS>(refs, src, i0, d)) continue;
    st_fe(&pp[j * T + s], acc);
    acc = fe_mul(acc, d);
  }
  st_fe(&tot[s], acc);
}

// Backward half: the block shares one inversion of its lanes' totals (every
// lane reaches it first, before any slot), then each slot takes its inverse
// at two products from the running inverse and writes its sum.
template <bool REFS>
__global__ void __launch_bounds__(kPairThreads, APG_PAIR_MIN_BLOCKS)
    k_pair_bwd(const uint32_t* refs, const Affine* src, const uint32_t* ends_in, const uint32_t* start_out,
               uint32_t nbins, const uint32_t* mode, size_t T, const Fq* pp, const Fq* tot, Affine* out,
               uint32_t* flags) {
  const size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (*mode) return;  // uniform across the grid: set before this launch
  const size_t E = start_out[nbins];
  const PairLane L = pair_lane(s, E, T);
  Fq inv = block_inverse(s < T ? ld_fe(&tot[s]) : fe_one<FqConsts>(), flags);  // every thread of the block
  if (s >= T || !L.steps) return;
  uint32_t b = pair_bucket(start_out, nbins, L.o0 + 32 * (L.steps - 1));
  for (size_t j = L.steps; j-- > 0;) {
    const size_t o = L.o0 + 32 * j;
    b = pair_seek_down(start_out, b, o);
    bool two;
    PairSlot t;
    pair_load<REFS>(refs, src, pair_input(ends_in, start_out, b, o, two), two, t);
    if (t.kind < kPairAdd) {
      pair_store<REFS>(refs, src, t, t.num, t.num, &out[o]);
      continue;
    }
    const Fq2 di = pmul2(inv, ld_fe(&pp[j * T + s]), inv, t.d);  // 1/d, and the running inverse one back
    inv = di.b;
    const Fq lam = pmul(t.num, di.a);
    pair_store<REFS>(refs, src, t, lam, psqr(lam), &out[o]);
  }
}

// The backward half over the forward half's slot words (see `idx` above). A
// slot's chain of dependent loads (its word, then its references, then its
// points) is spread over consecutive iterations: the word and the
// references are loaded while the two slots before it are summed, so only
// the point gather itself waits at the slot's start.
template <bool REFS>
__device__ __forceinline__ Affine pair_fetch(const Affine* src, uint32_t e) {
  return ld_affine(&src[REFS ? (e & 0x7fffffffu) : e]);
}

template <bool REFS>
__device__ __forceinline__ void pair_sign(Affine& p, uint32_t e) {
  if (REFS && (e >> 31)) p.y = fe_neg(p.y);
}

// One slot from its loaded inputs: the same kinds, running inverse and sum
// as pair_load/pair_store.
__device__ __forceinline__ void pair_finish(const Affine& p0, const Affine& p1, bool two, const Fq& ppj, Fq& inv,
                                            Affine* dst) {
  const int kind = two ? pair_kind(p0, p1) : (int)kPairFirst;
  if (kind < kPairAdd) {
    Fq x = p0.x, y = p0.y;
    if (kind == kPairSecond) {
      x = p1.x;
      y = p1.y;
    } else if (kind == kPairInf) {
      x = fe_zero<FqConsts>();
      y = fe_zero<FqConsts>();
    }
    st_fe(&dst->x, x);
    st_fe(&dst->y, y);
    return;
  }
  Fq d, num;
  if (kind == kPairAdd) {
    d = fe_sub(p1.x, p0.x);
    num = fe_sub(p1.y, p0.y);
  } else {
    d = fe_add(p0.y, p0.y);
    const Fq q = psqr(p0.x);
    num = fe_add(q, fe_add(q, q));
  }
  const Fq2 di = pmul2(inv, ppj, inv, d);  // 1/d, and the running inverse one back
  inv = di.b;
  const Fq lam = pmul(num, di.a);
  const Fq x = fe_sub(fe_sub(psqr(lam), p0.x), p1.x);
  st_fe(&dst->x, x);
  st_fe(&dst->y, fe_sub(pmul(lam, fe_sub(p0.x, x)), p0.y));
}

#ifndef APG_PAIR_PF_MIN_BLOCKS
#define APG_PAIR_PF_MIN_BLOCKS 5
#endif

template <bool REFS>
__global__ void __launch_bounds__(kPairThreads, APG_PAIR_PF_MIN_BLOCKS)
    k_pair_bwd_pf(const uint32_t* refs, const Affine* src, const uint32_t* idx, const uint32_t* start_out,
                  uint32_t nbins, const uint32_t* mode, size_t T, const Fq* pp, const Fq* tot, Affine* out,
                  uint32_t* flags) {
  const size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (*mode) return;  // uniform across the grid: set before this launch
  const size_t E = start_out[nbins];
  const PairLane L = pair_lane(s, E, T);
  Fq inv = block_inverse(s < T ? ld_fe(&tot[s]) : fe_one<FqConsts>(), flags);  // every thread of the block
  if (s >= T || !L.steps) return;
  // Entering the loop for slot j: slot j's word and references, slot j - 1's
  // word. Each pass issues slot j's point and running-product loads, slot
  // j - 1's reference loads and slot j - 2's word load together, then sums
  // slot j.
  size_t j = L.steps - 1;
  uint32_t wa = idx[j * T + s], ea0, ea1;
  pair_refs<REFS>(refs, wa, ea0, ea1);
  uint32_t wb = j >= 1 ? idx[(j - 1) * T + s] : 0u;
  for (;;) {
    Affine p0 = pair_fetch<REFS>(src, ea0), p1 = pair_fetch<REFS>(src, ea1);
    const Fq ppj = ld_fe(&pp[j * T + s]);
    uint32_t nb0 = 0, nb1 = 0, nw = 0;
    if (j >= 1) pair_refs<REFS>(refs, wb, nb0, nb1);
    if (j >= 2) nw = idx[(j - 2) * T + s];
    pair_sign<REFS>(p0, ea0);
    pair_sign<REFS>(p1, ea1);
    pair_finish(p0, p1, (wa & kPairTwo) != 0, ppj, inv, &out[L.o0 + 32 * j]);
    if (j == 0) break;
    --j;
    wa = wb;
    ea0 = nb0;
    ea1 = nb1;
    wb = nw;
  }
}

// Bucket reduction of a small bucket set (K <= kSmallK), one block per space:
// thread t holds B_t (weight t + 1); a suffix scan turns it into
// S_t = sum_{k >= t} B_k, and sum_k (k + 1) B_k = sum_t S_t is a tree sum, so
// the dependent chain is 2 log2 K additions instead of the running-sum levels.
constexpr int kSmallK = 256;

__global__ void __launch_bounds__(kSmallK) k_reduce_small(const Xyzz* buckets, int K, Xyzz* out) {
  __shared__ Xyzz shx[kSmallK];
  const int sp = blockIdx.x, t = threadIdx.x;
  Xyzz v = ld_xyzz(&buckets[(size_t)sp * K + t]);
  shx[t] = v;
  __syncthreads();
  for (int off = 1; off < K; off <<= 1) {
    const bool has = t + off < K;
    Xyzz nb = has ? shx[t + off] : xyzz_inf();
    __syncthreads();
    if (has) v = xyzz_add(v, nb);
    shx[t] = v;
    __syncthreads();
  }
  for (int off = K / 2; off > 0; off >>= 1) {
    if (t < off) shx[t] = xyzz_add(shx[t], shx[t + off]);
    __syncthreads();
  }
  if (t == 0) st_xyzz(&out[sp], shx[0]);
}

// One thread per column: Horner over the reduction levels (in `fan`) and the
// column's spaces (windows, in 2^c), then the canonical affine bytes.
__global__ void k_finish_cols(const Xyzz* tsum, int levels, int spaces_total, int spaces_per_col, int ncols,
                              int fan_log, int c, uint32_t* out64, uint32_t* flags) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncols) return;
  Xyzz total = xyzz_inf();
  for (int w = spaces_per_col - 1; w >= 0; --w) {
    if (w != spaces_per_col - 1)
      for (int j = 0; j < c; ++j) total = xyzz_dbl(total);
    const int sp = col * spaces_per_col + w;
    Xyzz s = xyzz_inf();
    for (int l = levels - 1; l >= 0; --l) {
      if (l != levels - 1)
        for (int j = 0; j < fan_log; ++j) s = xyzz_dbl(s);
      s = xyzz_add(s, ld_xyzz(&tsum[(size_t)l * spaces_total + sp]));
    }
    total = xyzz_add(total, s);
  }
  const Affine a = xyzz_to_affine(total, flags);
  const Fq x = fe_from_mont(a.x), y = fe_from_mont(a.y);
  uint32_t* o = out64 + 16 * (size_t)col;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    o[k] = x.v[k];
    o[8 + k] = y.v[k];
  }
}

// out64 = the sum of m canonical affine points in64[0..m) (a stack whose
// columns took more than one group).
__global__ void k_add_points(const uint32_t* in64, int m, uint32_t* out64, uint32_t* flags) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  Xyzz acc = xyzz_inf();
  for (int j = 0; j < m; ++j) {
    Affine a;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      a.x.v[k] = in64[16 * j + k];
      a.y.v[k] = in64[16 * j + 8 + k];
    }
    if (aff_is_inf(a)) continue;
    a.x = fe_to_mont(a.x);
    a.y = fe_to_mont(a.y);
    acc = xyzz_add(acc, xyzz_from_affine(a));
  }
  const Affine r = xyzz_to_affine(acc, flags);
  const Fq x = fe_from_mont(r.x), y = fe_from_mont(r.y);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    out64[k] = x.v[k];
    out64[8 + k] = y.v[k];
  }
}

template <class T>
inline unsigned blocks_for(size_t n, int threads) {
  return (unsigned)((n + threads - 1) / threads);
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

void upload_points_async(Ctx& c, const uint8_t* host, size_t n, Affine* dst) {
  if (n == 0) return;
  uint4* raw = c.scratch[S_TMP7].as<uint4>(4 * n);
  APG_CUDA(cudaMemcpyAsync(raw, host, 64 * n, cudaMemcpyHostToDevice, c.stream));
  launch(c, k_points_in, blocks_for<int>(n, 256), 256, 0, (const uint4*)raw, n, dst, c.d_flags);
}

void upload_points(Ctx& c, const uint8_t* host, size_t n, Affine* dst) {
  upload_points_async(c, host, n, dst);
  if (n) c.check_flags();
}

void download_points(Ctx& c, const Affine* src, size_t n, uint8_t* host) {
  if (n == 0) return;
  uint4* raw = c.scratch[S_TMP7].as<uint4>(4 * n);
  launch(c, k_points_out, blocks_for<int>(n, 256), 256, 0, src, n, raw);
  APG_CUDA(cudaMemcpyAsync(host, raw, 64 * n, cudaMemcpyDeviceToHost, c.stream));
  APG_CUDA(cudaStreamSynchronize(c.stream));
}

void generate_srs(Ctx& c, const uint8_t tau_canonical[32], size_t n, Affine* dst) {
  Fr* d_tau = c.scratch[S_TMP6].as<Fr>(1);
  APG_CUDA(cudaMemcpyAsync(d_tau, tau_canonical, 32, cudaMemcpyHostToDevice, c.stream));
  launch(c, k_fr_to_mont, 1, 1, 0, d_tau, (size_t)1, c.d_flags);
  c.check_flags();
  Fr tau_mont;
  APG_CUDA(cudaMemcpyAsync(&tau_mont, d_tau, 32, cudaMemcpyDeviceToHost, c.stream));
  APG_CUDA(cudaStreamSynchronize(c.stream));
  launch(c, k_srs_powers, blocks_for<int>(n, 128), 128, 0, tau_mont, n, dst, c.d_flags);
  APG_CUDA(cudaStreamSynchronize(c.stream));
}

static int default_window(size_t n, bool small) {
  int lg = 0;
  while (((size_t)1 << (lg + 1)) <= n) ++lg;
  int cb;
  if (lg <= 4) cb = 3;
  else if (lg <= 8) cb = 5;
  else if (lg <= 12) cb = 9;
  else if (lg <= 16) cb = 12;
  else if (lg <= 20) cb = 15;
  else cb = 16;
  if (small && cb > 11) cb = 11;  // 32-bit scalars: three windows
  return cb;
}

static int window_count(int bits, int cb) { return (bits + 1 + cb - 1) / cb; }

const SrsTable* srs_table(Ctx& c, int cbits, size_t need) {
  for (auto& t : c.tables)
    if (t.c == cbits && t.n >= need) return &t;
  if (!c.srs || c.srs_n < need) return nullptr;
  // The wide table covers the whole SRS, a narrow one a 2^16 prefix.
  size_t n = cbits >= 12 ? c.srs_n : std::min(c.srs_n, (size_t)1 << 16);
  if (n < need) n = c.srs_n;
  for (auto it = c.tables.begin(); it != c.tables.end(); ++it)
    if (it->c == cbits) {
      APG_CUDA(cudaStreamSynchronize(c.stream));
      if (it->owned) cudaFree(it->tab);
      c.tables.erase(it);
      break;
    }
  SrsTable t;
  t.c = cbits;
  t.windows = window_count(254, cbits);
  t.n = n;
  // Sorted references carry the table index in 31 bits.
  if ((size_t)t.windows * n >= ((size_t)1 << 31)) throw Error(APG_ERR_OUT_OF_MEMORY, "SRS window table too large");
  APG_CUDA(cudaMalloc(&t.tab, (size_t)t.windows * n * sizeof(Affine)));
  launch(c, k_window_table, blocks_for<int>(n, 128), 128, 0, (const Affine*)c.srs, n, cbits, t.windows, t.tab,
         c.d_flags);
  APG_CUDA(cudaStreamSynchronize(c.stream));
  c.tables.push_back(t);
  return &c.tables.back();
}

static int ceil_log2(size_t n) {
  int k = 0;
  while (((size_t)1 << k) < n) ++k;
  return k;
}

const SrsTable* srs_table_for(Ctx& c, size_t n, bool tuned) {
  const int cls = ceil_log2(n);
  if (tuned && cls < 64 && c.tuned_c[cls]) {
    const SrsTable* t = srs_table(c, c.tuned_c[cls], n);
    if (t) return t;
  }
  if (n <= ((size_t)1 << 14)) {
    const SrsTable* t = srs_table(c, 8, n);
    if (t) return t;
  }
  if (n >= kWideTableMin) {
    const SrsTable* t = srs_table(c, 20, n);
    if (t) return t;
  }
  return srs_table(c, 16, n);
}

void msm_autotune(Ctx& c, const void* d_sample, size_t sample_len, int kmin, int kmax, const int* cands,
                  size_t ncands, int* chosen) {
  cudaEvent_t e0, e1;
  APG_CUDA(cudaEventCreate(&e0));
  APG_CUDA(cudaEventCreate(&e1));
  uint8_t* d_out = c.scratch[S_TMP4].as<uint8_t>(64);
  for (int k = kmin; k <= kmax; ++k) {
    const size_t n = (size_t)1 << k;
    int best_c = 0;
    float best_ms = 0;
    if (k < 64 && n <= sample_len && n <= c.srs_n) {
      for (size_t j = 0; j < ncands; ++j) {
        const int cb = cands[j];
        if (cb < 2 || cb > 20) continue;
        if (cb < 12 && n > ((size_t)1 << 16)) continue;  // narrow tables cover a 2^16 prefix
        const SrsTable* t = srs_table(c, cb, n);
        if (!t) continue;
        msm_device(c, nullptr, t, d_sample, false, false, n, d_out, nullptr);  // warm-up
        APG_CUDA(cudaEventRecord(e0, c.stream));
        for (int r = 0; r < 2; ++r) msm_device(c, nullptr, t, d_sample, false, false, n, d_out, nullptr);
        APG_CUDA(cudaEventRecord(e1, c.stream));
        APG_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        APG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (!best_c || ms < best_ms) {
          best_c = cb;
          best_ms = ms;
        }
      }
      c.check_flags();
      c.tuned_c[k] = best_c;
    }
    if (chosen) chosen[k - kmin] = best_c;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
}

MsmPlan msm_plan(size_t n, bool small_scalars, const SrsTable* table) {
  MsmPlan p;
  if (table) {
    p.c = table->c;
    p.windows = small_scalars ? window_count(32, table->c) : table->windows;
    p.precomp = true;
  } else {
    p.c = default_window(n, small_scalars);
    p.windows = window_count(small_scalars ? 32 : 254, p.c);
    p.precomp = false;
  }
  return p;
}

namespace {

// Threads of k_bucket_acc resident on the whole device (one wave).
size_t acc_resident_threads(Ctx& c) {
  static std::once_flag once;
  static int per_sm = 0;
  std::call_once(once, [] {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bucket_acc, 128, 0) != cudaSuccess || per_sm < 1)
      per_sm = 1;
  });
  return (size_t)c.sm_count * (size_t)per_sm * 128;
}

size_t pair_resident_threads(Ctx& c) {
  static std::once_flag once;
  static int per_sm = 0;
  std::call_once(once, [] {
    int a = 0, b = 0;
    if (APG_PAIR_PF) {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_pair_bwd_pf<true>, kPairThreads, 0) != cudaSuccess)
        a = 1;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_pair_bwd_pf<false>, kPairThreads, 0) != cudaSuccess)
        b = 1;
    } else {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_pair_bwd<true>, kPairThreads, 0) != cudaSuccess) a = 1;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_pair_bwd<false>, kPairThreads, 0) != cudaSuccess)
        b = 1;
    }
    per_sm = std::max(1, std::min(a, b));
  });
  return (size_t)c.sm_count * (size_t)per_sm * kPairThreads;
}

constexpr size_t kMaxBins = (size_t)(kScanBlock - 1) * kScanBlock * kScanItems;  // one pass of the 3-kernel scan
constexpr size_t kMaxGroupEntries = (size_t)1 << 28;                           // 1 GiB of sorted references

// The accumulation's slices hold at least this many references: a group too
// small to fill the resident wave gets fewer, longer slices, trading serial
// additions a thread against levels of the edge fold. Measured on a GB300 over
// 2^12 openings and 2^8-2^14-row shards: 4 beat 16 (4.85 -> 4.61 ms an
// opening at 2^12) and tied 2.
#ifndef APG_ACC_SEG_MIN
#define APG_ACC_SEG_MIN 4
#endif
constexpr size_t kAccSegMin = APG_ACC_SEG_MIN;

// One group: columns share the plan, the bases and one pass of every kernel.
void msm_group(Ctx& c, const Affine* bases, const SrsTable* table, const MsmCols& cols, int ncols, size_t nmax,
               const MsmPlan& p, bool small_scalars, bool scalars_canonical, uint8_t* d_out) {
  const uint32_t K = 1u << (p.c - 1);
  const int spaces_per_col = p.precomp ? 1 : p.windows;
  const int nout = cols.shared ? 1 : ncols;  // results: one per column, or the stack's sum
  const int S = spaces_per_col * nout;
  const size_t nbins = (size_t)S * K;
  size_t emax = 0;
  for (int j = 0; j < ncols; ++j) emax += (size_t)p.windows * cols.len[j];
  const Affine* src = p.precomp ? table->tab : bases;
  const uint32_t tab_n = p.precomp ? (uint32_t)table->n : 0;

  uint32_t* counts = c.scratch[S_COUNTS].as<uint32_t>(nbins + 1);
  const size_t scan_blocks = (nbins + kScanBlock * kScanItems - 1) / (kScanBlock * kScanItems);
  uint32_t* blk = c.scratch[S_SCANBLK].as<uint32_t>(kScanBlock + 1);
  uint32_t* total = c.scratch[S_OFFSETS].as<uint32_t>(1);
  uint32_t* sorted = c.scratch[S_SORTED].as<uint32_t>(std::max<size_t>(emax, 1));
  Xyzz* buckets = c.scratch[S_BUCKETS].as<Xyzz>(nbins);

  const size_t nseg =
      std::max<size_t>(1, std::min(acc_resident_threads(c), (emax + kAccSegMin - 1) / kAccSegMin));
  constexpr int kFoldLen = 8;
  uint32_t* ikeys[2] = {c.scratch[S_HEAD].as<uint32_t>(2 * nseg), c.scratch[S_TAIL].as<uint32_t>(2 * nseg)};
  Xyzz* ipts[2] = {c.scratch[S_TMP0].as<Xyzz>(2 * nseg), c.scratch[S_TMP1].as<Xyzz>(2 * nseg)};
  uint8_t* ipres[2] = {c.scratch[S_FLAGS].as<uint8_t>(2 * nseg), c.scratch[S_TMP2].as<uint8_t>(2 * nseg)};

  int fan_log = 0;
  while ((1 << fan_log) < kLevelFan) ++fan_log;
  int levels = 0;
  for (int M = (int)K;; M = (M + kLevelFan - 1) / kLevelFan) {
    ++levels;
    if (M <= kLevelFan) break;
  }
  Xyzz* tsum = c.scratch[S_TSUM].as<Xyzz>((size_t)levels * S);
  const int G0 = ((int)K + kLevelFan - 1) / kLevelFan;
  Xyzz* outT = c.scratch[S_LEVEL_T].as<Xyzz>((size_t)S * G0);
  Xyzz* lvlA = c.scratch[S_LEVEL_A].as<Xyzz>((size_t)S * G0);
  Xyzz* lvlB = c.scratch[S_LEVEL_B].as<Xyzz>((size_t)S * G0);

  cudaEvent_t t_total = c.timer_begin();
  APG_CUDA(cudaMemsetAsync(counts, 0, (nbins + 1) * sizeof(uint32_t), c.stream));
  APG_CUDA(cudaMemsetAsync(buckets, 0, nbins * sizeof(Xyzz), c.stream));
  const dim3 dgrid(blocks_for<int>(std::max<size_t>(nmax, 1), 256), (unsigned)ncols);
  const int canon = scalars_canonical ? 1 : 0;
  if (small_scalars)
    launch(c, k_digits<true, false>, dgrid, 256, 0, cols, p.c, p.windows, (int)p.precomp, tab_n, canon, counts,
           (uint32_t*)nullptr, c.d_flags);
  else
    launch(c, k_digits<false, false>, dgrid, 256, 0, cols, p.c, p.windows, (int)p.precomp, tab_n, canon, counts,
           (uint32_t*)nullptr, c.d_flags);
  launch(c, k_scan_local, (unsigned)scan_blocks, kScanBlock, 0, counts, nbins, blk);
  launch(c, k_scan_blocks, 1, kScanBlock, 0, blk, (int)scan_blocks);
  launch(c, k_scan_add, blocks_for<int>(nbins, 256), 256, 0, counts, nbins, (const uint32_t*)blk, total);
  if (small_scalars)
    launch(c, k_digits<true, true>, dgrid, 256, 0, cols, p.c, p.windows, (int)p.precomp, tab_n, canon, counts, sorted,
           c.d_flags);
  else
    launch(c, k_digits<false, true>, dgrid, 256, 0, cols, p.c, p.windows, (int)p.precomp, tab_n, canon, counts,
           sorted, c.d_flags);
  cudaEvent_t t_acc = c.timer_begin();
  const uint32_t* pair_mode = nullptr;
  const uint32_t* pair_ends = nullptr;
  const Affine* pair_pts = nullptr;
  if (kPairRounds > 0 && emax >= kPairMinEntries) {
    // Round r's list fits cap[r]: a round keeps ceil(len/2) of each run, so
    // a list never grows and at most halves plus one point per bucket.
    size_t cap[kPairRounds > 0 ? kPairRounds : 1];
    cap[0] = std::min((emax + nbins + 1) / 2, kPairMaxPoints);
    for (int r = 1; r < kPairRounds; ++r) cap[r] = std::min(cap[r - 1], (cap[r - 1] + nbins + 1) / 2);
    const size_t T = pair_resident_threads(c);
    Affine* lst[2] = {c.scratch[S_PAIR_A].as<Affine>(cap[0]),
                      c.scratch[S_PAIR_B].as<Affine>(kPairRounds > 1 ? cap[1] : 1)};
    // Running products (one a slot, j * T + s), the lanes' totals and, with
    // APG_PAIR_PF, the slot words (4 bytes a slot) after them.
    const size_t P = (cap[0] + T - 1) / T * T;
    Fq* pp = c.scratch[S_PAIR_PP].as<Fq>(P + T + (APG_PAIR_PF ? (P + 7) / 8 : 0));
    Fq* tot = pp + P;
    uint32_t* idx = APG_PAIR_PF ? reinterpret_cast<uint32_t*>(tot + T) : nullptr;
    uint32_t* cnt = c.scratch[S_PAIR_CNT].as<uint32_t>((size_t)kPairRounds * (nbins + 1) + 2);
    uint32_t* mode = cnt + (size_t)kPairRounds * (nbins + 1);
    APG_CUDA(cudaMemsetAsync(mode, 0, 2 * sizeof(uint32_t), c.stream));
    const size_t scan_n = nbins + 1;
    const unsigned sblocks = (unsigned)((scan_n + kScanBlock * kScanItems - 1) / (kScanBlock * kScanItems));
    const uint32_t* ends_in = counts;
    const unsigned pblocks = (unsigned)((T + kPairThreads - 1) / kPairThreads);
    for (int r = 0; r < kPairRounds; ++r) {
      uint32_t* st = cnt + (size_t)r * scan_n;
      launch(c, k_halve_counts, blocks_for<int>(scan_n, 256), 256, 0, ends_in, (uint32_t)nbins, st);
      launch(c, k_scan_local, sblocks, kScanBlock, 0, st, scan_n, blk);
      launch(c, k_scan_blocks, 1, kScanBlock, 0, blk, (int)sblocks);
      launch(c, k_scan_add, blocks_for<int>(scan_n, 256), 256, 0, st, scan_n, (const uint32_t*)blk, mode + 1);
      const uint32_t* rr = r == 0 ? (const uint32_t*)sorted : (const uint32_t*)nullptr;
      const Affine* in = r == 0 ? src : lst[(r - 1) & 1];
      if (r == 0) {
        launch(c, k_pair_fwd<true>, pblocks, kPairThreads, 0, rr, in, ends_in, (const uint32_t*)st, (uint32_t)nbins,
               cap[0], mode, T, pp, tot, idx);
        if (APG_PAIR_PF)
          launch(c, k_pair_bwd_pf<true>, pblocks, kPairThreads, 0, rr, in, (const uint32_t*)idx, (const uint32_t*)st,
                 (uint32_t)nbins, (const uint32_t*)mode, T, (const Fq*)pp, (const Fq*)tot, lst[0], c.d_flags);
        else
          launch(c, k_pair_bwd<true>, pblocks, kPairThreads, 0, rr, in, ends_in, (const uint32_t*)st,
                 (uint32_t)nbins, (const uint32_t*)mode, T, (const Fq*)pp, (const Fq*)tot, lst[0], c.d_flags);
      } else {
        launch(c, k_pair_fwd<false>, pblocks, kPairThreads, 0, rr, in, ends_in, (const uint32_t*)st, (uint32_t)nbins,
               cap[r], mode, T, pp, tot, idx);
        if (APG_PAIR_PF)
          launch(c, k_pair_bwd_pf<false>, pblocks, kPairThreads, 0, rr, in, (const uint32_t*)idx,
                 (const uint32_t*)st, (uint32_t)nbins, (const uint32_t*)mode, T, (const Fq*)pp, (const Fq*)tot,
                 lst[r & 1], c.d_flags);
        else
          launch(c, k_pair_bwd<false>, pblocks, kPairThreads, 0, rr, in, ends_in, (const uint32_t*)st,
                 (uint32_t)nbins, (const uint32_t*)mode, T, (const Fq*)pp, (const Fq*)tot, lst[r & 1], c.d_flags);
      }
      ends_in = st + 1;
    }
    pair_mode = mode;
    pair_ends = ends_in;
    pair_pts = lst[(kPairRounds - 1) & 1];
  }
  launch(c, k_bucket_acc, blocks_for<int>(nseg, 128), 128, 0, (const uint32_t*)sorted, (const uint32_t*)counts,
         (uint32_t)nbins, (const uint32_t*)total, nseg, src, buckets, ikeys[0], ipts[0], ipres[0], pair_mode,
         pair_ends, pair_pts);
  c.timer_end(APG_TIMER_MSM_ACCUMULATE, t_acc);
  {
    size_t len = 2 * nseg;
    int cur = 0;
    for (size_t fseg = nseg; fseg > 1;) {
      fseg = (len + kFoldLen - 1) / kFoldLen;
      launch(c, k_fold_edges, blocks_for<int>(fseg, 128), 128, 0, (const uint32_t*)ikeys[cur],
             (const Xyzz*)ipts[cur], (const uint8_t*)ipres[cur], len, kFoldLen, fseg, buckets, ikeys[cur ^ 1],
             ipts[cur ^ 1], ipres[cur ^ 1]);
      cur ^= 1;
      len = 2 * fseg;
    }
  }
  if ((int)K <= kSmallK) {
    launch(c, k_reduce_small, (unsigned)S, (unsigned)K, 0, (const Xyzz*)buckets, (int)K, tsum);
    levels = 1;
  }
  const Xyzz* lvl_in = buckets;
  int M = (int)K;
  for (int l = 0; l < levels && (int)K > kSmallK; ++l) {
    const int G = (M + kLevelFan - 1) / kLevelFan;
    Xyzz* outR = (l & 1) ? lvlB : lvlA;
    launch(c, k_level, blocks_for<int>((size_t)S * G, 64), 64, 0, lvl_in, M, S, kLevelFan, outT, outR);
    if (G > 256) {
      // Wide levels: a two-stage tree keeps the serial chain short.
      const int nblk = (G + 255) / 256;
      Xyzz* part = c.scratch[S_TMP3].as<Xyzz>((size_t)S * nblk);
      launch(c, k_sum_blocks, dim3(nblk, S), 128, 0, (const Xyzz*)outT, G, part);
      launch(c, k_sum, S, 128, 0, (const Xyzz*)part, nblk, tsum + (size_t)l * S);
    } else {
      launch(c, k_sum, S, 128, 0, (const Xyzz*)outT, G, tsum + (size_t)l * S);
    }
    lvl_in = outR;
    M = G;
  }
  launch(c, k_finish_cols, blocks_for<int>(nout, 32), 32, 0, (const Xyzz*)tsum, levels, S, spaces_per_col, nout,
         fan_log, p.c, (uint32_t*)d_out, c.d_flags);
  c.timer_end(APG_TIMER_MSM_TOTAL, t_total);
}

}  // namespace

void msm_multi(Ctx& c, const Affine* bases, const SrsTable* table, const void* const* scalars, const size_t* lens,
               size_t k, bool small_scalars, bool scalars_canonical, uint8_t* d_out, const MsmBatchOpts& o) {
  // A stack sums its columns: every group writes one partial result, added
  // at the end when there is more than one.
  uint8_t* partial = nullptr;
  size_t ngroups = 0;
  if (o.stack) partial = c.scratch[S_TMP7].as<uint8_t>(64 * ((k + kMaxCols - 1) / kMaxCols + k));
  size_t j = 0;
  while (j < k) {
    // Grow the group while the plan, the bucket range and the sorted list fit.
    size_t nmax = 0;
    MsmPlan p{};
    size_t g = 0;
    while (j + g < k && g < (size_t)kMaxCols) {
      const size_t n = lens[j + g];
      if (n >= ((size_t)1 << 31)) throw Error(APG_ERR_INVALID_ARGUMENT, "MSM longer than 2^31 - 1 points");
      const size_t nm = std::max(nmax, n);
      const MsmPlan q = msm_plan(std::max<size_t>(nm, 1), small_scalars, table);
      const size_t spaces = q.precomp ? 1 : (size_t)q.windows;
      const size_t bins = (g + 1) * spaces * ((size_t)1 << (q.c - 1));
      size_t e = 0;
      for (size_t t = 0; t <= g; ++t) e += (size_t)q.windows * lens[j + t];
      if (g > 0 && (bins > kMaxBins || e > kMaxGroupEntries || q.c != p.c || q.windows != p.windows)) break;
      if (bins > kMaxBins) throw Error(APG_ERR_INVALID_ARGUMENT, "too many buckets");
      p = q;
      nmax = nm;
      ++g;
    }
    MsmCols cols{};
    for (size_t t = 0; t < g; ++t) {
      cols.s[t] = scalars[j + t];
      cols.len[t] = (uint32_t)lens[j + t];
      cols.off[t] = o.offs ? (uint32_t)o.offs[j + t] : 0u;
    }
    cols.shared = o.stack ? 1 : 0;
    cols.bits = o.bits;
    uint8_t* dst = o.stack ? partial + 64 * ngroups : d_out + 64 * j;
    msm_group(c, bases, table, cols, (int)g, nmax, p, small_scalars, scalars_canonical, dst);
    ++ngroups;
    j += g;
  }
  if (o.stack) {
    if (ngroups == 0) APG_CUDA(cudaMemsetAsync(d_out, 0, 64, c.stream));
    else if (ngroups == 1) APG_CUDA(cudaMemcpyAsync(d_out, partial, 64, cudaMemcpyDeviceToDevice, c.stream));
    else launch(c, k_add_points, 1, 32, 0, (const uint32_t*)partial, (int)ngroups, (uint32_t*)d_out, c.d_flags);
  }
}

void msm_device(Ctx& c, const Affine* bases, const SrsTable* table, const void* scalars, bool small_scalars,
                bool scalars_canonical, size_t n, uint8_t* out64_device, uint8_t* host_out) {
  if (n == 0) {
    if (out64_device) APG_CUDA(cudaMemsetAsync(out64_device, 0, 64, c.stream));
    if (host_out) memset(host_out, 0, 64);
    return;
  }
  uint8_t* d_out = out64_device ? out64_device : c.scratch[S_RESULT].as<uint8_t>(64);
  msm_multi(c, bases, table, &scalars, &n, 1, small_scalars, scalars_canonical, d_out);
  if (host_out) {
    APG_CUDA(cudaMemcpyAsync(host_out, d_out, 64, cudaMemcpyDeviceToHost, c.stream));
    c.check_flags();
  }
}

// ---------------------------------------------------------------------------
// The allocation-free MSM (apg_msm_noalloc).
//
// Some callers cannot let a library allocate device memory on their behalf:
// a serving loop that has already promised every byte of HBM to admitted
// requests (a cudaMalloc there can fail a request that was admitted, or push
// another tenant out of memory), or a latency-critical pipeline that cannot
// afford the device-wide synchronisation cudaMalloc and cudaFree imply. For
// them this variant of the MSM runs the same kernels with all of its scratch
// in one fixed array that lives in the module's global memory, reserved when
// the module is loaded on a device (with CUDA's lazy loading: the first call,
// or the first launch of any kernel of this file, on that device -- make it
// before the device's memory is promised) and held until the process exits.
// It calls no cudaMalloc, no cudaFree and no allocating library routine.
//
// Limit: at most kNoAllocMaxPoints bases. The plan is fixed: 9-bit signed
// windows (29 of them) with one bucket set per window, 16 entries per
// accumulation segment, so every buffer has a size known at compile time.
// ---------------------------------------------------------------------------

namespace {

constexpr size_t kNoAllocMaxPoints = 4096;
constexpr int kNoAllocC = 9;
constexpr int kNoAllocWindows = (254 + 1 + kNoAllocC - 1) / kNoAllocC;  // 29
constexpr int kNoAllocK = 1 << (kNoAllocC - 1);                          // 256 buckets a window
constexpr size_t kNoAllocBins = (size_t)kNoAllocWindows * kNoAllocK;
constexpr size_t kNoAllocEntries = (size_t)kNoAllocWindows * kNoAllocMaxPoints;
constexpr int kNoAllocSeg = 16;
constexpr size_t kNoAllocSegs = (kNoAllocEntries + kNoAllocSeg - 1) / kNoAllocSeg;
constexpr int kNoAllocG0 = kNoAllocK / kLevelFan;  // 32 groups in the first reduction level
constexpr int kNoAllocLevels = 3;                  // 256 -> 32 -> 4 -> one group

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Byte offsets of every buffer inside the array.
constexpr size_t kOffFlags = 0;
constexpr size_t kOffTotal = kOffFlags + 256;
constexpr size_t kOffResult = kOffTotal + 256;
constexpr size_t kOffBases = kOffResult + 256;
constexpr size_t kOffEntries = kOffBases + align256(kNoAllocMaxPoints * sizeof(Affine));
constexpr size_t kOffSorted = kOffEntries + align256(kNoAllocEntries * 8);
constexpr size_t kOffCounts = kOffSorted + align256(kNoAllocEntries * 8);
constexpr size_t kOffScanBlk = kOffCounts + align256((kNoAllocBins + 1) * 4);
constexpr size_t kOffBuckets = kOffScanBlk + align256((kScanBlock + 1) * 4);
constexpr size_t kOffKeys0 = kOffBuckets + align256(kNoAllocBins * sizeof(Xyzz));
constexpr size_t kOffKeys1 = kOffKeys0 + align256(2 * kNoAllocSegs * 4);
constexpr size_t kOffPts0 = kOffKeys1 + align256(2 * kNoAllocSegs * 4);
constexpr size_t kOffPts1 = kOffPts0 + align256(2 * kNoAllocSegs * sizeof(Xyzz));
constexpr size_t kOffPres0 = kOffPts1 + align256(2 * kNoAllocSegs * sizeof(Xyzz));
constexpr size_t kOffPres1 = kOffPres0 + align256(2 * kNoAllocSegs);
constexpr size_t kOffLvlT = kOffPres1 + align256(2 * kNoAllocSegs);
constexpr size_t kOffLvlA = kOffLvlT + align256((size_t)kNoAllocWindows * kNoAllocG0 * sizeof(Xyzz));
constexpr size_t kOffLvlB = kOffLvlA + align256((size_t)kNoAllocWindows * kNoAllocG0 * sizeof(Xyzz));
constexpr size_t kOffTsum = kOffLvlB + align256((size_t)kNoAllocWindows * kNoAllocG0 * sizeof(Xyzz));
constexpr size_t kNoAllocBytes = kOffTsum + align256((size_t)kNoAllocLevels * kNoAllocWindows * sizeof(Xyzz));

}  // namespace

// The scratch itself (about 8.5 MB). In host code this name is only a
// stand-in for the device symbol: its device address comes from
// cudaGetSymbolAddress, once per device.
static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocBytes];

namespace {

std::mutex g_noalloc_mu;
void* g_noalloc_addr[256] = {nullptr};

// The array's device address, looked up once per device, on the first call
// made with that device current (the set-up step; with CUDA's lazy module
// loading that lookup, or the first launch of any other kernel of this file
// on the device, loads the module, which is when the array is reserved). The
// address belongs to the device's primary context, the one the CUDA runtime
// uses: the entry point assumes no cudaDeviceReset while the library is
// loaded and no other current context.
int noalloc_scratch(int device, uint8_t** out) {
  if (device < 0 || device >= 256) return APG_ERR_NO_DEVICE;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[device]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return APG_ERR_CUDA;
    g_noalloc_addr[device] = p;
  }
  *out = (uint8_t*)g_noalloc_addr[device];
  return APG_OK;
}

#define APG_NA(call)                                \
  do {                                              \
    if ((call) != cudaSuccess) return APG_ERR_CUDA; \
  } while (0)
#define APG_NA_LAUNCH()                                     \
  do {                                                      \
    if (cudaGetLastError() != cudaSuccess) return APG_ERR_CUDA; \
  } while (0)

int msm_noalloc(const void* d_bases, const void* d_scalars, size_t n, void* d_out, cudaStream_t st) {
  if (n > kNoAllocMaxPoints) return APG_ERR_NOALLOC_TOO_LARGE;
  if (!d_out || (n && (!d_bases || !d_scalars))) return APG_ERR_INVALID_ARGUMENT;
  int device = 0;
  APG_NA(cudaGetDevice(&device));
  uint8_t* s = nullptr;
  int rc = noalloc_scratch(device, &s);
  if (rc) return rc;
  if (n == 0) {
    APG_NA(cudaMemsetAsync(d_out, 0, 64, st));
    APG_NA(cudaStreamSynchronize(st));
    return APG_OK;
  }
  uint32_t* flags = (uint32_t*)(s + kOffFlags);
  uint32_t* total = (uint32_t*)(s + kOffTotal);
  Affine* bases = (Affine*)(s + kOffBases);
  uint64_t* entries = (uint64_t*)(s + kOffEntries);
  uint64_t* sorted = (uint64_t*)(s + kOffSorted);
  uint32_t* counts = (uint32_t*)(s + kOffCounts);
  uint32_t* blk = (uint32_t*)(s + kOffScanBlk);
  Xyzz* buckets = (Xyzz*)(s + kOffBuckets);
  uint32_t* ikeys[2] = {(uint32_t*)(s + kOffKeys0), (uint32_t*)(s + kOffKeys1)};
  Xyzz* ipts[2] = {(Xyzz*)(s + kOffPts0), (Xyzz*)(s + kOffPts1)};
  uint8_t* ipres[2] = {s + kOffPres0, s + kOffPres1};
  Xyzz* outT = (Xyzz*)(s + kOffLvlT);
  Xyzz* lvlA = (Xyzz*)(s + kOffLvlA);
  Xyzz* lvlB = (Xyzz*)(s + kOffLvlB);
  Xyzz* tsum = (Xyzz*)(s + kOffTsum);

  const int K = kNoAllocK, W = kNoAllocWindows, spaces = W;
  const size_t nbins = kNoAllocBins;
  const size_t E = (size_t)W * n;
  const size_t nseg = (E + kNoAllocSeg - 1) / kNoAllocSeg;
  const size_t scan_blocks = (nbins + kScanBlock * kScanItems - 1) / (kScanBlock * kScanItems);

  // What a call must find at zero: the error flag, the histogram, the buckets.
  APG_NA(cudaMemsetAsync(flags, 0, 4, st));
  APG_NA(cudaMemsetAsync(counts, 0, (nbins + 1) * sizeof(uint32_t), st));
  APG_NA(cudaMemsetAsync(buckets, 0, nbins * sizeof(Xyzz), st));
  k_points_in<<<blocks_for<int>(n, 256), 256, 0, st>>>((const uint4*)d_bases, n, bases, flags);
  APG_NA_LAUNCH();
  k_recode<false><<<blocks_for<int>(n, 256), 256, 0, st>>>(d_scalars, n, kNoAllocC, W, 0, 0, 0, entries, counts,
                                                            flags);
  APG_NA_LAUNCH();
  k_scan_local<<<(unsigned)scan_blocks, kScanBlock, 0, st>>>(counts, nbins, blk);
  k_scan_blocks<<<1, kScanBlock, 0, st>>>(blk, (int)scan_blocks);
  k_scan_add<<<blocks_for<int>(nbins, 256), 256, 0, st>>>(counts, nbins, (const uint32_t*)blk, total);
  k_scatter<<<blocks_for<int>(E, 256), 256, 0, st>>>((const uint64_t*)entries, E, counts, sorted);
  APG_NA_LAUNCH();
  k_accumulate<<<blocks_for<int>(nseg, 128), 128, 0, st>>>((const uint64_t*)sorted, (const uint32_t*)total,
                                                            kNoAllocSeg, nseg, (const Affine*)bases, buckets,
                                                            ikeys[0], ipts[0], ipres[0]);
  APG_NA_LAUNCH();
  {
    constexpr int kFold = 8;
    size_t len = 2 * nseg;
    int cur = 0;
    for (size_t fseg = nseg; fseg > 1;) {
      fseg = (len + kFold - 1) / kFold;
      k_fold_edges<<<blocks_for<int>(fseg, 128), 128, 0, st>>>((const uint32_t*)ikeys[cur], (const Xyzz*)ipts[cur],
                                                               (const uint8_t*)ipres[cur], len, kFold, fseg, buckets,
                                                               ikeys[cur ^ 1], ipts[cur ^ 1], ipres[cur ^ 1]);
      APG_NA_LAUNCH();
      cur ^= 1;
      len = 2 * fseg;
    }
  }
  const Xyzz* lvl_in = buckets;
  int M = K;
  for (int l = 0; l < kNoAllocLevels; ++l) {
    int G = (M + kLevelFan - 1) / kLevelFan;
    Xyzz* outR = (l & 1) ? lvlB : lvlA;
    k_level<<<blocks_for<int>((size_t)spaces * G, 64), 64, 0, st>>>(lvl_in, M, spaces, kLevelFan, outT, outR);
    k_sum<<<spaces, 128, 0, st>>>((const Xyzz*)outT, G, tsum + (size_t)l * spaces);
    APG_NA_LAUNCH();
    lvl_in = outR;
    M = G;
  }
  int fan_log = 0;
  while ((1 << fan_log) < kLevelFan) ++fan_log;
  k_finish<<<1, 32, 0, st>>>((const Xyzz*)tsum, kNoAllocLevels, spaces, fan_log, kNoAllocC, (uint32_t*)d_out, flags);
  APG_NA_LAUNCH();
  uint32_t f = 0;
  APG_NA(cudaMemcpyAsync(&f, flags, 4, cudaMemcpyDeviceToHost, st));
  APG_NA(cudaStreamSynchronize(st));
  if (f & DEV_NONCANONICAL) return APG_ERR_NONCANONICAL;
  if (f & DEV_OFF_CURVE) return APG_ERR_INVALID_POINT;
  if (f) return APG_ERR_INTERNAL;
  return APG_OK;
}

static_assert(kNoAllocLevels == 3 && kNoAllocK / kLevelFan / kLevelFan <= kLevelFan,
              "the reduction plan above assumes 256 buckets folded 8 at a time");

}  // namespace

}  // namespace apg

extern "C" int apg_msm_noalloc(const void* d_bases, const void* d_scalars, size_t n, void* d_out, void* stream) {
  return apg::msm_noalloc(d_bases, d_scalars, n, d_out, (cudaStream_t)stream);
}
