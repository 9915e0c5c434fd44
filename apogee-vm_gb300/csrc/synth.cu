// Seeded benchmark columns generated on the device.
//
// The benchmarks draw their inputs from a ChaCha20 keystream (RFC 8439 §2.3
// block function, written here) keyed from a 64-bit seed, the way the
// reference's bench tool draws its own; the rule that turns the keystream into
// field elements is the reference's: 32 little-endian bytes with the top two
// bits cleared, rejected while >= r or zero (tools/bench/src/timing.rs:56-67).
// synth.py states the same layout in numpy, so a column made on the host and
// one made here from the same seed are the same bytes.
//
// Keystream layout (key = seed as 8 LE bytes then 24 zero bytes; every block
// counter starts at 0):
//   stream 0 (nonce 0,0,0)   entry i reads the word pair (2j, 2j+1), j = i mod 8,
//                            of block i/8: a 32-bit value and, in the low 16
//                            bits of the second word, its class draw c.
//                            c < 16384 -> value & 1 (a bit, 25%)
//                            c < 55706 -> value     (a register word, 60%)
//                            otherwise -> a uniform Fr (15%)
//   stream t+1 (nonce t+1,0,0) attempt t of entry i's uniform Fr: words
//                            8(i mod 2) .. 8(i mod 2)+7 of block i/2.
// A uniform column (kind 1) takes every entry from the attempt streams.
#include "common.cuh"

namespace apg {

namespace {

constexpr uint32_t kClassBits = 16384;  // 25% of 2^16
constexpr uint32_t kClassWord = 55706;  // 85% of 2^16, rounded up
constexpr uint32_t kMaxAttempts = 64;   // each attempt is accepted with p > 3/4

__device__ __forceinline__ void quarter(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d) {
  a += b;
  d = __funnelshift_l(d ^ a, d ^ a, 16);
  c += d;
  b = __funnelshift_l(b ^ c, b ^ c, 12);
  a += b;
  d = __funnelshift_l(d ^ a, d ^ a, 8);
  c += d;
  b = __funnelshift_l(b ^ c, b ^ c, 7);
}

// One 64-byte ChaCha20 block as sixteen little-endian words.
__device__ __forceinline__ void chacha_block(uint64_t seed, uint32_t nonce0, uint32_t counter, uint32_t out[16]) {
  const uint32_t in[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, (uint32_t)seed,
                           (uint32_t)(seed >> 32), 0u, 0u, 0u, 0u, 0u, 0u, counter, nonce0, 0u, 0u};
  uint32_t x[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) x[k] = in[k];
#pragma unroll 1
  for (int r = 0; r < 10; ++r) {
    quarter(x[0], x[4], x[8], x[12]);
    quarter(x[1], x[5], x[9], x[13]);
    quarter(x[2], x[6], x[10], x[14]);
    quarter(x[3], x[7], x[11], x[15]);
    quarter(x[0], x[5], x[10], x[15]);
    quarter(x[1], x[6], x[11], x[12]);
    quarter(x[2], x[7], x[8], x[13]);
    quarter(x[3], x[4], x[9], x[14]);
  }
#pragma unroll
  for (int k = 0; k < 16; ++k) out[k] = x[k] + in[k];
}

__global__ void __launch_bounds__(256) k_synth_column(uint64_t seed, int kind, size_t n, Fr* out, uint32_t* flags) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t v[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
  bool field = kind == 1;
  uint32_t blk[16];
  if (!field) {
    chacha_block(seed, 0u, (uint32_t)(i >> 3), blk);
    uint32_t w = 0, c = 0;
    const uint32_t j = (uint32_t)(i & 7);
#pragma unroll
    for (uint32_t k = 0; k < 8; ++k) {
      if (k == j) {
        w = blk[2 * k];
        c = blk[2 * k + 1] & 0xFFFFu;
      }
    }
    if (c < kClassBits) {
      v[0] = w & 1u;
    } else if (c < kClassWord) {
      v[0] = w;
    } else {
      field = true;
    }
  }
  if (field) {
    bool ok = false;
    const bool hi = (i & 1) != 0;
    for (uint32_t t = 0; t < kMaxAttempts && !ok; ++t) {
      chacha_block(seed, t + 1, (uint32_t)(i >> 1), blk);
      uint32_t any = 0;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        v[k] = hi ? blk[8 + k] : blk[k];
      }
      v[7] &= 0x3FFFFFFFu;
#pragma unroll
      for (int k = 0; k < 8; ++k) any |= v[k];
      ok = any != 0 && fe_lt_mod<FrConsts>(v);
    }
    if (!ok) atomicOr(flags, (uint32_t)DEV_NONCANONICAL);
  }
  Fr r;
#pragma unroll
  for (int k = 0; k < 8; ++k) r.v[k] = v[k];
  st_fe(&out[i], r);
}

}  // namespace

void synth_column(Ctx& c, uint64_t seed, int kind, size_t n, void* d_out) {
  if (n) launch(c, k_synth_column, (unsigned)((n + 255) / 256), 256, 0, seed, kind, n, (Fr*)d_out, c.d_flags);
}

}  // namespace apg
