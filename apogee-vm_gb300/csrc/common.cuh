// Library-internal plumbing: the device context behind an apg_ctx handle,
// status propagation and scratch memory.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/apogee_gpu.h"
#include "curve.cuh"

namespace apg {

// A failure carrying the C ABI status it maps to. Every entry point catches
// it at the boundary; nothing escapes into the caller's process as a throw.
struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define APG_CUDA(call)                                                                                      \
  do {                                                                                                      \
    cudaError_t e_ = (call);                                                                                \
    if (e_ != cudaSuccess)                                                                                  \
      throw ::apg::Error(e_ == cudaErrorMemoryAllocation ? APG_ERR_OUT_OF_MEMORY : APG_ERR_CUDA,          \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                              \
  } while (0)

#define APG_LAUNCH_CHECK() APG_CUDA(cudaGetLastError())

// Device-side error flags a kernel may raise; read back after a sync.
enum DeviceFlag : uint32_t {
  DEV_NONCANONICAL = 1u,   // an input coordinate or scalar was >= its modulus
  DEV_OFF_CURVE = 2u,      // an input point failed y^2 = x^3 + 3
  DEV_TRANSCRIPT = 4u,     // a transcript invariant was broken
  DEV_DEGENERATE = 8u,     // Mercury's {z, 1/z, alpha} had a repeat
  DEV_NONZERO_REM = 16u,   // a division that must be exact left a remainder
  DEV_INVERSE = kFlagInverse,  // a field inversion did not converge (field.cuh)
};

// A grow-only device buffer.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  void* get(size_t bytes) {
    if (bytes > cap) {
      if (p) cudaFree(p);
      p = nullptr;
      cap = 0;
      size_t want = bytes + bytes / 8 + 256;
      APG_CUDA(cudaMalloc(&p, want));
      cap = want;
    }
    return p;
  }
  template <class T>
  T* as(size_t count) {
    return reinterpret_cast<T*>(get(count * sizeof(T)));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

// The precomputed window table of the resident SRS for one window width:
// tab[w * n + i] = 2^(c*w) * P_i, affine Montgomery.
struct SrsTable {
  int c = 0, windows = 0;
  size_t n = 0;
  Affine* tab = nullptr;
  bool owned = true;  // false: borrowed from another context (apg_srs_share)
};

enum ScratchSlot {
  S_ENTRIES, S_SORTED, S_COUNTS, S_OFFSETS, S_SCANBLK, S_BUCKETS, S_HEAD, S_TAIL, S_FLAGS, S_LEVEL_A,
  S_LEVEL_B, S_LEVEL_T, S_TSUM, S_RESULT, S_BASES, S_SCALARS, S_TMP0, S_TMP1, S_TMP2, S_TMP3, S_TMP4,
  S_TMP5, S_TMP6, S_TMP7, S_ROUND, S_PAIR_A, S_PAIR_B, S_PAIR_PP, S_PAIR_CNT, S_PAIR_TERMS, S_COUNT
};

// Per-kernel CUDA-event timers (ids are public: APG_TIMER_* in the header).
struct Timers {
  static constexpr int N = 8;
  bool on = false;
  bool kernels = false;  // also bracket every launch (APG_TIMER_KERNELS)
  std::vector<cudaEvent_t> pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  double ms[N] = {0};
  uint64_t count[N] = {0};
  cudaEvent_t get() {
    if (pool.empty()) {
      cudaEvent_t e;
      APG_CUDA(cudaEventCreate(&e));
      return e;
    }
    cudaEvent_t e = pool.back();
    pool.pop_back();
    return e;
  }
  void flush() {
    for (auto& p : pending) {
      APG_CUDA(cudaEventSynchronize(p.second.second));
      float t = 0;
      APG_CUDA(cudaEventElapsedTime(&t, p.second.first, p.second.second));
      ms[p.first] += t;
      count[p.first] += 1;
      pool.push_back(p.second.first);
      pool.push_back(p.second.second);
    }
    pending.clear();
  }
};

struct Ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  std::string last_error;
  Affine* srs = nullptr;
  size_t srs_n = 0;
  bool srs_owned = true;  // false: borrowed from another context (apg_srs_share)
  std::vector<SrsTable> tables;
  // Window width chosen by apg_msm_autotune per size class (index: ceil of
  // log2 of the point count); 0 = the default rule of srs_table_for.
  int tuned_c[64] = {0};
  DevBuf scratch[S_COUNT];
  uint32_t* d_flags = nullptr;  // device error flags (DeviceFlag bits)
  uint64_t launches = 0;        // kernels launched on this context
  Timers timers;
  // A second stream with its own scratch that borrows this context's SRS:
  // batches of commits alternate between the two so that one MSM's
  // latency-bound tail (and the next column's copy) overlaps another's
  // bucket accumulation.
  std::unique_ptr<Ctx> lane;
  // Host-to-device copies of batch commits' host columns.
  cudaStream_t copy_stream = nullptr;

  // A small pinned host buffer for per-round device-to-host reads (a true
  // asynchronous copy, no staging through pageable memory).
  void* pinned = nullptr;
  void* host_pinned() {
    if (!pinned) APG_CUDA(cudaMallocHost(&pinned, 4096));
    return pinned;
  }

  // Bracket work on the stream with a timer's events (no-op unless enabled).
  cudaEvent_t timer_begin() {
    if (!timers.on) return nullptr;
    cudaEvent_t e = timers.get();
    APG_CUDA(cudaEventRecord(e, stream));
    return e;
  }
  void timer_end(int id, cudaEvent_t begin) {
    if (!timers.on || !begin) return;
    cudaEvent_t e = timers.get();
    APG_CUDA(cudaEventRecord(e, stream));
    timers.pending.push_back({id, {begin, e}});
  }

  void check_flags() {
    uint32_t f = 0;
    APG_CUDA(cudaMemcpyAsync(&f, d_flags, 4, cudaMemcpyDeviceToHost, stream));
    APG_CUDA(cudaStreamSynchronize(stream));
    if (f) {
      APG_CUDA(cudaMemsetAsync(d_flags, 0, 4, stream));
      if (f & DEV_NONCANONICAL) throw Error(APG_ERR_NONCANONICAL, "an input value is not below its modulus");
      if (f & DEV_OFF_CURVE) throw Error(APG_ERR_INVALID_POINT, "an input point is not on the curve");
      if (f & DEV_DEGENERATE) throw Error(APG_ERR_DEGENERATE_CHALLENGE, "degenerate Mercury challenge set");
      if (f & DEV_NONZERO_REM) throw Error(APG_ERR_INTERNAL, "an exact division left a remainder");
      if (f & DEV_INVERSE) throw Error(APG_ERR_INTERNAL, "a field inversion did not converge");
      throw Error(APG_ERR_INTERNAL, "device invariant failed");
    }
  }
};

// Launch a kernel on the context's stream, check the launch and count it.
// With kernel timing on, every launch is bracketed by a pair of events, so
// the sum of kernel durations (the device's busy time on this stream) can be
// set against the wall clock.
template <class... KArgs, class... Args>
inline void launch(Ctx& c, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, Args... args) {
  cudaEvent_t e0 = nullptr;
  if (c.timers.on && c.timers.kernels) {
    if (c.timers.pending.size() > 4096) c.timers.flush();
    e0 = c.timers.get();
    APG_CUDA(cudaEventRecord(e0, c.stream));
  }
  kernel<<<grid, block, smem, c.stream>>>(args...);
  APG_CUDA(cudaGetLastError());
  ++c.launches;
  if (e0) {
    cudaEvent_t e1 = c.timers.get();
    APG_CUDA(cudaEventRecord(e1, c.stream));
    c.timers.pending.push_back({APG_TIMER_KERNELS, {e0, e1}});
  }
}

// ---------------------------------------------------------------------------
// Entry points implemented in the .cu files.
// ---------------------------------------------------------------------------

// Canonical Fr -> Montgomery in place, raising DEV_NONCANONICAL for values >= p.
__global__ void k_fr_to_mont(Fr* v, size_t n, uint32_t* flags);

// Canonical 64-byte points (host) -> device affine Montgomery, validated.
void upload_points(Ctx& c, const uint8_t* host, size_t n, Affine* dst);
// The same without waiting: the flags are the caller's to check.
void upload_points_async(Ctx& c, const uint8_t* host, size_t n, Affine* dst);
// Device affine Montgomery -> canonical 64-byte points (host).
void download_points(Ctx& c, const Affine* src, size_t n, uint8_t* host);
// SRS [tau^i]G for i < n, generated on the device.
void generate_srs(Ctx& c, const uint8_t tau_canonical[32], size_t n, Affine* dst);
// n seeded benchmark Fr (canonical, 8 LE words each) from the ChaCha20 keystream:
// kind 0 trace-like (bits, register words, uniform Fr), kind 1 uniform Fr.
void synth_column(Ctx& c, uint64_t seed, int kind, size_t n, void* d_out);

// Pippenger over device inputs; the result (canonical affine bytes, 64) is
// written to device memory `out64` when non-null and returned to `host_out`
// when non-null.
struct MsmPlan {
  int c;         // window width
  int windows;   // signed-digit windows
  bool precomp;  // read bases from an SRS window table
};
MsmPlan msm_plan(size_t n, bool small_scalars, const SrsTable* table);
void msm_device(Ctx& c, const Affine* bases, const SrsTable* table, const void* scalars, bool small_scalars,
                bool scalars_canonical, size_t n, uint8_t* out64_device, uint8_t* host_out);
// k MSMs over the same bases (lens[j] scalars each, device pointers); result
// j is written to d_out + 64 * j. Columns are processed in groups that share
// one sort, one accumulation and one bucket reduction.
struct MsmBatchOpts {
  const size_t* offs = nullptr;  // first base of each column (nullable: all 0)
  bool stack = false;            // one result: the sum of every column's MSM
  int bits = 32;                 // width of small scalars: 32, 16, 8 or 1 (bit-packed u64)
};
void msm_multi(Ctx& c, const Affine* bases, const SrsTable* table, const void* const* scalars, const size_t* lens,
               size_t k, bool small_scalars, bool scalars_canonical, uint8_t* d_out,
               const MsmBatchOpts& o = MsmBatchOpts());
const SrsTable* srs_table(Ctx& c, int cbits, size_t need);
// The table an MSM of the first n SRS powers reads: 8-bit windows up to 2^14
// points (a cheap bucket reduction), 16-bit windows below kWideTableMin and
// 20-bit windows from there (13 windows instead of 16; the 2^19 buckets a
// column are amortised over at least 2^20 points). Null if the SRS is short.
// `tuned`: use the width apg_msm_autotune chose for the size class, if any
// (commits of the caller's columns); openings commit uniformly random
// quotient polynomials, for which the default rule is the uniform-scalar one.
constexpr size_t kWideTableMin = (size_t)1 << 20;
const SrsTable* srs_table_for(Ctx& c, size_t n, bool tuned = true);
// Time SRS commits of the first 2^k sample scalars for k in [kmin, kmax] with
// each candidate width and record the fastest in c.tuned_c (see
// apg_msm_autotune).
void msm_autotune(Ctx& c, const void* d_sample, size_t sample_len, int kmin, int kmax, const int* cands,
                  size_t ncands, int* chosen);
double probe_fq_mul_rate(Ctx& c, double target_ms);
// The group side of pcs::discharge (weights null) or check_pairings (one
// weight a check): see apg_discharge_msms / apg_pairing_msms.
int accumulator_msms(Ctx& c, const uint8_t* sides, const uint8_t* scalars, const uint8_t* points, size_t n,
                     const size_t* checks, size_t nchecks, const uint8_t* weights, uint8_t* a_out, uint8_t* b_out,
                     uint8_t* nu_out);

}  // namespace apg
