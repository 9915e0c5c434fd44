// The C ABI boundary (include/apogee_gpu.h): argument checks in the
// reference's refusal order, context locking, and the mapping of every
// failure to an apg_status. No exception crosses this file's functions.
#include <chrono>

#include "common.cuh"
#include "sumcheck.cuh"

using namespace apg;

struct apg_ctx {
  Ctx c;
};

// A host-only entry point: library errors become their status, nothing
// escapes to the caller.
template <class Fn>
static int host_call(Fn&& f) {
  try {
    return f();
  } catch (const Error& e) {
    return e.status;
  } catch (...) {
    return APG_ERR_INTERNAL;
  }
}

extern "C" {
static void release_lane(Ctx& c);
}

namespace {

template <class F>
int guarded(apg_ctx* ctx, F&& f) {
  if (!ctx) return APG_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(ctx->c.mu);
  try {
    APG_CUDA(cudaSetDevice(ctx->c.device));
    int st = f(ctx->c);
    if (st == APG_OK) ctx->c.last_error.clear();
    return st;
  } catch (const Error& e) {
    ctx->c.last_error = e.what();
    return e.status;
  } catch (const std::exception& e) {
    ctx->c.last_error = e.what();
    return APG_ERR_INTERNAL;
  }
}

// Mercury's instance rule (crates/pcs-verify/src/lib.rs:97-102).
bool mercury_num_vars_ok(size_t nv) { return nv >= 2 && nv <= 54 && nv % 2 == 0; }

const SrsTable* commit_table(Ctx& c, size_t n) { return srs_table_for(c, n); }

int commit_common(Ctx& c, const void* evals, bool on_device, bool small, size_t num_vars, uint8_t* out) {
  if (!out || (!evals && num_vars > 0)) return APG_ERR_INVALID_ARGUMENT;
  if (!mercury_num_vars_ok(num_vars)) {
    c.last_error = "unsupported num_vars";
    return APG_ERR_UNSUPPORTED_NUM_VARS;
  }
  if (!c.srs) return APG_ERR_NO_SRS;
  size_t n = (size_t)1 << num_vars;
  if (c.srs_n < n) {
    c.last_error = "the SRS holds fewer powers than the column has evaluations";
    return APG_ERR_SRS_TOO_SMALL;
  }
  const size_t elem = small ? 4 : 32;
  const void* d = evals;
  if (!on_device) {
    void* buf = c.scratch[S_SCALARS].get(n * elem);
    APG_CUDA(cudaMemcpyAsync(buf, evals, n * elem, cudaMemcpyHostToDevice, c.stream));
    d = buf;
  }
  const SrsTable* t = commit_table(c, n);
  if (!t) throw Error(APG_ERR_INTERNAL, "no SRS window table");
  msm_device(c, nullptr, t, d, small, false, n, nullptr, out);
  return APG_OK;
}

int msm_common(Ctx& c, const uint8_t* bases, size_t nb, const void* scalars, size_t ns, bool small, uint8_t* out) {
  if (!out) return APG_ERR_INVALID_ARGUMENT;
  if (nb != ns) {
    c.last_error = "one scalar per base";
    return APG_ERR_LENGTH_MISMATCH;
  }
  if (nb == 0) {
    memset(out, 0, 64);
    return APG_OK;
  }
  if (!bases || !scalars) return APG_ERR_INVALID_ARGUMENT;
  Affine* d_bases = c.scratch[S_BASES].as<Affine>(nb);
  upload_points(c, bases, nb, d_bases);
  const size_t elem = small ? 4 : 32;
  void* d_s = c.scratch[S_SCALARS].get(ns * elem);
  APG_CUDA(cudaMemcpyAsync(d_s, scalars, ns * elem, cudaMemcpyHostToDevice, c.stream));
  msm_device(c, d_bases, nullptr, d_s, small, false, nb, nullptr, out);
  return APG_OK;
}

}  // namespace

extern "C" {

int apg_ctx_create(int device, apg_ctx** out) {
  if (!out) return APG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= device || device < 0) return APG_ERR_NO_DEVICE;
  apg_ctx* ctx = new apg_ctx();
  ctx->c.device = device;
  try {
    APG_CUDA(cudaSetDevice(device));
    APG_CUDA(cudaDeviceGetAttribute(&ctx->c.sm_count, cudaDevAttrMultiProcessorCount, device));
    APG_CUDA(cudaStreamCreateWithFlags(&ctx->c.stream, cudaStreamNonBlocking));
    APG_CUDA(cudaMalloc(&ctx->c.d_flags, 4));
    APG_CUDA(cudaMemset(ctx->c.d_flags, 0, 4));
    // Memory freed to the device's stream-ordered pool (GKR layer values,
    // staged columns) stays in the pool for the next request instead of
    // going back to the driver at every synchronisation.
    cudaMemPool_t pool;
    APG_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t keep = UINT64_MAX;
    APG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
  } catch (const Error& e) {
    delete ctx;
    return e.status;
  }
  *out = ctx;
  return APG_OK;
}

void apg_ctx_destroy(apg_ctx* ctx) {
  if (!ctx) return;
  {
    std::lock_guard<std::mutex> lock(ctx->c.mu);
    Ctx& c = ctx->c;
    cudaSetDevice(c.device);
    if (c.stream) cudaStreamSynchronize(c.stream);
    release_lane(c);
    for (auto& b : c.scratch) b.release();
    for (auto& t : c.tables)
      if (t.owned) cudaFree(t.tab);
    if (c.srs && c.srs_owned) cudaFree(c.srs);
    if (c.d_flags) cudaFree(c.d_flags);
    if (c.pinned) cudaFreeHost(c.pinned);
    if (c.copy_stream) cudaStreamDestroy(c.copy_stream);
    if (c.stream) cudaStreamDestroy(c.stream);
  }
  delete ctx;
}

const char* apg_last_error(apg_ctx* ctx) { return ctx ? ctx->c.last_error.c_str() : "null context"; }

void* apg_ctx_stream(apg_ctx* ctx) { return ctx ? (void*)ctx->c.stream : nullptr; }

int apg_ctx_synchronize(apg_ctx* ctx) {
  return guarded(ctx, [&](Ctx& c) {
    APG_CUDA(cudaStreamSynchronize(c.stream));
    return APG_OK;
  });
}

static void drop_srs(Ctx& c) {
  APG_CUDA(cudaStreamSynchronize(c.stream));
  for (auto& t : c.tables)
    if (t.owned) cudaFree(t.tab);
  c.tables.clear();
  if (c.srs && c.srs_owned) cudaFree(c.srs);
  c.srs = nullptr;
  c.srs_n = 0;
  c.srs_owned = true;
}

int apg_srs_share(apg_ctx* dst, apg_ctx* src) {
  if (!dst || !src || dst == src) return APG_ERR_INVALID_ARGUMENT;
  if (dst->c.device != src->c.device) return APG_ERR_INVALID_ARGUMENT;
  std::vector<SrsTable> tabs;
  int tuned[64];
  Affine* srs;
  size_t n;
  {
    std::lock_guard<std::mutex> lock(src->c.mu);
    if (!src->c.srs) return APG_ERR_NO_SRS;
    srs = src->c.srs;
    n = src->c.srs_n;
    tabs.assign(src->c.tables.begin(), src->c.tables.end());
    memcpy(tuned, src->c.tuned_c, sizeof(tuned));
    cudaStreamSynchronize(src->c.stream);
  }
  return guarded(dst, [&](Ctx& c) {
    drop_srs(c);
    c.srs = srs;
    c.srs_n = n;
    c.srs_owned = false;
    for (auto t : tabs) {
      t.owned = false;
      c.tables.push_back(t);
    }
    memcpy(c.tuned_c, tuned, sizeof(tuned));
    return (int)APG_OK;
  });
}

int apg_msm_autotune(apg_ctx* ctx, const void* d_sample, size_t n_sample, int min_log2n, int max_log2n,
                     const int* cands, size_t n_cands, int* chosen_out) {
  return guarded(ctx, [&](Ctx& c) {
    if (!d_sample || !cands || n_cands == 0 || min_log2n < 0 || max_log2n < min_log2n || max_log2n > 40)
      return (int)APG_ERR_INVALID_ARGUMENT;
    if (!c.srs) return (int)APG_ERR_NO_SRS;
    msm_autotune(c, d_sample, n_sample, min_log2n, max_log2n, cands, n_cands, chosen_out);
    return (int)APG_OK;
  });
}

int apg_srs_upload(apg_ctx* ctx, const uint8_t* g1_points, size_t n) {
  return guarded(ctx, [&](Ctx& c) {
    if (!g1_points || n == 0) return (int)APG_ERR_INVALID_ARGUMENT;
    drop_srs(c);
    Affine* d = nullptr;
    APG_CUDA(cudaMalloc(&d, n * sizeof(Affine)));
    try {
      upload_points(c, g1_points, n, d);
    } catch (...) {
      cudaFree(d);
      throw;
    }
    c.srs = d;
    c.srs_n = n;
    return (int)APG_OK;
  });
}

int apg_srs_generate(apg_ctx* ctx, const uint8_t tau[32], size_t n) {
  return guarded(ctx, [&](Ctx& c) {
    if (!tau || n == 0) return (int)APG_ERR_INVALID_ARGUMENT;
    drop_srs(c);
    Affine* d = nullptr;
    APG_CUDA(cudaMalloc(&d, n * sizeof(Affine)));
    try {
      generate_srs(c, tau, n, d);
    } catch (...) {
      cudaFree(d);
      throw;
    }
    c.srs = d;
    c.srs_n = n;
    return (int)APG_OK;
  });
}

int apg_srs_download(apg_ctx* ctx, uint8_t* g1_points, size_t n) {
  return guarded(ctx, [&](Ctx& c) {
    if (!c.srs) return (int)APG_ERR_NO_SRS;
    if (!g1_points || n > c.srs_n) return (int)APG_ERR_INVALID_ARGUMENT;
    download_points(c, c.srs, n, g1_points);
    return (int)APG_OK;
  });
}

size_t apg_srs_len(apg_ctx* ctx) {
  if (!ctx) return 0;
  std::lock_guard<std::mutex> lock(ctx->c.mu);
  return ctx->c.srs_n;
}

int apg_srs_prepare(apg_ctx* ctx, int cbits) {
  return guarded(ctx, [&](Ctx& c) {
    if (!c.srs) return (int)APG_ERR_NO_SRS;
    if (cbits == 0) {
      srs_table(c, 8, std::min(c.srs_n, (size_t)1 << 14));
      if (c.srs_n > ((size_t)1 << 14)) srs_table(c, 16, c.srs_n);
      if (c.srs_n >= kWideTableMin) srs_table(c, 20, c.srs_n);
    } else {
      if (cbits < 2 || cbits > 20) return (int)APG_ERR_INVALID_ARGUMENT;
      srs_table(c, cbits, c.srs_n);
    }
    return (int)APG_OK;
  });
}

int apg_msm(apg_ctx* ctx, const uint8_t* bases, size_t n_bases, const uint8_t* scalars, size_t n_scalars,
            uint8_t out[64]) {
  return guarded(ctx, [&](Ctx& c) { return msm_common(c, bases, n_bases, scalars, n_scalars, false, out); });
}

int apg_msm_small_u32(apg_ctx* ctx, const uint8_t* bases, size_t n_bases, const uint32_t* scalars,
                      size_t n_scalars, uint8_t out[64]) {
  return guarded(ctx, [&](Ctx& c) { return msm_common(c, bases, n_bases, scalars, n_scalars, true, out); });
}

int apg_discharge_msms(apg_ctx* ctx, const uint8_t* sides, const uint8_t* scalars, const uint8_t* points, size_t n,
                       const size_t* checks, size_t n_checks, uint8_t a_out[64], uint8_t b_out[64],
                       uint8_t nu_out[32]) {
  return guarded(ctx, [&](Ctx& c) {
    return accumulator_msms(c, sides, scalars, points, n, checks, n_checks, nullptr, a_out, b_out, nu_out);
  });
}

int apg_pairing_msms(apg_ctx* ctx, const uint8_t* sides, const uint8_t* scalars, const uint8_t* points, size_t n,
                     const size_t* checks, const uint8_t* weights, size_t n_checks, uint8_t a_out[64],
                     uint8_t b_out[64]) {
  return guarded(ctx, [&](Ctx& c) {
    if (n_checks && !weights) return (int)APG_ERR_INVALID_ARGUMENT;
    static const uint8_t kNone[32] = {0};
    return accumulator_msms(c, sides, scalars, points, n, checks, n_checks, weights ? weights : kNone, a_out, b_out,
                            nullptr);
  });
}

int apg_commit(apg_ctx* ctx, const uint8_t* evals, size_t num_vars, uint8_t out[64]) {
  return guarded(ctx, [&](Ctx& c) { return commit_common(c, evals, false, false, num_vars, out); });
}

int apg_commit_u32(apg_ctx* ctx, const uint32_t* evals, size_t num_vars, uint8_t out[64]) {
  return guarded(ctx, [&](Ctx& c) { return commit_common(c, evals, false, true, num_vars, out); });
}

int apg_commit_device(apg_ctx* ctx, const void* d_evals, size_t num_vars, uint8_t out[64]) {
  return guarded(ctx, [&](Ctx& c) { return commit_common(c, d_evals, true, false, num_vars, out); });
}

// pcs::commit_stack (crates/pcs/src/lib.rs:256-277): column j over the powers
// from j * 2^n, all columns into one bucket set, one result. The reference's
// refusal order: EmptyBatch, SrsTooSmall (k * 2^n powers), MixedColumnSizes.
static int commit_stack_common(Ctx& c, const void* const* cols, const size_t* num_vars, size_t k, bool on_device,
                               uint8_t* out) {
  if (!out) return APG_ERR_INVALID_ARGUMENT;
  if (k == 0) return APG_ERR_EMPTY_BATCH;
  if (!cols || !num_vars) return APG_ERR_INVALID_ARGUMENT;
  if (!c.srs) return APG_ERR_NO_SRS;
  const size_t width = num_vars[0];
  if (width > 40) return APG_ERR_SRS_TOO_SMALL;
  const size_t n = (size_t)1 << width;
  if (c.srs_n / k < n) {
    c.last_error = "the SRS holds fewer powers than the stack has slots";
    return APG_ERR_SRS_TOO_SMALL;
  }
  for (size_t j = 0; j < k; ++j) {
    if (num_vars[j] != width) {
      c.last_error = "stacked columns of different sizes";
      return APG_ERR_MIXED_COLUMN_SIZES;
    }
    if (!cols[j]) return APG_ERR_INVALID_ARGUMENT;
  }
  const SrsTable* t = srs_table_for(c, n * k);
  if (!t) throw Error(APG_ERR_INTERNAL, "no SRS window table");
  std::vector<const void*> ptrs(cols, cols + k);
  if (!on_device) {
    uint8_t* buf = c.scratch[S_SCALARS].as<uint8_t>(32 * n * k);
    for (size_t j = 0; j < k; ++j) {
      APG_CUDA(cudaMemcpyAsync(buf + 32 * n * j, cols[j], 32 * n, cudaMemcpyHostToDevice, c.stream));
      ptrs[j] = buf + 32 * n * j;
    }
  }
  std::vector<size_t> lens(k, n), offs(k);
  for (size_t j = 0; j < k; ++j) offs[j] = j * n;
  MsmBatchOpts o;
  o.offs = offs.data();
  o.stack = true;
  uint8_t* d_out = c.scratch[S_RESULT].as<uint8_t>(64);
  msm_multi(c, nullptr, t, ptrs.data(), lens.data(), k, false, false, d_out, o);
  APG_CUDA(cudaMemcpyAsync(out, d_out, 64, cudaMemcpyDeviceToHost, c.stream));
  c.check_flags();
  return APG_OK;
}

int apg_commit_stack(apg_ctx* ctx, const uint8_t* const* cols, const size_t* num_vars, size_t k, uint8_t out[64]) {
  return guarded(ctx, [&](Ctx& c) {
    return commit_stack_common(c, (const void* const*)cols, num_vars, k, false, out);
  });
}

int apg_commit_stack_device(apg_ctx* ctx, const void* const* d_cols, const size_t* num_vars, size_t k,
                            uint8_t out[64]) {
  return guarded(ctx, [&](Ctx& c) { return commit_stack_common(c, d_cols, num_vars, k, true, out); });
}

int apg_commit_narrow(apg_ctx* ctx, const void* vals, int bits, size_t num_vars, uint8_t out[64]) {
  return guarded(ctx, [&](Ctx& c) {
    if (!out || !vals || (bits != 1 && bits != 8 && bits != 16 && bits != 32)) return (int)APG_ERR_INVALID_ARGUMENT;
    if (!mercury_num_vars_ok(num_vars)) {
      c.last_error = "unsupported num_vars";
      return (int)APG_ERR_UNSUPPORTED_NUM_VARS;
    }
    if (!c.srs) return (int)APG_ERR_NO_SRS;
    const size_t n = (size_t)1 << num_vars;
    if (c.srs_n < n) {
      c.last_error = "the SRS holds fewer powers than the column has evaluations";
      return (int)APG_ERR_SRS_TOO_SMALL;
    }
    const size_t bytes = bits == 1 ? 8 * ((n + 63) / 64) : n * (size_t)bits / 8;
    void* buf = c.scratch[S_SCALARS].get(bytes);
    APG_CUDA(cudaMemcpyAsync(buf, vals, bytes, cudaMemcpyHostToDevice, c.stream));
    const SrsTable* t = commit_table(c, n);
    if (!t) throw Error(APG_ERR_INTERNAL, "no SRS window table");
    const void* ptr = buf;
    MsmBatchOpts o;
    o.bits = bits;
    uint8_t* d_out = c.scratch[S_RESULT].as<uint8_t>(64);
    msm_multi(c, nullptr, t, &ptr, &n, 1, true, false, d_out, o);
    APG_CUDA(cudaMemcpyAsync(out, d_out, 64, cudaMemcpyDeviceToHost, c.stream));
    c.check_flags();
    return (int)APG_OK;
  });
}

// The context's second lane, borrowing its SRS and every window table built
// so far (refreshed per batch so the lane never builds a table of its own).
static Ctx& lane_of(Ctx& c) {
  if (!c.lane) {
    std::unique_ptr<Ctx> L(new Ctx());
    L->device = c.device;
    L->sm_count = c.sm_count;
    APG_CUDA(cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking));
    APG_CUDA(cudaMalloc(&L->d_flags, 4));
    APG_CUDA(cudaMemset(L->d_flags, 0, 4));
    c.lane = std::move(L);
  }
  Ctx& L = *c.lane;
  for (auto& t : L.tables)
    if (t.owned) cudaFree(t.tab);
  L.tables.clear();
  for (auto t : c.tables) {
    t.owned = false;
    L.tables.push_back(t);
  }
  L.srs = c.srs;
  L.srs_n = c.srs_n;
  L.srs_owned = false;
  memcpy(L.tuned_c, c.tuned_c, sizeof(c.tuned_c));
  L.timers.on = c.timers.on;
  L.timers.kernels = c.timers.kernels;
  return L;
}

static void release_lane(Ctx& c) {
  if (!c.lane) return;
  Ctx& L = *c.lane;
  cudaStreamSynchronize(L.stream);
  for (auto& b : L.scratch) b.release();
  for (auto& t : L.tables)
    if (t.owned) cudaFree(t.tab);
  if (L.d_flags) cudaFree(L.d_flags);
  if (L.stream) cudaStreamDestroy(L.stream);
  c.lane.reset();
}

// Groups a batch commit is split into (build knob for measurement).
#ifndef APG_BATCH_GROUPS
#define APG_BATCH_GROUPS 4
#endif

// k commits of one size over the resident SRS. Columns go in groups (one
// sort, accumulation and bucket reduction per group) that alternate between
// the context's two lanes, so one group's latency-bound reduction (and the
// next group's copies) overlap another's bucket accumulation. Columns come
// from device pointers or, when `host` is set, from host memory copied on the
// lane that commits them.
static int commit_batch_lanes(Ctx& c, const void* const* cols, bool host, size_t k, size_t num_vars, uint8_t* out) {
  if (!cols || !out) return APG_ERR_INVALID_ARGUMENT;
  if (!mercury_num_vars_ok(num_vars)) return APG_ERR_UNSUPPORTED_NUM_VARS;
  if (!c.srs) return APG_ERR_NO_SRS;
  const size_t n = (size_t)1 << num_vars;
  if (c.srs_n < n) return APG_ERR_SRS_TOO_SMALL;
  if (k == 0) return APG_OK;
  if (!commit_table(c, n)) throw Error(APG_ERR_INTERNAL, "no SRS window table");
  Ctx& L = lane_of(c);
  Ctx* lanes[2] = {&c, &L};
  uint8_t* d_out = c.scratch[S_TMP5].as<uint8_t>(64 * k);
  // The second lane starts after everything already queued on the first.
  cudaEvent_t ev;
  APG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  APG_CUDA(cudaEventRecord(ev, c.stream));
  APG_CUDA(cudaStreamWaitEvent(L.stream, ev, 0));
  const size_t group = std::max<size_t>(1, (k + APG_BATCH_GROUPS - 1) / APG_BATCH_GROUPS);
  const size_t ngroups = (k + group - 1) / group;
  std::vector<const void*> ptrs(cols, cols + k);
  std::vector<size_t> lens(k, n);
  // Host columns land in one device buffer through a copy stream of their
  // own, group after group, so the copies run back to back at full bandwidth
  // and each group's MSMs start as soon as its own columns are in.
  std::vector<cudaEvent_t> landed;
  if (host) {
    if (!c.copy_stream) APG_CUDA(cudaStreamCreateWithFlags(&c.copy_stream, cudaStreamNonBlocking));
    uint8_t* buf = c.scratch[S_SCALARS].as<uint8_t>(32 * n * k);
    APG_CUDA(cudaStreamWaitEvent(c.copy_stream, ev, 0));  // the buffer's previous users are done
    landed.resize(ngroups, nullptr);
    for (size_t gi = 0; gi < ngroups; ++gi) {
      for (size_t j = gi * group; j < std::min(k, (gi + 1) * group); ++j) {
        APG_CUDA(cudaMemcpyAsync(buf + 32 * n * j, cols[j], 32 * n, cudaMemcpyHostToDevice, c.copy_stream));
        ptrs[j] = buf + 32 * n * j;
      }
      APG_CUDA(cudaEventCreateWithFlags(&landed[gi], cudaEventDisableTiming));
      APG_CUDA(cudaEventRecord(landed[gi], c.copy_stream));
    }
  }
  for (size_t j0 = 0, gi = 0; j0 < k; j0 += group, ++gi) {
    Ctx& X = *lanes[gi & 1];
    const size_t m = std::min(group, k - j0);
    const SrsTable* t = commit_table(X, n);
    if (host) APG_CUDA(cudaStreamWaitEvent(X.stream, landed[gi], 0));
    msm_multi(X, nullptr, t, ptrs.data() + j0, lens.data() + j0, m, false, false, d_out + 64 * j0);
  }
  for (auto e : landed) cudaEventDestroy(e);
  APG_CUDA(cudaEventRecord(ev, L.stream));
  APG_CUDA(cudaStreamWaitEvent(c.stream, ev, 0));
  APG_CUDA(cudaEventDestroy(ev));
  APG_CUDA(cudaMemcpyAsync(out, d_out, 64 * k, cudaMemcpyDeviceToHost, c.stream));
  L.check_flags();
  c.check_flags();
  c.launches += L.launches;
  L.launches = 0;
  if (L.timers.on) {  // the lane's timers count as the context's
    L.timers.flush();
    for (int i = 0; i < Timers::N; ++i) {
      c.timers.ms[i] += L.timers.ms[i];
      c.timers.count[i] += L.timers.count[i];
      L.timers.ms[i] = 0;
      L.timers.count[i] = 0;
    }
  }
  return APG_OK;
}

int apg_commit_batch_device(apg_ctx* ctx, const void* const* d_cols, size_t k, size_t num_vars, uint8_t* out) {
  return guarded(ctx, [&](Ctx& c) { return commit_batch_lanes(c, d_cols, false, k, num_vars, out); });
}

int apg_fr_to_mont_device(apg_ctx* ctx, void* d_vals, size_t n) {
  return guarded(ctx, [&](Ctx& c) {
    if (!d_vals && n) return (int)APG_ERR_INVALID_ARGUMENT;
    if (n) launch(c, k_fr_to_mont, (unsigned)((n + 255) / 256), 256, 0, (Fr*)d_vals, n, c.d_flags);
    c.check_flags();
    return (int)APG_OK;
  });
}

int apg_synth_column(apg_ctx* ctx, uint64_t seed, int kind, size_t n, void* d_out) {
  return guarded(ctx, [&](Ctx& c) {
    if ((!d_out && n) || (kind != 0 && kind != 1) || n > ((size_t)1 << 32)) return (int)APG_ERR_INVALID_ARGUMENT;
    synth_column(c, seed, kind, n, d_out);
    c.check_flags();
    return (int)APG_OK;
  });
}

int apg_prove_zerocheck(apg_ctx* ctx, size_t arity, const uint8_t* coefs, const uint32_t* a, const uint32_t* b,
                        size_t nterms, const uint8_t* const* polys, size_t num_vars, uint8_t* transcript,
                        uint8_t* rounds_out, uint8_t* finals_out) {
  return guarded(ctx, [&](Ctx& c) {
    return prove_zerocheck_impl(c, arity, coefs, a, b, nterms, polys, false, num_vars, transcript, rounds_out,
                                finals_out);
  });
}

int apg_prove_zerocheck_device(apg_ctx* ctx, size_t arity, const uint8_t* coefs, const uint32_t* a,
                               const uint32_t* b, size_t nterms, const void* const* d_polys, size_t num_vars,
                               uint8_t* transcript, uint8_t* rounds_out, uint8_t* finals_out) {
  return guarded(ctx, [&](Ctx& c) {
    return prove_zerocheck_impl(c, arity, coefs, a, b, nterms, (const uint8_t* const*)d_polys, true, num_vars,
                                transcript, rounds_out, finals_out);
  });
}

int apg_prove_zerocheck_narrow(apg_ctx* ctx, size_t arity, const uint8_t* coefs, const uint32_t* a,
                               const uint32_t* b, size_t nterms, const void* const* polys, const uint8_t* bits,
                               int polys_on_device, size_t num_vars, uint8_t* transcript, uint8_t* rounds_out,
                               uint8_t* finals_out) {
  if (!bits) return APG_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&](Ctx& c) {
    return prove_zerocheck_impl(c, arity, coefs, a, b, nterms, (const uint8_t* const*)polys, polys_on_device != 0,
                                num_vars, transcript, rounds_out, finals_out, bits);
  });
}

int apg_witness_digest(apg_ctx* ctx, const uint8_t* const* cols, size_t k, size_t num_vars, uint8_t out[32]) {
  return guarded(ctx, [&](Ctx& c) { return witness_digest_impl(c, cols, k, num_vars, out); });
}

static bool read_points_u(const uint8_t* u, size_t nv, std::vector<host::F>& out) {
  out.resize(nv);
  for (size_t i = 0; i < nv; ++i) {
    memcpy(out[i].w, u + 32 * i, 32);
    if (!host::below_p(out[i].w)) return false;
  }
  return true;
}

int apg_mercury_open(apg_ctx* ctx, const uint8_t* evals, size_t num_vars, const uint8_t cm[64], const uint8_t* u,
                     size_t u_len, uint8_t* transcript, uint8_t v_out[32], uint8_t proof_out[704]) {
  return guarded(ctx, [&](Ctx& c) {
    if (!evals || !cm || (!u && u_len) || !transcript || !v_out || !proof_out) return (int)APG_ERR_INVALID_ARGUMENT;
    if (num_vars < 2 || num_vars > 54 || num_vars % 2) return (int)APG_ERR_UNSUPPORTED_NUM_VARS;
    if (u_len != num_vars) return (int)APG_ERR_POINT_LENGTH_MISMATCH;
    if (num_vars > 40) return (int)APG_ERR_OUT_OF_MEMORY;
    std::vector<host::F> uu;
    if (!read_points_u(u, num_vars, uu)) return (int)APG_ERR_NONCANONICAL;
    host::Transcript tr;
    if (!tr.load(transcript)) return (int)APG_ERR_INVALID_ARGUMENT;
    const size_t n = (size_t)1 << num_vars;
    if (c.srs && c.srs_n < n) return (int)APG_ERR_SRS_TOO_SMALL;
    Fr* d = c.scratch[S_SCALARS].as<Fr>(n);
    APG_CUDA(cudaMemcpyAsync(d, evals, 32 * n, cudaMemcpyHostToDevice, c.stream));
    host::F v;
    int st = mercury_open_impl(c, d, num_vars, cm, uu, tr, v, proof_out);
    if (st) return st;
    memcpy(v_out, v.w, 32);
    tr.save(transcript);
    return (int)APG_OK;
  });
}

// batch_open_stacked's refusals (crates/pcs/src/lib.rs:713-754) in its order,
// then the opening. cols: every stack's columns, stack after stack (host or
// device pointers), num_vars: each column's variable count.
static int stacked_open_common(Ctx& c, const void* const* cols, bool on_device, const size_t* num_vars,
                               const size_t* stack_lens, size_t n_stacks, const uint8_t* cms, size_t n_cms,
                               const uint8_t* u, size_t u_len, const uint8_t* r, size_t r_len, uint8_t* transcript,
                               uint8_t* vs_out, uint8_t* proof_out) {
  if (n_stacks == 0) return APG_ERR_EMPTY_BATCH;
  if (!stack_lens) return APG_ERR_INVALID_ARGUMENT;
  size_t ncols = 0;
  for (size_t j = 0; j < n_stacks; ++j) {
    if (stack_lens[j] == 0) return APG_ERR_EMPTY_BATCH;
    ncols += stack_lens[j];
  }
  if (!cols || !num_vars || (!cms && n_cms) || (!u && u_len) || (!r && r_len) || !transcript || !vs_out ||
      !proof_out)
    return APG_ERR_INVALID_ARGUMENT;
  if (n_cms != n_stacks) return APG_ERR_BATCH_LENGTH_MISMATCH;
  const size_t width = num_vars[0];
  for (size_t i = 1; i < ncols; ++i)
    if (num_vars[i] != width) return APG_ERR_MIXED_COLUMN_SIZES;
  const size_t nv = width + r_len;
  if (width > 54 || r_len > 54 || nv < 2 || nv > 54 || nv % 2) return APG_ERR_UNSUPPORTED_NUM_VARS;
  if (u_len != width) return APG_ERR_POINT_LENGTH_MISMATCH;
  for (size_t j = 0; j < n_stacks; ++j)
    if (stack_lens[j] > ((size_t)1 << r_len)) return APG_ERR_BATCH_LENGTH_MISMATCH;
  if (nv > 40) return APG_ERR_OUT_OF_MEMORY;
  std::vector<host::F> uu, rr;
  if (!read_points_u(u, u_len, uu) || !read_points_u(r, r_len, rr)) return APG_ERR_NONCANONICAL;
  host::Transcript tr;
  if (!tr.load(transcript)) return APG_ERR_INVALID_ARGUMENT;
  if (!c.srs) return APG_ERR_NO_SRS;
  if (c.srs_n < ((size_t)1 << nv)) return APG_ERR_SRS_TOO_SMALL;
  const size_t column = (size_t)1 << width;
  std::vector<const Fr*> ptrs(ncols);
  Fr* staged = nullptr;
  if (on_device) {
    for (size_t i = 0; i < ncols; ++i) ptrs[i] = (const Fr*)cols[i];
  } else {
    APG_CUDA(cudaMallocAsync((void**)&staged, 32 * column * ncols, c.stream));
    for (size_t i = 0; i < ncols; ++i) {
      APG_CUDA(cudaMemcpyAsync(staged + i * column, cols[i], 32 * column, cudaMemcpyHostToDevice, c.stream));
      ptrs[i] = staged + i * column;
    }
  }
  std::vector<host::F> vs;
  int st;
  try {
    st = mercury_batch_open_stacked_impl(c, ptrs.data(), stack_lens, n_stacks, width, cms, uu, rr, tr, vs,
                                         proof_out);
  } catch (...) {
    if (staged) cudaFreeAsync(staged, c.stream);
    throw;
  }
  if (staged) APG_CUDA(cudaFreeAsync(staged, c.stream));
  if (st) return st;
  memcpy(vs_out, vs.data(), 32 * n_stacks);
  tr.save(transcript);
  return APG_OK;
}

// batch_open (crates/pcs/src/lib.rs:688-703): one column a stack, r = [].
static int batch_open_common(Ctx& c, const void* const* cols, bool on_device, size_t k, size_t num_vars,
                             const uint8_t* cms, const uint8_t* u, size_t u_len, uint8_t* transcript,
                             uint8_t* vs_out, uint8_t* proof_out) {
  const std::vector<size_t> ones(k, 1), nvs(k, num_vars);
  return stacked_open_common(c, cols, on_device, nvs.data(), ones.data(), k, cms, k, u, u_len, nullptr, 0,
                             transcript, vs_out, proof_out);
}

int apg_mercury_batch_open(apg_ctx* ctx, const uint8_t* const* cols, size_t k, size_t num_vars, const uint8_t* cms,
                           const uint8_t* u, size_t u_len, uint8_t* transcript, uint8_t* vs_out,
                           uint8_t proof_out[704]) {
  return guarded(ctx, [&](Ctx& c) {
    return batch_open_common(c, (const void* const*)cols, false, k, num_vars, cms, u, u_len, transcript, vs_out,
                             proof_out);
  });
}

int apg_mercury_batch_open_device(apg_ctx* ctx, const void* const* d_cols, size_t k, size_t num_vars,
                                  const uint8_t* cms, const uint8_t* u, size_t u_len, uint8_t* transcript,
                                  uint8_t* vs_out, uint8_t proof_out[704]) {
  return guarded(ctx, [&](Ctx& c) {
    return batch_open_common(c, d_cols, true, k, num_vars, cms, u, u_len, transcript, vs_out, proof_out);
  });
}

int apg_mercury_batch_open_stacked(apg_ctx* ctx, const uint8_t* const* cols, const size_t* num_vars,
                                   const size_t* stack_lens, size_t n_stacks, const uint8_t* cms, size_t n_cms,
                                   const uint8_t* u, size_t u_len, const uint8_t* r, size_t r_len,
                                   uint8_t* transcript, uint8_t* vs_out, uint8_t proof_out[704]) {
  return guarded(ctx, [&](Ctx& c) {
    return stacked_open_common(c, (const void* const*)cols, false, num_vars, stack_lens, n_stacks, cms, n_cms, u,
                               u_len, r, r_len, transcript, vs_out, proof_out);
  });
}

int apg_mercury_batch_open_stacked_device(apg_ctx* ctx, const void* const* d_cols, const size_t* num_vars,
                                          const size_t* stack_lens, size_t n_stacks, const uint8_t* cms,
                                          size_t n_cms, const uint8_t* u, size_t u_len, const uint8_t* r,
                                          size_t r_len, uint8_t* transcript, uint8_t* vs_out,
                                          uint8_t proof_out[704]) {
  return guarded(ctx, [&](Ctx& c) {
    return stacked_open_common(c, d_cols, true, num_vars, stack_lens, n_stacks, cms, n_cms, u, u_len, r, r_len,
                               transcript, vs_out, proof_out);
  });
}

// The device bytes a context holds: its and its lane's scratch, the window
// tables and SRS it owns.
static size_t ctx_bytes(const Ctx& c) {
  size_t b = 0;
  for (const auto& d : c.scratch) b += d.cap;
  for (const auto& t : c.tables)
    if (t.owned) b += (size_t)t.windows * t.n * sizeof(Affine);
  if (c.srs && c.srs_owned) b += c.srs_n * sizeof(Affine);
  if (c.lane) b += ctx_bytes(*c.lane);
  return b;
}

struct apg_gkr_values {
  GkrValues* v;
  apg_ctx* ctx;
};

int apg_gkr_forward(apg_ctx* ctx, const uint8_t* circuit, size_t circuit_len, const uint8_t* const* base,
                    const uint32_t* slots, const uint8_t* slot_values, size_t n_slots, apg_gkr_values** out) {
  if (!out) return APG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  return guarded(ctx, [&](Ctx& c) {
    GkrValues* v = gkr_forward_impl(c, circuit, circuit_len, (const void* const*)base, nullptr, false, slots,
                                    slot_values, n_slots);
    *out = new apg_gkr_values{v, ctx};
    return (int)APG_OK;
  });
}

int apg_gkr_values_read(apg_gkr_values* values, size_t layer, size_t col, uint8_t* out) {
  if (!values) return APG_ERR_INVALID_ARGUMENT;
  return guarded(values->ctx, [&](Ctx&) { return gkr_values_read_impl(values->v, layer, col, out); });
}

size_t apg_gkr_values_len(apg_gkr_values* values, size_t layer) {
  return values ? gkr_values_len(values->v, layer) : 0;
}

void apg_gkr_values_free(apg_gkr_values* values) {
  if (!values) return;
  if (values->ctx) {
    std::lock_guard<std::mutex> lock(values->ctx->c.mu);
    cudaSetDevice(values->ctx->c.device);
    cudaStreamSynchronize(values->ctx->c.stream);
    gkr_values_free(values->v);
  }
  delete values;
}

size_t apg_gkr_proof_len(const uint8_t* circuit, size_t circuit_len) {
  try {
    return gkr_proof_len_impl(circuit, circuit_len);
  } catch (...) {
    return 0;
  }
}

int apg_gkr_verify(const uint8_t* circuit, size_t circuit_len, const uint8_t* const* outputs,
                   const size_t* output_lens, size_t n_outputs, const uint8_t* proof, size_t proof_len,
                   const uint32_t* slots, const uint8_t* slot_values, size_t n_slots, uint8_t* transcript,
                   uint8_t* point_out, uint8_t* values_out, uint64_t* info) {
  try {
    return gkr_verify_impl(circuit, circuit_len, outputs, output_lens, n_outputs, proof, proof_len, slots,
                           slot_values, n_slots, transcript, point_out, values_out, info);
  } catch (const Error& e) {
    return e.status;
  } catch (...) {
    return APG_ERR_INTERNAL;
  }
}

int apg_mercury_verify_deferred(const uint8_t cm[64], const uint8_t* u, size_t u_len, const uint8_t v[32],
                                const uint8_t proof[704], uint8_t* transcript, uint8_t sides_out[12],
                                uint8_t* scalars_out, uint8_t* points_out, uint64_t* info) {
  try {
    return mercury_verify_deferred_impl(cm, u, u_len, v, proof, transcript, sides_out, scalars_out, points_out,
                                        info);
  } catch (const Error& e) {
    return e.status;
  } catch (...) {
    return APG_ERR_INTERNAL;
  }
}

int apg_mercury_batch_verify_deferred(const uint8_t* cms, size_t k, const uint8_t* u, size_t u_len,
                                      const uint8_t* vs, size_t n_vs, const uint8_t proof[704], uint8_t* transcript,
                                      uint8_t sides_out[12], uint8_t* scalars_out, uint8_t* points_out,
                                      uint64_t* info) {
  try {
    return mercury_batch_verify_deferred_impl(cms, k, u, u_len, vs, n_vs, proof, transcript, sides_out, scalars_out,
                                              points_out, info);
  } catch (const Error& e) {
    return e.status;
  } catch (...) {
    return APG_ERR_INTERNAL;
  }
}

int apg_pairing(const uint8_t p[64], const uint8_t q[128], uint8_t out[384]) {
  return host_call([&] { return pairing_impl(p, q, out); });
}

int apg_g2_mul(const uint8_t q[128], const uint8_t k[32], uint8_t out[128]) {
  return host_call([&] { return g2_mul_impl(q, k, out); });
}

int apg_pairing_check(const uint8_t* ps, const uint8_t* qs, size_t n, int* holds) {
  return host_call([&] { return pairing_check_impl(ps, qs, n, holds); });
}

int apg_mercury_verify(const uint8_t vsrs[320], const uint8_t cm[64], const uint8_t* u, size_t u_len,
                       const uint8_t v[32], const uint8_t proof[704], uint8_t* transcript, uint64_t* info) {
  return host_call([&] { return mercury_verify_impl(vsrs, cm, u, u_len, v, proof, transcript, info); });
}

int apg_mercury_batch_verify(const uint8_t vsrs[320], const uint8_t* cms, size_t k, const uint8_t* u, size_t u_len,
                             const uint8_t* vs, size_t n_vs, const uint8_t proof[704], uint8_t* transcript,
                             uint64_t* info) {
  return host_call(
      [&] { return mercury_batch_verify_impl(vsrs, cms, k, u, u_len, vs, n_vs, proof, transcript, info); });
}

int apg_discharge(apg_ctx* ctx, const uint8_t vsrs[320], const uint8_t* sides, const uint8_t* scalars,
                  const uint8_t* points, size_t n, const size_t* checks, size_t n_checks) {
  return guarded(ctx, [&](Ctx& c) {
    uint8_t a[64], b[64], nu[32];
    const int st = accumulator_msms(c, sides, scalars, points, n, checks, n_checks, nullptr, a, b, nu);
    if (st) return st;
    return discharge_pairing_impl(vsrs, a, b);
  });
}

int apg_verify_zerocheck(size_t arity, const uint8_t* coefs, const uint32_t* a, const uint32_t* b, size_t nterms,
                         size_t num_vars, const uint8_t* rounds, size_t n_rounds, const uint8_t* finals,
                         size_t n_finals, uint8_t* transcript, uint8_t* point_out, uint64_t* info) {
  try {
    return verify_zerocheck_impl(arity, coefs, a, b, nterms, num_vars, rounds, n_rounds, finals, n_finals,
                                 transcript, point_out, info);
  } catch (const Error& e) {
    return e.status;
  } catch (...) {
    return APG_ERR_INTERNAL;
  }
}

int apg_gkr_prove(apg_ctx* ctx, const uint8_t* circuit, size_t circuit_len, apg_gkr_values* values,
                  const uint32_t* slots, const uint8_t* slot_values, size_t n_slots, uint8_t* transcript,
                  uint8_t* proof_out, size_t proof_cap, size_t* proof_len, uint8_t* point_out) {
  if (!values || values->ctx != ctx) return APG_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&](Ctx& c) {
    return gkr_prove_impl(c, circuit, circuit_len, values->v, slots, slot_values, n_slots, transcript, proof_out,
                          proof_cap, proof_len, point_out);
  });
}

int apg_gkr_prove_sumcheck(apg_ctx* ctx, const uint8_t* circuit, size_t circuit_len, size_t layer,
                           const uint8_t* weights, size_t n_weights, const uint32_t* slots, const uint8_t* slot_values,
                           size_t n_slots, const uint8_t* eq_point, size_t num_vars, const void* const* d_lower,
                           const void* const* d_upper, size_t width, uint8_t* transcript, uint8_t* rounds_out,
                           uint8_t* point_out, uint8_t* finals_out) {
  return guarded(ctx, [&](Ctx& c) {
    return gkr_prove_sumcheck_impl(c, circuit, circuit_len, layer, weights, n_weights, slots, slot_values, n_slots,
                                   eq_point, num_vars, d_lower, d_upper, width, transcript, rounds_out, point_out,
                                   finals_out);
  });
}

int apg_gkr_forward_device(apg_ctx* ctx, const uint8_t* circuit, size_t circuit_len, const void* const* d_base,
                           const uint32_t* slots, const uint8_t* slot_values, size_t n_slots, apg_gkr_values** out) {
  if (!out) return APG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  return guarded(ctx, [&](Ctx& c) {
    GkrValues* v = gkr_forward_impl(c, circuit, circuit_len, d_base, nullptr, true, slots, slot_values, n_slots);
    *out = new apg_gkr_values{v, ctx};
    return (int)APG_OK;
  });
}

int apg_gkr_forward_narrow(apg_ctx* ctx, const uint8_t* circuit, size_t circuit_len, const void* const* base,
                           const uint8_t* bits, int base_on_device, const uint32_t* slots,
                           const uint8_t* slot_values, size_t n_slots, apg_gkr_values** out) {
  if (!out) return APG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (!bits) return APG_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&](Ctx& c) {
    GkrValues* v = gkr_forward_impl(c, circuit, circuit_len, base, bits, base_on_device != 0, slots, slot_values,
                                    n_slots);
    *out = new apg_gkr_values{v, ctx};
    return (int)APG_OK;
  });
}

void apg_transcript_init(uint8_t snapshot[226]) {
  if (snapshot) host::Transcript().save(snapshot);
}

int apg_transcript_append_scalars(uint8_t snapshot[226], uint64_t tag, const uint8_t* xs, size_t n) {
  host::Transcript tr;
  if (!snapshot || (n && !xs) || !tr.load(snapshot)) return APG_ERR_INVALID_ARGUMENT;
  std::vector<host::F> v(n);
  for (size_t i = 0; i < n; ++i) {
    memcpy(v[i].w, xs + 32 * i, 32);
    if (!host::below_p(v[i].w)) return APG_ERR_NONCANONICAL;
  }
  tr.absorb(tag, v);
  tr.save(snapshot);
  return APG_OK;
}

int apg_transcript_challenge(uint8_t snapshot[226], uint64_t tag, uint8_t out[32]) {
  host::Transcript tr;
  if (!snapshot || !out || !tr.load(snapshot)) return APG_ERR_INVALID_ARGUMENT;
  host::F x = tr.challenge(tag);
  memcpy(out, x.w, 32);
  tr.save(snapshot);
  return APG_OK;
}

int apg_transcript_observe(uint8_t snapshot[226], const uint8_t x[32]) {
  host::Transcript tr;
  if (!snapshot || !x || !tr.load(snapshot)) return APG_ERR_INVALID_ARGUMENT;
  host::F v;
  memcpy(v.w, x, 32);
  if (!host::below_p(v.w)) return APG_ERR_NONCANONICAL;
  tr.observe(v);
  tr.save(snapshot);
  return APG_OK;
}

int apg_transcript_sample(uint8_t snapshot[226], uint8_t out[32]) {
  host::Transcript tr;
  if (!snapshot || !out || !tr.load(snapshot)) return APG_ERR_INVALID_ARGUMENT;
  host::F x = tr.sample();
  memcpy(out, x.w, 32);
  tr.save(snapshot);
  return APG_OK;
}

int apg_transcript_append_bytes(uint8_t snapshot[226], uint64_t tag, const uint8_t* bytes, size_t len) {
  host::Transcript tr;
  if (!snapshot || (len && !bytes) || !tr.load(snapshot)) return APG_ERR_INVALID_ARGUMENT;
  tr.absorb_bytes(tag, bytes, len);
  tr.save(snapshot);
  return APG_OK;
}

int apg_io_digest(const uint8_t* input, size_t input_len, const uint8_t* output, size_t output_len,
                  uint8_t out[32]) {
  if (!out || (input_len && !input) || (output_len && !output)) return APG_ERR_INVALID_ARGUMENT;
  host::F d = host::io_digest(input, input_len, output, output_len);
  memcpy(out, d.w, 32);
  return APG_OK;
}

int apg_poseidon2_permute(uint8_t state[96]) {
  if (!state) return APG_ERR_INVALID_ARGUMENT;
  host::F s[3];
  for (int i = 0; i < 3; ++i)
    if (!host::from_bytes(state + 32 * i, s[i])) return APG_ERR_NONCANONICAL;
  host::permute(s);
  for (int i = 0; i < 3; ++i) host::to_bytes(s[i], state + 32 * i);
  return APG_OK;
}

int apg_ctx_set_timing(apg_ctx* ctx, int on) {
  return guarded(ctx, [&](Ctx& c) {
    c.timers.flush();
    c.timers.on = on != 0;
    c.timers.kernels = on == 2;
    for (int i = 0; i < Timers::N; ++i) {
      c.timers.ms[i] = 0;
      c.timers.count[i] = 0;
    }
    return (int)APG_OK;
  });
}

int apg_ctx_timer(apg_ctx* ctx, int timer, double* ms, uint64_t* launches) {
  return guarded(ctx, [&](Ctx& c) {
    if (timer < 0 || timer >= Timers::N || !ms || !launches) return (int)APG_ERR_INVALID_ARGUMENT;
    c.timers.flush();
    *ms = c.timers.ms[timer];
    *launches = c.timers.count[timer];
    return (int)APG_OK;
  });
}

int apg_probe_fq_mul_rate(apg_ctx* ctx, double ms, double* fq_mul_per_s) {
  return guarded(ctx, [&](Ctx& c) {
    if (!fq_mul_per_s || ms <= 0) return (int)APG_ERR_INVALID_ARGUMENT;
    *fq_mul_per_s = probe_fq_mul_rate(c, ms);
    return (int)APG_OK;
  });
}

uint64_t apg_ctx_launch_count(apg_ctx* ctx) {
  if (!ctx) return 0;
  std::lock_guard<std::mutex> lock(ctx->c.mu);
  return ctx->c.launches;
}

int apg_commit_batch(apg_ctx* ctx, const uint8_t* const* cols, size_t k, size_t num_vars, uint8_t* out) {
  return guarded(ctx, [&](Ctx& c) { return commit_batch_lanes(c, (const void* const*)cols, true, k, num_vars, out); });
}


// One shard: commit, shard transcript, GKR forward and proof, batched opening
// at the base point (crates/prover/src/lib.rs:798-1102, the hot-path slice).
// Host columns are copied once into a stream-ordered device buffer that every
// phase reads; the transcript stays on the host between phases.
static int prove_shard_common(Ctx& c, const apg_shard* sh, apg_shard_proof* out) {
  using Clock = std::chrono::steady_clock;
  if (!sh || !out || !sh->circuit || !sh->cols || !sh->statement_digest || !out->cms || !out->gkr_proof ||
      !out->point || !out->values)
    return APG_ERR_INVALID_ARGUMENT;
  const size_t k = sh->n_cols, nv = sh->num_vars;
  if (k == 0) return APG_ERR_EMPTY_BATCH;
  if (!mercury_num_vars_ok(nv) || nv > 30) return APG_ERR_UNSUPPORTED_NUM_VARS;
  const size_t n = (size_t)1 << nv;
  host::F digest;
  memcpy(digest.w, sh->statement_digest, 32);
  if (!host::below_p(digest.w)) return APG_ERR_NONCANONICAL;
  for (size_t j = 0; j < k; ++j)
    if (!sh->cols[j]) return APG_ERR_INVALID_ARGUMENT;
  if (sh->decoder_width > 7 || (sh->n_ext && (!sh->ext_slots || !sh->ext_values)) || sh->n_ext > 64)
    return APG_ERR_INVALID_ARGUMENT;
  for (size_t e = 0; e < sh->n_ext; ++e) {
    const uint32_t sl = sh->ext_slots[e];
    if (sl == 0 || (sl >= 6 && sl <= 13)) return APG_ERR_INVALID_ARGUMENT;  // drawn by the shard itself
    for (size_t f = 0; f < e; ++f)
      if (sh->ext_slots[f] == sl) return APG_ERR_INVALID_ARGUMENT;
    if (!host::below_p(reinterpret_cast<const uint64_t*>(sh->ext_values + 32 * e))) return APG_ERR_NONCANONICAL;
  }
  std::vector<const void*> d_cols(sh->cols, sh->cols + k);
  Fr* staged = nullptr;
  auto t0 = Clock::now();
  if (!sh->cols_on_device) {
    APG_CUDA(cudaMallocAsync((void**)&staged, 32 * n * k, c.stream));
    for (size_t j = 0; j < k; ++j) {
      APG_CUDA(cudaMemcpyAsync(staged + j * n, sh->cols[j], 32 * n, cudaMemcpyHostToDevice, c.stream));
      d_cols[j] = staged + j * n;
    }
  }
  struct Staged {
    Ctx& c;
    Fr* p;
    ~Staged() {
      if (p) cudaFreeAsync(p, c.stream);
    }
  } guard{c, staged};
  auto ms_since = [](Clock::time_point a) {
    return std::chrono::duration<double, std::milli>(Clock::now() - a).count();
  };
  int st = commit_batch_lanes(c, d_cols.data(), false, k, nv, out->cms);
  if (st) return st;
  out->phase_ms[0] = ms_since(t0);

  // verifier_core::shard_transcript (statement.rs:548-572).
  host::Transcript tr;
  const host::F seed[3] = {digest, host::from_u64(sh->family), host::from_u64(sh->index)};
  tr.absorb(39, seed, 3);  // SHARD_SEED
  const host::F window[2] = {host::from_u64(sh->ts_lo), host::from_u64(sh->ts_hi)};
  tr.absorb(40, window, 2);  // SHARD_TS_WINDOW
  tr.absorb_g1(host::T_COMMITMENT, out->cms, k);
  const host::F g = tr.challenge(33), beta = tr.challenge(33);  // LOOKUP_CHALLENGE
  // verifier_core::shard_challenges: the statement's slots from the caller,
  // then insert_lookup_challenges (crates/gkr-verify/src/lookup.rs:28-61).
  std::vector<uint32_t> slots;
  std::vector<uint8_t> slot_values;
  auto put = [&](uint32_t slot, const host::F& v) {
    slots.push_back(slot);
    slot_values.insert(slot_values.end(), (const uint8_t*)v.w, (const uint8_t*)v.w + 32);
  };
  put(0, g);  // the test circuits' one challenge
  put(6, g);  // LOOKUP_G
  host::F power = beta;
  for (uint32_t j = 0; j < 6; ++j) {  // LOOKUP_BETA .. LOOKUP_BETA_6
    put(7 + j, power);
    power = host::fmul(power, beta);
  }
  if (sh->decoder_width > 0) {  // LOOKUP_DECODER_NEUTRAL = g - sum_{j<W} beta^j
    host::F sum = host::fzero(), pw = host::fone();
    for (uint32_t j = 0; j < sh->decoder_width; ++j) {
      sum = host::fadd(sum, pw);
      pw = host::fmul(pw, beta);
    }
    put(13, host::fsub(g, sum));
  }
  for (size_t e = 0; e < sh->n_ext; ++e) {
    host::F v;
    memcpy(v.w, sh->ext_values + 32 * e, 32);
    put(sh->ext_slots[e], v);
  }
  uint8_t snap[226];
  tr.save(snap);

  auto t1 = Clock::now();
  std::unique_ptr<GkrValues, void (*)(GkrValues*)> V(
      gkr_forward_impl(c, sh->circuit, sh->circuit_len, d_cols.data(), nullptr, true, slots.data(),
                       slot_values.data(), slots.size()),
      gkr_values_free);
  APG_CUDA(cudaStreamSynchronize(c.stream));
  out->phase_ms[1] = ms_since(t1);
  auto t2 = Clock::now();
  st = gkr_prove_impl(c, sh->circuit, sh->circuit_len, V.get(), slots.data(), slot_values.data(), slots.size(), snap,
                      out->gkr_proof,
                      out->gkr_cap, &out->gkr_len, out->point);
  if (st) return st;
  V.reset();
  out->phase_ms[2] = ms_since(t2);

  auto t3 = Clock::now();
  st = batch_open_common(c, d_cols.data(), true, k, nv, out->cms, out->point, nv, snap, out->values, out->opening);
  if (st) return st;
  out->phase_ms[3] = ms_since(t3);
  memcpy(out->transcript, snap, 226);
  return APG_OK;
}

size_t apg_shard_device_bytes(const apg_shard* sh) {
  if (!sh || !sh->circuit || sh->num_vars > 40) return 0;
  try {
    const size_t n = (size_t)1 << sh->num_vars, k = sh->n_cols;
    size_t b = sh->cols_on_device ? 0 : 32 * n * k;  // the staged columns
    b += gkr_device_bytes_impl(sh->circuit, sh->circuit_len);
    // The commits' two lanes: a group of ceil(k / 4) columns sorts up to 15
    // windows a point (4-byte references), and the affine pair rounds hold
    // two point lists and the running products at about half and a quarter
    // of that (capped as msm.cu caps them), plus buckets and levels.
    const size_t g = (k + 3) / 4;
    const size_t E = std::min<size_t>((size_t)15 * n * g, (size_t)1 << 28);
    const size_t cap = (size_t)48 << 20;
    size_t lane = 4 * E + ((size_t)96 << 20);
    if (E >= ((size_t)1 << 21))
      lane += 64 * std::min(E / 2, cap) + 64 * std::min(E / 4, cap) + 32 * std::min(E / 2, cap);
    b += 2 * lane;
    b += 12 * 32 * n;  // the opening's O(n) tables
    return b;
  } catch (...) {
    return 0;
  }
}

int apg_ctx_device(apg_ctx* ctx) { return ctx ? ctx->c.device : -1; }

size_t apg_abi_sizes(size_t* out, size_t n) {
  const size_t sizes[5] = {sizeof(apg_shard), sizeof(apg_shard_proof), sizeof(apg_request_times),
                           sizeof(apg_server_stats), sizeof(apg_server_config)};
  for (size_t i = 0; out && i < n && i < 5; ++i) out[i] = sizes[i];
  return 5;
}

size_t apg_ctx_device_bytes(apg_ctx* ctx) {
  if (!ctx) return 0;
  std::lock_guard<std::mutex> lock(ctx->c.mu);
  return ctx_bytes(ctx->c);
}

int apg_prove_shard(apg_ctx* ctx, const apg_shard* shard, apg_shard_proof* out) {
  return guarded(ctx, [&](Ctx& c) { return prove_shard_common(c, shard, out); });
}
}  // extern "C"
