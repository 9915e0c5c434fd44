// Device throughput probe: the integer-pipe ceiling the MSM's roofline is
// quoted against, measured on the device in use rather than assumed.
//
// Every thread runs four independent Fq Montgomery products per iteration,
// each feeding only itself on the next iteration, so nothing but the multiply
// pipe's issue rate bounds the loop.
#include "common.cuh"

namespace apg {
namespace {

__global__ void __launch_bounds__(256) k_fq_mul_rate(uint64_t iters, Fq* sink) {
  Fq a = fe_one<FqConsts>(), b = fe_one<FqConsts>(), c = fe_one<FqConsts>(), d = fe_one<FqConsts>();
  a.v[0] ^= threadIdx.x;
  b.v[1] ^= blockIdx.x;
  c.v[2] ^= threadIdx.x * 7u;
  d.v[3] ^= blockIdx.x * 13u;
  const Fq k = fe_add(a, b);
  for (uint64_t i = 0; i < iters; ++i) {
    a = fe_mul(a, k);
    b = fe_mul(b, k);
    c = fe_mul(c, k);
    d = fe_mul(d, k);
  }
  Fq s = fe_add(fe_add(a, b), fe_add(c, d));
  if (fe_is_zero(s)) st_fe(&sink[blockIdx.x], s);  // keeps the loop live; never true in practice
}

}  // namespace

double probe_fq_mul_rate(Ctx& c, double target_ms) {
  Fq* sink = c.scratch[S_TMP4].as<Fq>(4096);
  const unsigned blocks = (unsigned)c.sm_count * 4;
  const unsigned threads = 256;
  cudaEvent_t e0, e1;
  APG_CUDA(cudaEventCreate(&e0));
  APG_CUDA(cudaEventCreate(&e1));
  uint64_t iters = 64;
  double ms = 0;
  for (int attempt = 0; attempt < 12; ++attempt) {
    APG_CUDA(cudaEventRecord(e0, c.stream));
    launch(c, k_fq_mul_rate, blocks, threads, 0, iters, sink);
    APG_CUDA(cudaEventRecord(e1, c.stream));
    APG_CUDA(cudaEventSynchronize(e1));
    float t = 0;
    APG_CUDA(cudaEventElapsedTime(&t, e0, e1));
    ms = t;
    if (ms >= target_ms) break;
    iters = (uint64_t)(iters * std::min(16.0, std::max(2.0, 1.2 * target_ms / std::max(ms, 1e-3))));
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return (double)blocks * threads * 4.0 * (double)iters / (ms * 1e-3);
}

}  // namespace apg
