/*
 * apogee_gpu.h — the C ABI of the GB300 shard-proving hot path.
 *
 * A drop-in for the commit/open and sumcheck-prover interfaces that the
 * reference's crates/prover calls: crates/curve (msm), crates/pcs (commit,
 * open, batch_open), crates/sumcheck (prove_zerocheck) and crates/gkr
 * (forward, prove). Each entry point below names the reference function it
 * replaces (file:line, paths inside the reference project).
 *
 * Conventions (the reference's own, so a binding converts nothing):
 *  - Fr in memory: 32 bytes, the four 64-bit Montgomery limbs little-endian,
 *    exactly Fr::to_memory_bytes (crates/field/src/lib.rs:321); a `&[Fr]`
 *    slice is passed as its data pointer.
 *  - Fr on the wire (proof values, challenges, claims): 32 canonical
 *    little-endian bytes, Fr::to_bytes (lib.rs:252).
 *  - G1: 64 bytes x || y canonical little-endian, all-zero = infinity,
 *    G1Affine::to_bytes (crates/curve/src/g1.rs:92-100).
 *  - A transcript crosses as its 226-byte TranscriptSnapshot tuple
 *    (state[3], input[2], input_len:u8, output[2], output_len:u8; Fr
 *    canonical), in/out (crates/transcript/src/lib.rs:188-194, 353-376).
 *  - Every function returns an apg_status; 0 is success. Nothing aborts the
 *    caller's process; apg_last_error() describes the last failure.
 *  - A context is thread-safe (calls on one context serialise); use one
 *    context per concurrent caller to overlap work.
 */
#ifndef APOGEE_GPU_H
#define APOGEE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct apg_ctx apg_ctx;

/* Status codes. 1..9 mirror MsmError / PcsError variants
 * (crates/curve/src/msm.rs:29-33, crates/pcs-verify/src/lib.rs:40-86). */
enum apg_status {
  APG_OK = 0,
  APG_ERR_LENGTH_MISMATCH = 1,        /* MsmError::LengthMismatch */
  APG_ERR_UNSUPPORTED_NUM_VARS = 2,   /* PcsError::UnsupportedNumVars */
  APG_ERR_POINT_LENGTH_MISMATCH = 3,  /* PcsError::PointLengthMismatch */
  APG_ERR_SRS_TOO_SMALL = 4,          /* PcsError::SrsTooSmall */
  APG_ERR_DEGENERATE_CHALLENGE = 5,   /* PcsError::DegenerateChallenge */
  APG_ERR_EMPTY_BATCH = 6,            /* PcsError::EmptyBatch */
  APG_ERR_BATCH_LENGTH_MISMATCH = 7,  /* PcsError::BatchLengthMismatch */
  APG_ERR_MIXED_COLUMN_SIZES = 8,     /* PcsError::MixedColumnSizes */
  APG_ERR_INVALID_POINT = 9,          /* PcsError::InvalidPoint / off-curve input */
  APG_ERR_MALFORMED_ACCUMULATOR = 10, /* PcsError::MalformedAccumulator */
  APG_ERR_VERIFICATION_FAILED = 11,   /* PcsError::VerificationFailed: the pairing check failed */
  APG_ERR_NONCANONICAL = 20,          /* an input value is >= its modulus */
  APG_ERR_INVALID_ARGUMENT = 21,      /* null pointer, bad shape */
  APG_ERR_BAD_CIRCUIT = 22,           /* malformed circuit blob */
  APG_ERR_NO_SRS = 23,                /* no SRS resident on the context */
  APG_ERR_INTERNAL = 24,              /* a device invariant failed */
  APG_ERR_NOALLOC_TOO_LARGE = 25,     /* apg_msm_noalloc: more bases than its fixed scratch holds */
  APG_PENDING = 26,                   /* apg_poll: the request is queued or running */
  APG_ERR_UNKNOWN_TICKET = 27,        /* apg_poll / apg_wait: no such request */
  APG_ERR_MISSING_CHALLENGE = 28,     /* GkrError::MissingChallenge (info: the slot) */
  APG_ERR_OUTPUT_SHAPE = 29,          /* GkrError::OutputShape */
  APG_ERR_PROOF_SHAPE = 30,           /* GkrError::ProofShape (info: the gate list) */
  APG_ERR_LAYER_INCONSISTENCY = 31,   /* GkrError::LayerInconsistency (info: the gate list) */
  APG_ERR_ROUND_COUNT_MISMATCH = 32,  /* SumcheckError::RoundCountMismatch (info: rounds found) */
  APG_ERR_FINAL_COUNT_MISMATCH = 33,  /* SumcheckError::FinalEvalCountMismatch (info: finals found) */
  APG_ERR_ROUND_SUM_MISMATCH = 34,    /* SumcheckError::RoundSumMismatch (info: the round) */
  APG_ERR_FINAL_EVAL_MISMATCH = 35,   /* SumcheckError::FinalEvalMismatch */
  APG_ERR_CUDA = 100,                 /* a CUDA call failed */
  APG_ERR_OUT_OF_MEMORY = 101,        /* device allocation refused */
  APG_ERR_NO_DEVICE = 103             /* no usable CUDA device */
};

#define APG_TRANSCRIPT_BYTES 226
#define APG_PROOF_BYTES 704

/* ---- context ---------------------------------------------------------- */

/* Create a context on CUDA device `device` (one stream, its own scratch). */
int apg_ctx_create(int device, apg_ctx** out);
void apg_ctx_destroy(apg_ctx* ctx);
/* The last failure's message on this context ("" if none). */
const char* apg_last_error(apg_ctx* ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that time or
 * order work against it. */
void* apg_ctx_stream(apg_ctx* ctx);
/* The CUDA device ordinal of the context (-1 for null). */
int apg_ctx_device(apg_ctx* ctx);
/* Block until all work queued on the context has finished. */
int apg_ctx_synchronize(apg_ctx* ctx);

/* ---- SRS (crates/srs/src/lib.rs:96-100, 244: Srs::g1) ------------------- */

/* Make `n` G1 powers resident on the device (canonical 64-byte points, each
 * validated). Replaces handing `srs.g1()` to every commit. */
int apg_srs_upload(apg_ctx* ctx, const uint8_t* g1_points, size_t n);
/* Benchmark-only setup: [tau^i]G for i < n from a given tau (canonical Fr),
 * computed on the device. Not a secure setup. */
int apg_srs_generate(apg_ctx* ctx, const uint8_t tau[32], size_t n);
/* Copy the first n resident powers out (canonical 64-byte points). */
int apg_srs_download(apg_ctx* ctx, uint8_t* g1_points, size_t n);
/* Number of resident powers. */
size_t apg_srs_len(apg_ctx* ctx);
/* Let `dst` read the SRS (and the window tables built so far) that `src`
 * holds on the same device, without a copy: contexts that prove shards
 * concurrently share one resident SRS. `src` must outlive `dst`'s use of it
 * and must not replace its SRS meanwhile. */
int apg_srs_share(apg_ctx* dst, apg_ctx* src);
/* Precompute the window table that commits over the resident SRS read
 * (window width `cbits`, 0 = the library's choice). Optional: the first
 * commit builds it. Costs windows x n x 64 bytes of device memory. */
int apg_srs_prepare(apg_ctx* ctx, int cbits);
/* No reference counterpart (the reference derives its window from n alone,
 * crates/curve/src/msm.rs:112-118). The window-width autotuner: for each size
 * class 2^k, min_log2n <= k <= max_log2n, time commits of the first 2^k of
 * the n_sample device scalars (Fr in memory, drawn like the columns to be
 * committed) with every candidate width (bits, 2..20; widths below 12 only
 * up to 2^16 points), building the window tables it needs, and keep the
 * fastest for this context's later commits (shared contexts and lanes inherit
 * it; openings keep the default widths, their quotient polynomials being
 * uniformly random). chosen_out (nullable) receives max_log2n - min_log2n + 1
 * widths, 0 where a class exceeds the sample or the SRS. */
int apg_msm_autotune(apg_ctx* ctx, const void* d_sample, size_t n_sample, int min_log2n, int max_log2n,
                     const int* cands, size_t n_cands, int* chosen_out);

/* ---- MSM (crates/curve/src/msm.rs) ------------------------------------- */

/* msm::msm (msm.rs:48): sum scalars[i] * bases[i]. bases: canonical 64-byte
 * points; scalars: Fr in memory (Montgomery). Lengths must match
 * (APG_ERR_LENGTH_MISMATCH); empty input is the identity (64 zero bytes). */
int apg_msm(apg_ctx* ctx, const uint8_t* bases, size_t n_bases, const uint8_t* scalars, size_t n_scalars,
            uint8_t out[64]);
/* msm::msm_small_u32 (msm.rs:79): the same over u32 scalars. */
int apg_msm_small_u32(apg_ctx* ctx, const uint8_t* bases, size_t n_bases, const uint32_t* scalars,
                      size_t n_scalars, uint8_t out[64]);

/* No counterpart in the reference: an MSM that allocates no device memory,
 * for callers that cannot let a library allocate on their behalf -- a
 * serving loop whose HBM is already promised to admitted requests, or a
 * latency-critical pipeline that cannot take the device-wide synchronisation
 * of cudaMalloc/cudaFree. It computes exactly what apg_msm does, with every
 * buffer carved from one fixed array in the library's device global memory
 * (about 8.5 MB on every GPU the library's MSM module is loaded on, until
 * exit; under CUDA's lazy module loading the module loads at the first call
 * on a device, or at the first launch of another MSM kernel there, so make
 * that first call before the device's memory is promised elsewhere).
 *   d_bases:   n canonical 64-byte points in device memory (all-zero =
 *              infinity), d_scalars: n Fr in memory in device memory,
 *   d_out:     64 bytes of device memory for the canonical result,
 *   stream:    the cudaStream_t to run on (0 = legacy default stream), on the
 *              current device. The call returns when the result is written.
 * At most APG_MSM_NOALLOC_MAX_POINTS bases (APG_ERR_NOALLOC_TOO_LARGE above).
 * The first call on a device looks up the array's device address (and may
 * load the module); make that first call before any stream capture. The
 * address is the device's primary context's (the CUDA runtime's): no
 * cudaDeviceReset while the library is loaded. All calls on a device share the one
 * array (each clears what must start at zero), so calls that overlap on the
 * GPU race: serialise them, e.g. on one stream. */
#define APG_MSM_NOALLOC_MAX_POINTS 4096
int apg_msm_noalloc(const void* d_bases, const void* d_scalars, size_t n, void* d_out, void* stream);

/* ---- commit (crates/pcs/src/lib.rs:237-298) ---------------------------- */

/* pcs::commit over the resident SRS: the KZG commitment to the 2^num_vars
 * evaluations read as coefficients. evals: Fr in memory (Montgomery).
 * Errors: APG_ERR_UNSUPPORTED_NUM_VARS (odd or out of 2..54),
 * APG_ERR_SRS_TOO_SMALL, APG_ERR_NO_SRS. */
int apg_commit(apg_ctx* ctx, const uint8_t* evals, size_t num_vars, uint8_t out[64]);
/* pcs::commit of a narrow column (column_msm's U1/U8/U16/U32 arms,
 * lib.rs:280-298): u32 values through the small-scalar path. */
int apg_commit_u32(apg_ctx* ctx, const uint32_t* evals, size_t num_vars, uint8_t out[64]);
/* commit_all (crates/prover/src/lib.rs:444-471): k columns of one size,
 * cols[j] pointing at column j's evaluations (Fr in memory); out: k x 64. */
int apg_commit_batch(apg_ctx* ctx, const uint8_t* const* cols, size_t k, size_t num_vars, uint8_t* out);
/* As apg_commit, with the evaluations already in device memory (a pointer
 * the caller allocated on this context's device). */
int apg_commit_device(apg_ctx* ctx, const void* d_evals, size_t num_vars, uint8_t out[64]);
/* As apg_commit_batch over device-resident columns; the k MSMs run back to
 * back on the context's stream and the call returns once all are done. */
int apg_commit_batch_device(apg_ctx* ctx, const void* const* d_cols, size_t k, size_t num_vars, uint8_t* out);
/* pcs::commit_stack (crates/pcs/src/lib.rs:256-277): the commitment of the
 * stack whose evaluations [j*2^n, (j+1)*2^n) are column j, read as
 * coefficients over the resident SRS (the stack is never materialised: column
 * j is an MSM over the powers from j*2^n, every column into one bucket set).
 * num_vars[j] is column j's variable count, n = num_vars[0]; columns are host
 * Fr in memory. Errors, in the reference's order: APG_ERR_EMPTY_BATCH
 * (k = 0), APG_ERR_SRS_TOO_SMALL (fewer than k*2^n powers),
 * APG_ERR_MIXED_COLUMN_SIZES. */
int apg_commit_stack(apg_ctx* ctx, const uint8_t* const* cols, const size_t* num_vars, size_t k, uint8_t out[64]);
/* As apg_commit_stack with the columns in device memory. */
int apg_commit_stack_device(apg_ctx* ctx, const void* const* d_cols, const size_t* num_vars, size_t k,
                            uint8_t out[64]);
/* pcs::commit of a narrow backing (column_msm, crates/pcs/src/lib.rs:280-298):
 * 2^num_vars unsigned values of `bits` bits (8, 16 or 32: little-endian
 * integers; 1: bit-packed in u64 limbs, value i at bit i % 64 of limb i / 64,
 * like PolyBacking::U1) committed through the small-scalar path, never lifted
 * to Fr; host memory. Errors as apg_commit. */
int apg_commit_narrow(apg_ctx* ctx, const void* vals, int bits, size_t num_vars, uint8_t out[64]);

/* ---- Mercury opening (crates/pcs/src/lib.rs) ----------------------------- */

/* pcs::open (lib.rs:313): open the commitment `cm` (64 bytes, absorbed as
 * passed) of the 2^num_vars evaluations `evals` (Fr in memory) at the point
 * u (u_len Fr in memory) over the resident SRS, on the transcript (226-byte
 * snapshot, in/out; left where the verifier leaves it, PAIRING_MERGE drawn).
 * Writes v = f(u) (Fr in memory) and the 704-byte MercuryProof::to_bytes.
 * Errors, in the reference's order: APG_ERR_UNSUPPORTED_NUM_VARS,
 * APG_ERR_POINT_LENGTH_MISMATCH (u_len != num_vars), APG_ERR_SRS_TOO_SMALL,
 * APG_ERR_DEGENERATE_CHALLENGE. */
int apg_mercury_open(apg_ctx* ctx, const uint8_t* evals, size_t num_vars, const uint8_t cm[64], const uint8_t* u,
                     size_t u_len, uint8_t* transcript, uint8_t v_out[32], uint8_t proof_out[704]);
/* pcs::batch_open (lib.rs:688, batch_open_stacked at r = []): k columns of one
 * size at one point; cols[j] points at column j (host, Fr in memory), cms is
 * k x 64 bytes. Writes each column's value (vs_out, k x 32, Fr in memory)
 * and the one proof of cm* = sum rho^i cm_i. Errors add APG_ERR_EMPTY_BATCH
 * (k = 0); the column and commitment lists share k. */
int apg_mercury_batch_open(apg_ctx* ctx, const uint8_t* const* cols, size_t k, size_t num_vars, const uint8_t* cms,
                           const uint8_t* u, size_t u_len, uint8_t* transcript, uint8_t* vs_out,
                           uint8_t proof_out[704]);
/* As apg_mercury_batch_open with the columns in device memory. */
int apg_mercury_batch_open_device(apg_ctx* ctx, const void* const* d_cols, size_t k, size_t num_vars,
                                  const uint8_t* cms, const uint8_t* u, size_t u_len, uint8_t* transcript,
                                  uint8_t* vs_out, uint8_t proof_out[704]);
/* pcs::batch_open_stacked (lib.rs:705-789), the prover's opening
 * (crates/prover/src/lib.rs:1076): n_stacks stacks, stack j's columns in its
 * first stack_lens[j] slots of a table over u || r (slot s = the r-variables'
 * bits). cols lists every stack's columns, stack after stack (host, Fr in
 * memory), num_vars each column's variable count; cms is n_cms x 64 bytes (the
 * stacks' commit_stack commitments). Writes each stack's value
 * v_j = sum_s eq(r, s) col_{j,s}(u) (vs_out, n_stacks x 32) and the proof of
 * cm* = sum rho^j cm_j at u || r. Errors, in the reference's order:
 * APG_ERR_EMPTY_BATCH (no stack, or an empty one), APG_ERR_BATCH_LENGTH_MISMATCH
 * (n_cms != n_stacks), APG_ERR_MIXED_COLUMN_SIZES,
 * APG_ERR_UNSUPPORTED_NUM_VARS (of width + r_len), APG_ERR_POINT_LENGTH_MISMATCH
 * (u_len != the columns' width), APG_ERR_BATCH_LENGTH_MISMATCH (a stack longer
 * than 2^r_len), APG_ERR_SRS_TOO_SMALL. */
int apg_mercury_batch_open_stacked(apg_ctx* ctx, const uint8_t* const* cols, const size_t* num_vars,
                                   const size_t* stack_lens, size_t n_stacks, const uint8_t* cms, size_t n_cms,
                                   const uint8_t* u, size_t u_len, const uint8_t* r, size_t r_len,
                                   uint8_t* transcript, uint8_t* vs_out, uint8_t proof_out[704]);
/* As apg_mercury_batch_open_stacked with the columns in device memory. */
int apg_mercury_batch_open_stacked_device(apg_ctx* ctx, const void* const* d_cols, const size_t* num_vars,
                                          const size_t* stack_lens, size_t n_stacks, const uint8_t* cms,
                                          size_t n_cms, const uint8_t* u, size_t u_len, const uint8_t* r,
                                          size_t r_len, uint8_t* transcript, uint8_t* vs_out,
                                          uint8_t proof_out[704]);

/* ---- zerocheck (crates/sumcheck/src/lib.rs) ------------------------------ */

/* sumcheck::verify_zerocheck (lib.rs:418): check a zerocheck proof of the
 * gate (terms as for apg_prove_zerocheck) over num_vars variables. Host only
 * (no context). rounds: n_rounds x 4 Fr in memory (ascending coefficients),
 * finals: n_finals Fr in memory, as apg_prove_zerocheck writes them. The
 * transcript (226-byte snapshot) must have been driven as the prover's was,
 * the witness digest included; it is advanced in place on success and left
 * unchanged on failure. point_out (num_vars Fr) receives SumcheckClaim::point
 * (its final_evals are the caller's finals). Errors in the reference's order:
 * APG_ERR_ROUND_COUNT_MISMATCH (*info = n_rounds), APG_ERR_FINAL_COUNT_MISMATCH
 * (*info = n_finals), APG_ERR_ROUND_SUM_MISMATCH (*info = the round),
 * APG_ERR_FINAL_EVAL_MISMATCH; a gate with no inputs or a term naming an
 * undeclared input is APG_ERR_INVALID_ARGUMENT (GateError). */
int apg_verify_zerocheck(size_t arity, const uint8_t* coefs, const uint32_t* a, const uint32_t* b, size_t nterms,
                         size_t num_vars, const uint8_t* rounds, size_t n_rounds, const uint8_t* finals,
                         size_t n_finals, uint8_t* transcript, uint8_t* point_out, uint64_t* info);
/* sumcheck::prove_zerocheck (lib.rs:359): prove that the gate
 *   G = sum_t coefs[t] * x_{a[t]} * x_{b[t]}   (b[t] = 0xffffffff: no 2nd factor)
 * over `arity` columns of 2^num_vars evaluations vanishes on the hypercube.
 * coefs and columns are Fr in memory; polys[k] points at column k (host).
 * The transcript (226-byte snapshot, in/out) must already hold the witness
 * digest. Writes num_vars rounds of 4 ascending coefficients (rounds_out,
 * num_vars x 128 bytes) and the columns' values at the bound point
 * (finals_out, arity x 32), both Fr in memory. The columns are not modified:
 * the reference's binding of them in place is the returned final values. */
int apg_prove_zerocheck(apg_ctx* ctx, size_t arity, const uint8_t* coefs, const uint32_t* a, const uint32_t* b,
                        size_t nterms, const uint8_t* const* polys, size_t num_vars, uint8_t* transcript,
                        uint8_t* rounds_out, uint8_t* finals_out);
/* As apg_prove_zerocheck with the columns in device memory. */
int apg_prove_zerocheck_device(apg_ctx* ctx, size_t arity, const uint8_t* coefs, const uint32_t* a,
                               const uint32_t* b, size_t nterms, const void* const* d_polys, size_t num_vars,
                               uint8_t* transcript, uint8_t* rounds_out, uint8_t* finals_out);
/* As apg_prove_zerocheck with each column in its stored width (bits[k] as in
 * apg_gkr_forward_narrow: 1 a bitset in u64 limbs, 8/16/32 unsigned integers,
 * 0 Fr in memory), host or device (polys_on_device) pointers. Narrow columns
 * cross and stay narrow: the first two rounds read them through the lift and
 * the first bind writes Fr (MultilinearPoly::bind, crates/poly/src/lib.rs:156-185). */
int apg_prove_zerocheck_narrow(apg_ctx* ctx, size_t arity, const uint8_t* coefs, const uint32_t* a,
                               const uint32_t* b, size_t nterms, const void* const* polys, const uint8_t* bits,
                               int polys_on_device, size_t num_vars, uint8_t* transcript, uint8_t* rounds_out,
                               uint8_t* finals_out);
/* sumcheck::witness_digest (lib.rs:228-256): the Poseidon2 sponge over the
 * column count, the variable count and every cell, squeezed once. Columns
 * are host Fr in memory; out is Fr in memory. Inherently sequential. */
int apg_witness_digest(apg_ctx* ctx, const uint8_t* const* cols, size_t k, size_t num_vars, uint8_t out[32]);

/* ---- GKR (crates/gkr/src/lib.rs) ----------------------------------------- */

/* A circuit crosses the boundary as an "APGC" blob: the resolved form of a
 * constraints::CircuitArtifact (crates/constraints/src/lib.rs:549-672) that
 * the prover reads, all integers u32 little-endian, literals 32-byte
 * canonical Fr:
 *   'APGC'(0x43475041) version(1) trace_vars n_committed
 *   n_virtuals kind[n_virtuals]        (0 RowIndex, 1 RamLive, 2 Range19,
 *                                       3 Range16, 4 Xor8A, 5 Xor8B, 6 Xor8Out)
 *   n_outputs offset[n_outputs]        (top-layer columns, output-map order)
 *   depth, then per gate list k:
 *     halving num_vars(k+1) width(k+1) n_cached n_producing n_enforcing
 *     gates (cached, producing, enforcing), each:
 *       kind (0 Linear 1 Product 2 MaskIntoIdentity 3 AffineProduct
 *             4 TreeProduct 5 TreeCross 6 Quadratic) p1 p2 (Linear t; Affine
 *             t, u; Quadratic t, u; else 0)
 *       n_operands, (source, index)*  source 0 = column of layer k (layout
 *             order M, W, S at k = 0), 1 = virtual table, 2 = cached entry
 *       n_coeffs, (is_challenge, slot | Fr)*  in GateDef::coefficients order
 * Operand and coefficient orders are GateDef::operands / coefficients
 * (crates/constraints/src/lib.rs:375-421). Malformed blobs return
 * APG_ERR_BAD_CIRCUIT before any device work. */
typedef struct apg_gkr_values apg_gkr_values;

/* gkr::forward (lib.rs:279): materialise every layer on the device. base
 * holds n_committed host column pointers (Fr in memory, 2^trace_vars each);
 * the external challenges are slots[i] -> slot_values[i] (Fr in memory). The
 * values stay resident until apg_gkr_values_free. */
int apg_gkr_forward(apg_ctx* ctx, const uint8_t* circuit, size_t circuit_len, const uint8_t* const* base,
                    const uint32_t* slots, const uint8_t* slot_values, size_t n_slots, apg_gkr_values** out);
/* Read column `col` of layer `layer` (0 = base) into out (Fr in memory). */
int apg_gkr_values_read(apg_gkr_values* values, size_t layer, size_t col, uint8_t* out);
/* Entries per column of layer `layer`. */
size_t apg_gkr_values_len(apg_gkr_values* values, size_t layer);
/* Free forward's values; call it before destroying their context. */
void apg_gkr_values_free(apg_gkr_values* values);
/* Bytes of the proof apg_gkr_prove writes for this circuit (0 if malformed). */
size_t apg_gkr_proof_len(const uint8_t* circuit, size_t circuit_len);
/* gkr::prove (lib.rs:933): the backward pass over forward's values, on a
 * transcript the caller has bound to the base (226-byte snapshot, in/out).
 * The proof (GkrProof, crates/gkr-verify/src/lib.rs:90-92) is written as, for
 * each gate list k = 0 .. depth-1, its rounds (4 Fr each) then its claims,
 * all Fr in memory. point_out (nullable, trace_vars x 32 bytes) receives the
 * base layer's point, the one crates/prover's replay_point re-derives
 * (crates/prover/src/lib.rs:1111-1140) and the openings use. */
int apg_gkr_prove(apg_ctx* ctx, const uint8_t* circuit, size_t circuit_len, apg_gkr_values* values,
                  const uint32_t* slots, const uint8_t* slot_values, size_t n_slots, uint8_t* transcript,
                  uint8_t* proof_out, size_t proof_cap, size_t* proof_len, uint8_t* point_out);
/* gkr_verify::verify (crates/gkr-verify/src/lib.rs:647): reduce the output
 * claims to claims about the committed base columns, or reject. Host only
 * (no context, no device work).
 *   outputs:   n_outputs tables in the circuit's output-map order, table i
 *              output_lens[i] Fr in memory (2^top_vars each);
 *   proof:     as apg_gkr_prove writes it (proof_len bytes);
 *   slots / slot_values: the external challenges (Fr in memory);
 *   transcript: 226-byte snapshot bound to the base as the prover's was;
 *              advanced in place on success, left unchanged on failure.
 * Out: point_out (trace_vars Fr) and values_out (n_committed Fr): the base
 * claims (BaseClaim, one per committed column, all at one point).
 * Checks in the reference's order: APG_ERR_MISSING_CHALLENGE (*info = the
 * first missing slot, lists bottom up), APG_ERR_OUTPUT_SHAPE,
 * APG_ERR_PROOF_SHAPE (*info = the first gate list whose rounds and claims
 * do not fit in proof_len, or depth when bytes are left over),
 * APG_ERR_LAYER_INCONSISTENCY (*info = the gate list whose round or final
 * check failed). info is nullable. As in the reference, the enforcing gates'
 * claims are zero: a circuit whose enforcing gates do not vanish is
 * rejected. */
int apg_gkr_verify(const uint8_t* circuit, size_t circuit_len, const uint8_t* const* outputs,
                   const size_t* output_lens, size_t n_outputs, const uint8_t* proof, size_t proof_len,
                   const uint32_t* slots, const uint8_t* slot_values, size_t n_slots, uint8_t* transcript,
                   uint8_t* point_out, uint8_t* values_out, uint64_t* info);
/* gkr::prove_sumcheck (crates/gkr/src/lib.rs:792): one gate list's sumcheck
 * of claim = sum_y eq(eq_point, y) S(y), S = sum_j weights[j] gate_j over the
 * list's producing then enforcing gates (with the challenges of `slots`),
 * one cubic per variable absorbed as SUMCHECK_ROUND and followed by its
 * SUMCHECK_CHALLENGE on the caller's transcript (226-byte snapshot, in/out).
 *   layer:    the gate list's index in the circuit blob;
 *   weights:  n_weights Fr in memory, one per producing and enforcing gate;
 *   eq_point: num_vars Fr in memory, num_vars = the variables of the list's
 *             output (its rows' log, one less than its input's for a
 *             halving list);
 *   d_lower:  width device pointers to 2^num_vars Fr each, the list's input
 *             columns (child 0 of each column for a halving list);
 *   d_upper:  for a halving list, width device pointers to child 1 of each
 *             column (ignored otherwise);
 * Out: rounds_out 4 x num_vars Fr (ascending coefficients), point_out
 * num_vars Fr (the bound point), finals_out the tables bound to that point
 * (width Fr, then width more for a halving list). The caller's tables are
 * read, not bound in place (the reference binds its tables; their bound
 * values are finals_out). Virtual tables are evaluated in closed form, as in
 * the reference. */
int apg_gkr_prove_sumcheck(apg_ctx* ctx, const uint8_t* circuit, size_t circuit_len, size_t layer,
                           const uint8_t* weights, size_t n_weights, const uint32_t* slots, const uint8_t* slot_values,
                           size_t n_slots, const uint8_t* eq_point, size_t num_vars, const void* const* d_lower,
                           const void* const* d_upper, size_t width, uint8_t* transcript, uint8_t* rounds_out,
                           uint8_t* point_out, uint8_t* finals_out);
/* As apg_gkr_forward with the base columns already in device memory. */
int apg_gkr_forward_device(apg_ctx* ctx, const uint8_t* circuit, size_t circuit_len, const void* const* d_base,
                           const uint32_t* slots, const uint8_t* slot_values, size_t n_slots, apg_gkr_values** out);
/* As apg_gkr_forward with every committed column in its stored width, the
 * PolyBacking variants of crates/poly/src/lib.rs:44-57: bits[x] = 1 (a bitset,
 * ceil(2^n / 64) u64 limbs, entry i = bit i % 64 of limb i / 64), 8, 16 or 32
 * (unsigned integers, one per entry) or 0 (Fr in memory). base_on_device: the
 * columns are device pointers. The columns stay in their widths on the device:
 * the forward pass and the first two sumcheck rounds of gate list 0 read them
 * through the lift (PolyBacking::entry, :72-88), and that sumcheck's first
 * bind writes Fr, so no full-size Fr copy of a narrow column is made (the lazy
 * lift of MultilinearPoly::bind, :156-185). apg_gkr_prove and
 * apg_gkr_values_read take the handle as from apg_gkr_forward. A width other
 * than 0, 1, 8, 16, 32 is APG_ERR_INVALID_ARGUMENT. */
int apg_gkr_forward_narrow(apg_ctx* ctx, const uint8_t* circuit, size_t circuit_len, const void* const* base,
                           const uint8_t* bits, int base_on_device, const uint32_t* slots,
                           const uint8_t* slot_values, size_t n_slots, apg_gkr_values** out);

/* ---- shard proofs (crates/prover/src/lib.rs:798-1102) -------------------- */

/* One shard's hot path, the slice of prove_shard_columns that this library
 * replaces: commit every column (commit_all, lib.rs:444-471), seed the shard
 * transcript (verifier_core::shard_transcript, crates/verifier-core/src/
 * statement.rs:548-572: SHARD_SEED [statement digest, family, index],
 * SHARD_TS_WINDOW [ts_lo, ts_hi], the commitments as one G1 list under
 * COMMITMENT, then the lookup challenges g and beta under LOOKUP_CHALLENGE,
 * which the circuit reads as external challenge slots 0 and 1), run
 * gkr::forward and gkr::prove (gkr_part, lib.rs:850,943) and open every column
 * at the base point the proof leaves (opening_part -> batch_open_stacked at
 * r = [], lib.rs:1076). */
typedef struct apg_shard {
  const uint8_t* circuit;           /* APGC blob of the shard's circuit */
  size_t circuit_len;
  const void* const* cols;          /* n_cols columns, Fr in memory, 2^num_vars each */
  size_t n_cols;
  int cols_on_device;               /* 1: device pointers on the context's device */
  size_t num_vars;                  /* even, 2..30 */
  const uint8_t* statement_digest;  /* 32 bytes, Fr in memory */
  uint32_t family, index;           /* the shard's family and index (u32 in the reference) */
  uint64_t ts_lo, ts_hi;            /* its timestamp window */
  /* The challenge slots the circuit reads besides the ones the shard draws
   * itself (verifier_core::shard_challenges,
   * crates/verifier-core/src/statement.rs:616-635): n_ext (slot, value)
   * pairs, values 32 bytes each (Fr in memory), for the statement's memory
   * challenges (slots 1-4) and a window shard's constant (slot 5). The shard
   * draws g and beta from its own transcript and sets slot 6 = g, slots 7-12
   * = beta^1..beta^6 and, for a circuit with a decoder channel, slot 13 =
   * g - sum_{j<W} beta^j (gkr_verify::insert_lookup_challenges,
   * crates/gkr-verify/src/lookup.rs:28-61); slot 0, the test circuits' one
   * challenge (read by no production circuit), is g as well. An external
   * pair naming one of those slots, or a slot twice, is refused
   * (APG_ERR_INVALID_ARGUMENT). The arrays must stay valid until the proof
   * is done. */
  const uint32_t* ext_slots;
  const uint8_t* ext_values;
  size_t n_ext;
  uint32_t decoder_width;           /* W: the decoder lookup tuple's width, 0..7 (0: no decoder channel) */
} apg_shard;

/* Where a shard proof lands (caller-owned buffers, filled when it is done). */
typedef struct apg_shard_proof {
  uint8_t* cms;         /* n_cols x 64: the commitments */
  uint8_t* gkr_proof;   /* apg_gkr_proof_len(circuit) bytes: the GKR proof (Fr in memory) */
  size_t gkr_cap;
  size_t gkr_len;       /* out */
  uint8_t* point;       /* num_vars x 32: the base point (Fr in memory) */
  uint8_t* values;      /* n_cols x 32: the columns at the point (Fr in memory) */
  uint8_t opening[704]; /* the batched Mercury opening */
  uint8_t transcript[226];
  double phase_ms[4];   /* out: commit, forward, GKR proof, opening (host wall clock) */
} apg_shard_proof;

/* No reference counterpart: sizeof of the structs this header declares,
 * for bindings to check their layouts against: apg_shard, apg_shard_proof,
 * apg_request_times, apg_server_stats, apg_server_config, in that order.
 * Writes min(n, 5) sizes; returns 5. */
size_t apg_abi_sizes(size_t* out, size_t n);

/* Prove one shard on the context (columns on its device or host). */
int apg_prove_shard(apg_ctx* ctx, const apg_shard* shard, apg_shard_proof* out);
/* No reference counterpart: an estimate of the device bytes proving `shard`
 * holds at its peak on a context that holds nothing yet (staged columns, GKR
 * layers, the largest sumcheck's levels, both commit lanes' MSM scratch, the
 * opening's tables); 0 for a malformed circuit. The server admits by it. */
size_t apg_shard_device_bytes(const apg_shard* shard);
/* No reference counterpart: the device bytes the context (and its second
 * lane) holds in scratch, window tables it owns and its SRS if owned. */
size_t apg_ctx_device_bytes(apg_ctx* ctx);

/* ---- the shard-proof server (no reference counterpart) ------------------
 *
 * Continuous batching of shard proofs on one GPU: requests are queued as they
 * are submitted and admitted in arrival order as soon as a worker (a context
 * with its own stream and scratch, sharing the owner's SRS, window tables and
 * tuned widths) is idle or can be added, and the request's device bytes fit
 * the measured free HBM (cudaMemGetInfo plus what the stream-ordered pool
 * holds unused, minus the growth reserved for requests already admitted and
 * `hbm_reserve`) and the budget (`hbm_budget`, 0 = none: the workers' held
 * bytes plus reservations stay below it). Admitted requests run concurrently,
 * each on its own worker's stream, so their kernels overlap on the device; a
 * request keeps its columns, layer values, buckets and transcript state on
 * its worker until it completes. Workers are added as memory admits, up to
 * `max_workers` (0 = no cap beyond memory). Results are byte for byte those
 * of apg_prove_shard on the same request. Build the owner's window tables
 * (apg_srs_prepare, apg_msm_autotune) before creating the server: workers
 * borrow the tables the owner holds then. */
typedef struct apg_server apg_server;
typedef struct apg_server_config {
  size_t hbm_budget;  /* bytes; 0 = no budget beyond free HBM */
  size_t hbm_reserve; /* free bytes never handed to a request */
  int max_workers;    /* 0 = no cap */
  int timing;         /* 1: time every worker's kernels and host round steps (apg_server_query) */
} apg_server_config;
/* Per-request timestamps, nanoseconds since the server started, and what the
 * request reserved. */
typedef struct apg_request_times {
  uint64_t submit_ns, admit_ns, start_ns, done_ns;
  uint64_t reserved_bytes;
  int worker;
  double phase_ms[4];
} apg_request_times;
typedef struct apg_server_stats {
  uint64_t submitted, completed, failed, queued, in_flight;
  uint64_t workers, peak_workers, peak_in_flight;
  uint64_t held_bytes, reserved_bytes;
  double kernel_ms;     /* with timing: the sum of every worker kernel's duration */
  double host_round_ms; /* with timing: host time between sumcheck rounds, all workers */
} apg_server_stats;

/* A server whose workers share `owner`'s SRS and tables (`owner` must outlive
 * it and not replace its SRS meanwhile). */
int apg_server_create(apg_ctx* owner, const apg_server_config* cfg, apg_server** out);
/* Finish every admitted and queued request, then release the workers. */
void apg_server_destroy(apg_server* server);
/* Queue a request; `shard`'s arrays and `out`'s buffers must stay valid until
 * the request completes (host columns are copied to the device when the
 * request runs). Writes a ticket. */
int apg_submit(apg_server* server, const apg_shard* shard, apg_shard_proof* out, uint64_t* ticket);
/* APG_PENDING while the request is queued or running; APG_OK once its proof
 * is in `out`; else the request's failure status. times (nullable). */
int apg_poll(apg_server* server, uint64_t ticket, apg_request_times* times);
/* As apg_poll, blocking until the request is done. */
int apg_wait(apg_server* server, uint64_t ticket, apg_request_times* times);
/* Counters and held bytes of the server now. */
int apg_server_query(apg_server* server, apg_server_stats* out);

/* ---- deferred-pairing accumulator (crates/pcs/src/accumulator.rs) ------- */

/* pcs::verify_deferred (crates/pcs/src/lib.rs:632): every field-side check
 * of a Mercury verification and every point check, stopping before the
 * pairing. Host only (no context). cm: 64 bytes; u: u_len Fr in memory;
 * v: Fr in memory; proof: the 704-byte MercuryProof::to_bytes; the
 * transcript (226-byte snapshot) as the prover's was before its opening,
 * advanced in place on success, left unchanged on failure. Out: the twelve
 * AccumulatorEntry values of one deferred check (ENTRIES_PER_CHECK,
 * crates/pcs-verify/src/lib.rs:271-284) in apg_discharge_msms's form:
 * sides_out[12] (0 G2One, 1 G2X), scalars_out 12 Fr in memory, points_out
 * 12 canonical 64-byte points. Errors in the reference's order:
 * APG_ERR_UNSUPPORTED_NUM_VARS, APG_ERR_INVALID_POINT (*info = 0..7 the
 * proof's points h, q, g, s, d, pi_z, w, w', 8 the commitment),
 * APG_ERR_NONCANONICAL (a proof value), APG_ERR_DEGENERATE_CHALLENGE. */
int apg_mercury_verify_deferred(const uint8_t cm[64], const uint8_t* u, size_t u_len, const uint8_t v[32],
                                const uint8_t proof[704], uint8_t* transcript, uint8_t sides_out[12],
                                uint8_t* scalars_out, uint8_t* points_out, uint64_t* info);
/* pcs::batch_verify_deferred (lib.rs:661): k commitments (k x 64 bytes,
 * absorbed as passed) claimed to open to vs (n_vs Fr in memory) at u; the
 * preamble draws rho, cm* = sum rho^i cm_i is summed on the host and the
 * single-instance core runs on (cm*, u, v*). Errors add, first,
 * APG_ERR_EMPTY_BATCH and APG_ERR_BATCH_LENGTH_MISMATCH (check_batch), and a
 * commitment off the curve is APG_ERR_INVALID_POINT with *info = 8. */
int apg_mercury_batch_verify_deferred(const uint8_t* cms, size_t k, const uint8_t* u, size_t u_len,
                                      const uint8_t* vs, size_t n_vs, const uint8_t proof[704], uint8_t* transcript,
                                      uint8_t sides_out[12], uint8_t* scalars_out, uint8_t* points_out,
                                      uint64_t* info);
/* ---- the pairing and the full verifications (host) ----------------------- */

/* curve::pairing::pairing (crates/curve/src/pairing.rs): the optimal ate
 * pairing e(P, Q) = f_{6x+2,Q}(P)^((q^12 - 1)/r) of a canonical G1 point (64
 * bytes) and a canonical G2 point (128 bytes: x.c0 || x.c1 || y.c0 || y.c1),
 * written as the Fq12 c0 || c1 (each Fq6 c0 || c1 || c2, each Fq2 c0 || c1,
 * canonical Fq): 384 bytes. A point off its curve, a G2 point outside the
 * order-r subgroup or a coordinate >= q is APG_ERR_INVALID_POINT. */
int apg_pairing(const uint8_t p[64], const uint8_t q[128], uint8_t out[384]);
/* k Q for a canonical G2 point Q (G2Projective * k, crates/curve/src/g2.rs),
 * k 32 bytes little-endian (any 256-bit integer), the result canonical. */
int apg_g2_mul(const uint8_t q[128], const uint8_t k[32], uint8_t out[128]);
/* curve::pairing::pairing_check: prod_i e(P_i, Q_i) == 1 into *holds (1/0),
 * n pairs as n x 64 and n x 128 bytes; points validated as for apg_pairing. */
int apg_pairing_check(const uint8_t* ps, const uint8_t* qs, size_t n, int* holds);
/* pcs::verify (crates/pcs/src/lib.rs:614): apg_mercury_verify_deferred, then
 * its pairing over the SrsVerifier's wire form vsrs (320 bytes, [1]_1 ||
 * [1]_2 || [x]_2, crates/srs/src/lib.rs:279-290). APG_OK, its errors, or
 * APG_ERR_VERIFICATION_FAILED; the transcript advances only on APG_OK. */
int apg_mercury_verify(const uint8_t vsrs[320], const uint8_t cm[64], const uint8_t* u, size_t u_len,
                       const uint8_t v[32], const uint8_t proof[704], uint8_t* transcript, uint64_t* info);
/* pcs::batch_verify (lib.rs:648): as apg_mercury_verify over a batch. */
int apg_mercury_batch_verify(const uint8_t vsrs[320], const uint8_t* cms, size_t k, const uint8_t* u, size_t u_len,
                             const uint8_t* vs, size_t n_vs, const uint8_t proof[704], uint8_t* transcript,
                             uint64_t* info);
/* pcs::discharge (crates/pcs/src/accumulator.rs:146): apg_discharge_msms on
 * the device, then the pairing e(A, [1]_2) e(-B, [x]_2) == 1 on the host.
 * APG_OK, the MSMs' errors, or APG_ERR_VERIFICATION_FAILED. */
int apg_discharge(apg_ctx* ctx, const uint8_t vsrs[320], const uint8_t* sides, const uint8_t* scalars,
                  const uint8_t* points, size_t n, const size_t* checks, size_t n_checks);

/* The group side of pcs::discharge (crates/pcs/src/accumulator.rs:146-163),
 * everything before its pairing. The accumulator is n entries (the fields of
 * AccumulatorEntry, :37-42): sides[i] 0 = PairingSide::G2One, 1 = G2X;
 * scalars as n Fr in memory; points as n canonical 64-byte G1 encodings
 * (all zero = infinity); grouped into deferred checks by the counts
 * checks[0..n_checks). Every point is validated (APG_ERR_INVALID_POINT),
 * then the counts must partition the entries (APG_ERR_MALFORMED_ACCUMULATOR);
 * the merge challenge nu is drawn from the digest of the accumulator's words
 * (pcs-verify/src/lib.rs:315-319) and
 *   A = sum_j nu^j sum_{G2One entries of check j} s_i P_i,  B likewise over G2X,
 * are returned as canonical points; nu_out (nullable) receives nu (Fr in
 * memory). The caller's pairing check is e(A, [1]_2) * e(-B, [x]_2) == 1.
 * A side other than 0/1 is APG_ERR_INVALID_ARGUMENT, an unreduced scalar
 * APG_ERR_NONCANONICAL (neither can come from the reference's types). */
int apg_discharge_msms(apg_ctx* ctx, const uint8_t* sides, const uint8_t* scalars, const uint8_t* points, size_t n,
                       const size_t* checks, size_t n_checks, uint8_t a_out[64], uint8_t b_out[64],
                       uint8_t nu_out[32]);
/* The MSMs of check_pairings (accumulator.rs:171-214) with the caller's
 * weights, one Fr (in memory) a check: verify and batch_verify reach it with
 * one check of weight one. The partition is checked first, then the points. */
int apg_pairing_msms(apg_ctx* ctx, const uint8_t* sides, const uint8_t* scalars, const uint8_t* points, size_t n,
                     const size_t* checks, const uint8_t* weights, size_t n_checks, uint8_t a_out[64],
                     uint8_t b_out[64]);

/* ---- transcript (crates/transcript/src/lib.rs:214-346) ------------------- */

/* A fresh transcript snapshot (Transcript::new). */
void apg_transcript_init(uint8_t snapshot[226]);
/* Transcript::append_scalars(tag, xs): xs are n Fr in memory. */
int apg_transcript_append_scalars(uint8_t snapshot[226], uint64_t tag, const uint8_t* xs, size_t n);
/* Transcript::challenge_scalar(tag) -> out (Fr in memory). */
int apg_transcript_challenge(uint8_t snapshot[226], uint64_t tag, uint8_t out[32]);
/* Transcript::observe (lib.rs:241-251): one Fr (in memory) into the rate. */
int apg_transcript_observe(uint8_t snapshot[226], const uint8_t x[32]);
/* Transcript::sample (lib.rs:253-263): one raw squeeze -> out (Fr in memory). */
int apg_transcript_sample(uint8_t snapshot[226], uint8_t out[32]);
/* Transcript::append_bytes (lib.rs:324-338): tag, byte length, then 31-byte
 * little-endian limbs. */
int apg_transcript_append_bytes(uint8_t snapshot[226], uint64_t tag, const uint8_t* bytes, size_t len);
/* transcript::io_digest (lib.rs:464-475): the public I/O digest -> out (Fr in
 * memory). */
int apg_io_digest(const uint8_t* input, size_t input_len, const uint8_t* output, size_t output_len,
                  uint8_t out[32]);
/* poseidon2_permute (lib.rs:121-146) over three canonical little-endian Fr,
 * in place; APG_ERR_NONCANONICAL if one is >= p. */
int apg_poseidon2_permute(uint8_t state[96]);

/* ---- utilities ---------------------------------------------------------- */

/* Canonical Fr values in device memory -> Montgomery (in-memory) form, in
 * place; APG_ERR_NONCANONICAL if any value is >= p. */
int apg_fr_to_mont_device(apg_ctx* ctx, void* d_vals, size_t n);
/* Seeded benchmark input, not a reference interface: n canonical Fr (eight
 * little-endian u32 words each) written to device memory from the ChaCha20
 * keystream keyed by `seed`, the generator the reference's bench tool draws
 * its inputs from (tools/bench/src/timing.rs:56-67 for the Fr rule: 32 bytes,
 * top two bits cleared, rejected while >= r or zero). kind 0: trace-like
 * (25% {0,1}, 60% u32, 15% uniform Fr); kind 1: uniform Fr. n <= 2^32. */
int apg_synth_column(apg_ctx* ctx, uint64_t seed, int kind, size_t n, void* d_out);
/* Kernels this context has launched since it was created. */
uint64_t apg_ctx_launch_count(apg_ctx* ctx);

/* Per-kernel device timing with CUDA events on the context's stream. */
enum apg_timer {
  APG_TIMER_MSM_ACCUMULATE = 0, /* bucket accumulation kernel */
  APG_TIMER_MSM_TOTAL = 1,      /* one whole MSM, recode to normalisation */
  APG_TIMER_SUMCHECK_ROUND = 2, /* sumcheck evaluate+fold kernel */
  APG_TIMER_GKR_FORWARD = 3,    /* GKR forward layer kernel */
  APG_TIMER_MERCURY_PASS = 4,   /* Mercury O(n) field passes */
  APG_TIMER_KERNELS = 5,        /* every kernel launch (timing mode 2 only) */
  APG_TIMER_HOST_ROUND = 6      /* host time between a sumcheck round's sums and the next round's launch */
};
/* Enable (1) or disable (0) timers; enabling clears accumulated totals. Mode
 * 2 also brackets every kernel launch with events (APG_TIMER_KERNELS: the
 * device's busy time on the context's streams), at a small cost a launch. */
int apg_ctx_set_timing(apg_ctx* ctx, int on);
/* Total milliseconds and launch count recorded under `timer` so far. */
int apg_ctx_timer(apg_ctx* ctx, int timer, double* ms, uint64_t* launches);
/* Measure this device's Montgomery-multiply throughput: a dependency-free
 * stream of Fq products over every SM for about `ms` milliseconds. Writes
 * Fq multiplications per second. */
int apg_probe_fq_mul_rate(apg_ctx* ctx, double ms, double* fq_mul_per_s);

#ifdef __cplusplus
}
#endif

#endif /* APOGEE_GPU_H */
