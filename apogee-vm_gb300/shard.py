"""Shard proving over the C ABI, and the shard workloads the benchmark runs.

`prove_shard` (the library's apg_prove_shard) is the hot-path slice of
crates/prover's prove_shard_columns
(crates/prover/src/lib.rs:798-1102): commit every column (commit_all), seed the
shard transcript and absorb the commitments, run the GKR forward and backward
passes, and open every column at the base point GKR leaves with one batched
Mercury opening (opening_part -> batch_open_stacked at r = []).

Workloads:
  * `shard_mix`: 207 shards over 23 circuit families, sizes log-uniform over
    the even heights 2^8 .. 2^22 (Mercury takes even variable counts only),
    4 to 16 columns each, values drawn like VM trace columns.
  * `family_mix`: 207 shards over 23 families proved with the reference's
    own family circuits (its committed artifacts, decoded), the 13 artifacts
    cycled over the families, each shard committing every column its
    circuit's base layer reads (28 to 96).
  * `prove_sequential`: one shard at a time on one context (the plain path).
  * `prove_batched`: every shard submitted at once to the library's server
    (apg_server, continuous batching with admission by measured free HBM),
    largest first.
  * `serve`: a seeded Poisson stream of shard requests submitted to the
    server as they arrive; latency is completion minus arrival.
"""
import math
import random
import time

import apogee_gpu as A
import circuits as C
import synth

TAG_COMMITMENT = 3
TAG_SHARD_SEED = 39
SIZES = [8, 10, 12, 14, 16, 18, 20, 22]
FAMILIES = 23


def g1_limbs(p: bytes):
    """The transcript's four 128-bit limbs of a canonical G1 encoding;
    infinity absorbs 2^128 in each (crates/transcript/src/lib.rs:493-510)."""
    if p == bytes(64):
        return [1 << 128] * 4
    return [int.from_bytes(p[16 * k:16 * k + 16], "little") for k in range(4)]


def shard_mix(count: int = 207, seed: int = 20260903):
    rng = random.Random(seed)
    return [{"index": i, "family": i % FAMILIES, "log_rows": rng.choice(SIZES), "cols": rng.randint(4, 16)}
            for i in range(count)]


_circuits = {}


def shard_circuit(log_rows: int, cols: int) -> bytes:
    """List 0: row-wise degree-2 gates over the committed columns with a
    cached row-index term and one enforcing gate; then one halving
    TreeProduct list per variable down to a one-row top."""
    key = (log_rows, cols)
    if key not in _circuits:
        c = C.Circuit(log_rows, cols, [C.V_ROW])
        cac = [C.linear([(("ch", 0), C.col(0)), (1, C.virt(0))], 0)]
        prod = []
        for j in range(cols):
            a, b = C.col(j), C.col((j + 1) % cols)
            kind = j % 4
            if kind == 0:
                prod.append(C.product(3, a, b))
            elif kind == 1:
                prod.append(C.affine([(1, a), (2, C.cached(0))], 5, [(1, b)], 7))
            elif kind == 2:
                prod.append(C.mask(a, b))
            else:
                prod.append(C.quadratic(1, [(4, a)], [(("ch", 0), b, C.cached(0))]))
        enf = [C.quadratic(0, [(1, C.col(0)), (C.P_R - 1, C.col(1 % cols))], [(1, C.col(0), C.col(1 % cols))])]
        c.add_layer(prod, cached=cac, enforcing=enf)
        for _ in range(log_rows):
            c.add_layer([C.tree_product(C.col(j)) for j in range(cols)], halving=True)
        _circuits[key] = c.to_blob()
    return _circuits[key]


def device_columns(torch, n: int, k: int, seed: int, device: str, ctx):
    """k columns of n Fr on the device (Montgomery), mixed like VM traces
    (25% in {0,1}, 60% uniform u32, 15% uniform Fr), generated by the
    library from the ChaCha20 keystream of seed (seed << 16) + j for column
    j: the same values synth.mixed_column gives on the host."""
    cols = []
    for j in range(k):
        flat = synth.device_column(ctx, torch, n, (seed << 16) + j, "mixed", device)
        ctx.fr_to_mont_device(flat.data_ptr(), n)
        cols.append(flat)
    return cols


TAG_SHARD_TS_WINDOW = 40
TAG_LOOKUP_CHALLENGE = 33


def statement_digest(spec) -> int:
    """A stand-in for the statement digest a shard transcript is seeded with
    (the global phase's output, not part of the hot path): seeded per shard."""
    return random.Random(0x5EED0000 + spec["index"]).randrange(C.P_R)


def shard_transcript(spec, cms):
    """verifier_core::shard_transcript (crates/verifier-core/src/statement.rs:
    548-572): SHARD_SEED [digest, family, index], SHARD_TS_WINDOW [lo, hi],
    the witness commitments as one G1 list under COMMITMENT, then g and beta
    under LOOKUP_CHALLENGE. Returns the transcript snapshot, g and beta."""
    tr = A.transcript_append_scalars(A.transcript_init(), TAG_SHARD_SEED,
                                     [statement_digest(spec), spec["family"], spec["index"]])
    lo = spec["index"] << 22
    tr = A.transcript_append_scalars(tr, TAG_SHARD_TS_WINDOW, [lo, lo + (1 << spec["log_rows"])])
    limbs = []
    for cm in cms:
        limbs += g1_limbs(cm)
    tr = A.transcript_append_scalars(tr, TAG_COMMITMENT, limbs)
    tr, g = A.transcript_challenge(tr, TAG_LOOKUP_CHALLENGE)
    tr, beta = A.transcript_challenge(tr, TAG_LOOKUP_CHALLENGE)
    return tr, g, beta


# The 13 production family circuits among the reference's committed
# artifacts (crates/constraints/tests/vectors/*.bin; the toy circuits left out).
FAMILY_ARTIFACTS = ["add_sub", "atomics", "image_window", "jump_branch_slt", "mem_subword", "mem_word",
                    "memory_frame_alu", "memory_frame_atomics", "memory_frame_mem", "memory_frame_reg", "mul_div",
                    "shift_bitwise", "zero_window"]
DECODER_CHANNEL = 3  # constants::lookup_channel::DECODER
_families = {}


def family_circuit(artifact_dir: str, name: str, log_rows: int):
    """A family artifact over 2^log_rows rows: (APGC blob, committed columns,
    decoder tuple width)."""
    import os

    import artifact

    key = (artifact_dir, name, log_rows)
    if key not in _families:
        with open(os.path.join(artifact_dir, name + ".bin"), "rb") as f:
            art = artifact.decode(f.read())
        circ = artifact.to_circuit(art, log_rows)
        width = max([len(lk[3]) for lk in art["lookups"] if lk[1] == DECODER_CHANNEL] or [0])
        _families[key] = (circ.to_blob(), circ.n_committed, width)
    return _families[key]


def statement_challenges(seed: int = 0x57A7E):
    """Stand-ins for the statement-level challenge slots a family circuit
    reads (the memory challenges gamma_M, alpha_addr, alpha_ts, alpha_val in
    slots 1-4, drawn once per statement by the global phase, and a window
    shard's constant in slot 5): seeded, one set for the whole statement."""
    rng = random.Random(seed)
    return {slot: rng.randrange(C.P_R) for slot in (1, 2, 3, 4, 5)}


def shard_challenges(g: int, beta: int, decoder_width: int = 0, ext=None):
    """Every challenge slot the shard prover sets: the caller's statement
    slots, slot 0 (the test circuits' one challenge) and slot 6 = g, slots
    7-12 = beta^1..beta^6, and slot 13 = g - sum_{j<W} beta^j for a decoder
    channel of width W (gkr_verify::insert_lookup_challenges,
    crates/gkr-verify/src/lookup.rs:28-61)."""
    p = C.P_R
    ch = dict(ext or {})
    ch[0] = g
    ch[6] = g
    for j in range(6):
        ch[7 + j] = pow(beta, j + 1, p)
    if decoder_width:
        ch[13] = (g - sum(pow(beta, j, p) for j in range(decoder_width))) % p
    return ch


def family_mix(count: int = 207, seed: int = 20261204, sizes=(8, 10, 12, 14, 16)):
    """`count` shards over 23 families, family f proved with artifact
    FAMILY_ARTIFACTS[f % 13], sizes drawn uniformly from `sizes` (log2 of
    the rows); `cols` is filled in from the circuit when it is built."""
    rng = random.Random(seed)
    return [{"index": i, "family": i % FAMILIES, "log_rows": rng.choice(sizes),
             "artifact": FAMILY_ARTIFACTS[(i % FAMILIES) % len(FAMILY_ARTIFACTS)]} for i in range(count)]


def spec_circuit(spec, artifact_dir=None):
    """(blob, decoder width, statement challenges) of a spec: its family
    artifact when it names one, else the synthetic shard circuit."""
    if spec.get("artifact"):
        blob, ncols, width = family_circuit(artifact_dir, spec["artifact"], spec["log_rows"])
        spec.setdefault("cols", ncols)
        return blob, width, statement_challenges()
    return shard_circuit(spec["log_rows"], spec["cols"]), 0, None


def make_shard(spec, cols, blob=None, artifact_dir=None):
    """The library's shard request for `spec` over device columns `cols`:
    its circuit (the spec's family artifact, else the synthetic shard circuit,
    unless `blob` is given), the statement-level challenges a family circuit
    reads, and its transcript seed (statement digest, family, index, time
    window)."""
    lo = spec["index"] << 22
    own, width, ext = spec_circuit(spec, artifact_dir)
    return A.Shard(blob or own, [t.data_ptr() for t in cols], spec["log_rows"], statement_digest(spec),
                   spec["family"], spec["index"], lo, lo + (1 << spec["log_rows"]), ext=ext, decoder_width=width)


def _as_dict(p):
    return {"cms": p.cms, "gkr": p.gkr, "point": p.point, "vs": p.values, "opening": p.opening,
            "transcript": p.transcript, "phase_ms": p.phase_ms}


def prove_shard(ctx, spec, cols, blob=None, artifact_dir=None):
    """One shard through the library's shard prover (apg_prove_shard): the
    commitments, the GKR proof, the base point, the opened values, the
    opening proof and the transcript after it."""
    return _as_dict(ctx.prove_shard(make_shard(spec, cols, blob, artifact_dir)))


def prove_shard_composed(ctx, spec, cols, artifact_dir=None):
    """The same shard from the library's separate entry points, the schedule
    driven from here: what apg_prove_shard must reproduce."""
    n_vars = spec["log_rows"]
    ptrs = [t.data_ptr() for t in cols]
    cms = ctx.commit_batch_device(ptrs, n_vars)
    tr, g, beta = shard_transcript(spec, cms)
    blob, width, ext = spec_circuit(spec, artifact_dir)
    ch = shard_challenges(g, beta, width, ext)
    values = ctx.gkr_forward(blob, ptrs, ch, on_device=True)
    proof, tr, point = ctx.gkr_prove(blob, values, ch, tr, with_point=True)
    values.free()
    u = A.from_mont_bytes(point)
    vs, opening, tr = ctx.batch_open(ptrs, n_vars, cms, u, tr, on_device=True)
    return {"cms": cms, "gkr": proof, "point": u, "vs": vs, "opening": opening, "transcript": tr}


def prove_sequential(ctx, specs, columns, blobs=None, artifact_dir=None):
    """One shard at a time on one context (the plain path)."""
    t0 = time.perf_counter()
    outs = {s["index"]: prove_shard(ctx, s, columns[s["index"]], (blobs or {}).get(s["index"]), artifact_dir)
            for s in specs}
    return time.perf_counter() - t0, outs


def prove_batched(server, specs, columns, blobs=None, artifact_dir=None):
    """Every shard submitted at once to the library's server, largest first;
    it admits them as workers and memory allow and runs them side by side."""
    order = sorted(specs, key=lambda s: -(s["cols"] << s["log_rows"]))
    t0 = time.perf_counter()
    tickets = {s["index"]: server.submit(make_shard(s, columns[s["index"]], (blobs or {}).get(s["index"]),
                                                    artifact_dir))
               for s in order}
    outs, times = {}, {}
    for i, t in tickets.items():
        p, tm = server.wait(t)
        outs[i], times[i] = _as_dict(p), tm
    return time.perf_counter() - t0, outs, times


def serve(server, specs, columns, rate: float, seed: int = 7, blobs=None, artifact_dir=None):
    """A seeded Poisson stream of shard requests at `rate` a second, in the
    order of `specs`, submitted to the library's server as they arrive.
    Returns (wall seconds, sorted latencies in seconds, each shard's proof by
    index, each request's times)."""
    rng = random.Random(seed)
    arrivals = []
    t = 0.0
    for s in specs:
        t += rng.expovariate(rate)
        arrivals.append((t, s))
    tickets = {}
    start = time.perf_counter()
    for at, s in arrivals:
        delay = at - (time.perf_counter() - start)
        if delay > 0:
            time.sleep(delay)
        tickets[s["index"]] = server.submit(make_shard(s, columns[s["index"]], (blobs or {}).get(s["index"]),
                                                       artifact_dir))
    outs, times = {}, {}
    for i, tk in tickets.items():
        p, tm = server.wait(tk)
        outs[i], times[i] = _as_dict(p), tm
    wall = time.perf_counter() - start
    lat = sorted((tm["done_ns"] - tm["submit_ns"]) / 1e9 for tm in times.values())
    return wall, lat, outs, times


def latency_attribution(times, q_lo=0.99, q_hi=1.0):
    """Where a band of requests' time went: the requests whose latency lies
    between the q_lo- and q_hi-quantiles (0.99-1.0: the tail; 0.45-0.55:
    around the median), their mean latency, mean queueing (submit to
    admission) and mean phases (commit, forward, GKR proof, opening) in ms.
    Queueing plus the phases is about the latency; the rest is the host work
    between admission and the first phase and after the last."""
    lat = sorted(((tm["done_ns"] - tm["submit_ns"]) / 1e6, i) for i, tm in times.items())
    if not lat:
        return {}
    lo = max(0, min(len(lat) - 1, int(math.ceil(q_lo * len(lat))) - 1))
    hi = max(lo + 1, min(len(lat), int(math.ceil(q_hi * len(lat)))))
    band = lat[lo:hi]
    n = len(band)
    qwait = sum((times[i]["admit_ns"] - times[i]["submit_ns"]) / 1e6 for _, i in band) / n
    phases = [sum(times[i]["phase_ms"][j] for _, i in band) / n for j in range(4)]
    return {"requests": n, "quantiles": [q_lo, q_hi], "latency_ms": sum(x for x, _ in band) / n,
            "queue_ms": qwait, "commit_ms": phases[0], "forward_ms": phases[1], "gkr_ms": phases[2],
            "open_ms": phases[3]}


def percentile(xs, q):
    if not xs:
        return None
    k = max(0, min(len(xs) - 1, int(math.ceil(q * len(xs))) - 1))
    return xs[k]
