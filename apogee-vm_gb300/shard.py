"""Shard proving over the C ABI, and the shard workloads the benchmark runs.

`prove_shard` is the hot-path slice of crates/prover's prove_shard_columns
(crates/prover/src/lib.rs:798-1102): commit every column (commit_all), seed the
shard transcript and absorb the commitments, run the GKR forward and backward
passes, and open every column at the base point GKR leaves with one batched
Mercury opening (opening_part -> batch_open_stacked at r = []).

Workloads:
  * `shard_mix`: 207 shards over 23 circuit families, sizes log-uniform over
    the even heights 2^8 .. 2^22 (Mercury takes even variable counts only),
    4 to 16 columns each, values drawn like VM trace columns.
  * `prove_sequential`: one shard at a time on one context (the plain path).
  * `prove_batched`: shards spread over several contexts (streams) proved
    concurrently, largest first.
  * `serve`: a seeded Poisson stream of shard requests, admitted as a context
    and enough HBM (a fixed budget) free up, proved concurrently; latency is
    completion minus arrival.
"""
import heapq
import math
import random
import threading
import time

import apogee_gpu as A
import circuits as C

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
    """k columns of n Fr on the device (Montgomery), mixed like VM traces:
    25% in {0,1}, 60% uniform u32, 15% uniform Fr below p's top limb."""
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    cols = []
    for _ in range(k):
        w = torch.randint(-(1 << 31), 1 << 31, (n, 8), dtype=torch.int32, device=device, generator=g)
        cls = torch.rand(n, device=device, generator=g)
        w[:, 7] &= 0x2FFFFFFF
        small = cls < 0.85
        w[small, 1:] = 0
        bits = cls < 0.25
        w[bits, 0] &= 1
        flat = w.reshape(-1).contiguous()
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


def prove_shard(ctx, spec, cols):
    """One shard's hot path; cols are device tensors. Returns the commitments,
    the GKR proof, the base point, the opened values and the opening proof."""
    n_vars = spec["log_rows"]
    ptrs = [t.data_ptr() for t in cols]
    cms = ctx.commit_batch_device(ptrs, n_vars)
    tr, g, beta = shard_transcript(spec, cms)
    blob = shard_circuit(n_vars, spec["cols"])
    ch = {0: g, 1: beta}
    values = ctx.gkr_forward(blob, ptrs, ch, on_device=True)
    proof, tr, point = ctx.gkr_prove(blob, values, ch, tr, with_point=True)
    values.free()
    u = A.from_mont_bytes(point)
    vs, opening, tr = ctx.batch_open(ptrs, n_vars, cms, u, tr, on_device=True)
    return {"cms": cms, "gkr": proof, "point": u, "vs": vs, "opening": opening, "transcript": tr}


def hbm_estimate(spec) -> int:
    """Device bytes one shard proof holds at its peak: the columns, the GKR
    layer values (about twice the base), MSM and sumcheck scratch."""
    n = 1 << spec["log_rows"]
    base = 32 * n * spec["cols"]
    return 4 * base + 64 * 16 * n + (64 << 20)


def prove_sequential(ctx, specs, columns):
    t0 = time.perf_counter()
    outs = [prove_shard(ctx, s, columns[s["index"]]) for s in specs]
    return time.perf_counter() - t0, outs


def prove_batched(ctxs, specs, columns):
    """Largest shards first, each context proving the next unclaimed shard."""
    order = sorted(specs, key=lambda s: -(s["cols"] << s["log_rows"]))
    lock = threading.Lock()
    nxt = [0]
    outs = {}
    errors = []

    def worker(ctx):
        while True:
            with lock:
                if nxt[0] >= len(order):
                    return
                s = order[nxt[0]]
                nxt[0] += 1
            try:
                outs[s["index"]] = prove_shard(ctx, s, columns[s["index"]])
            except Exception as e:  # surfaced after the join
                errors.append(e)
                return

    t0 = time.perf_counter()
    threads = [threading.Thread(target=worker, args=(c,)) for c in ctxs]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    dt = time.perf_counter() - t0
    if errors:
        raise errors[0]
    return dt, outs


def serve(ctxs, specs, columns, rate: float, budget_bytes: int, seed: int = 7):
    """Poisson arrivals at `rate` requests/s over `specs` (in order), admitted
    first-come first-served when a context is idle and the request's HBM
    estimate fits the budget. Returns (wall seconds, sorted latencies in
    seconds, each shard's proof by index)."""
    rng = random.Random(seed)
    arrivals = []
    t = 0.0
    for s in specs:
        t += rng.expovariate(rate)
        arrivals.append((t, s))
    cv = threading.Condition()
    state = {"free": list(ctxs), "budget": budget_bytes, "queue": [], "done": 0}
    lat = []
    outputs = {}
    errors = []
    start = time.perf_counter()

    def run(ctx, s, arrival, need):
        try:
            res = prove_shard(ctx, s, columns[s["index"]])
            done = time.perf_counter() - start
            with cv:
                lat.append(done - arrival)
                outputs[s["index"]] = res
        except Exception as e:
            errors.append(e)
        finally:
            with cv:
                state["free"].append(ctx)
                state["budget"] += need
                state["done"] += 1
                cv.notify_all()

    def dispatcher():
        i = 0
        while True:
            with cv:
                now = time.perf_counter() - start
                while i < len(arrivals) and arrivals[i][0] <= now:
                    state["queue"].append(arrivals[i])
                    i += 1
                while state["queue"] and state["free"]:
                    arr, s = state["queue"][0]
                    need = hbm_estimate(s)
                    if need > state["budget"] and state["budget"] < budget_bytes:
                        break  # wait for memory to free up (head of line keeps its turn)
                    state["queue"].pop(0)
                    ctx = state["free"].pop()
                    state["budget"] -= need
                    threading.Thread(target=run, args=(ctx, s, arr, need), daemon=True).start()
                if state["done"] == len(arrivals):
                    return
                wait = 0.05
                if i < len(arrivals):
                    wait = max(0.0, min(wait, arrivals[i][0] - (time.perf_counter() - start)))
                cv.wait(timeout=wait)

    dispatcher()
    wall = time.perf_counter() - start
    if errors:
        raise errors[0]
    return wall, sorted(lat), outputs


def percentile(xs, q):
    if not xs:
        return None
    k = max(0, min(len(xs) - 1, int(math.ceil(q * len(xs))) - 1))
    return xs[k]
