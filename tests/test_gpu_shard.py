"""End-to-end parity of the shard pipeline (commit every column, seed the shard
transcript, GKR forward + prove, batched Mercury opening at the GKR base point)
against the oracle driving the same schedule, and the serving invariant: a
shard's proof is the same alone, in a concurrent batch and in the served mix."""
import ctypes
import random

import pytest

import oracle_lib as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch

    import apogee_gpu as A

    ctx = A.Context(0)
    tau = 0x51A9D
    ctx.srs_generate(tau, 1 << 10)
    ctx.srs_prepare()
    yield ctx, torch, tau
    ctx.close()


def oracle_shard(spec, cols_ints, srs, tau):
    import shard

    nv = spec["log_rows"]
    n = 1 << nv
    cms = []
    for c in cols_ints:
        out = O.buf(64)
        assert O.lib().oracle_commit(srs, ctypes.c_size_t(n), b"".join(O.fe(x) for x in c), nv, 4, out) == 0
        cms.append(out.raw)
    # The shard transcript's schedule (verifier-core statement.rs:548-572).
    snap = O.new_snapshot()
    lo = spec["index"] << 22
    seed = [shard.statement_digest(spec), spec["family"], spec["index"]]
    O.transcript_op(snap, 2, 39, b"".join(O.fe(x) for x in seed), 3)
    O.transcript_op(snap, 2, 40, O.fe(lo) + O.fe(lo + n), 2)
    limbs = []
    for cm in cms:
        limbs += shard.g1_limbs(cm)
    O.transcript_op(snap, 2, 3, b"".join(O.fe(x) for x in limbs), len(limbs))
    g = O.fe_int(O.transcript_op(snap, 4, 33))
    beta = O.fe_int(O.transcript_op(snap, 4, 33))
    blob = shard.shard_circuit(nv, spec["cols"])
    proof_elems = 4 * nv + spec["cols"] + sum(4 * (nv - 1 - k) + 2 * spec["cols"] for k in range(nv))
    slots = (ctypes.c_uint32 * 2)(0, 1)
    s = (ctypes.c_uint8 * O.SNAP).from_buffer(snap)
    pr = O.buf(32 * proof_elems)
    top = O.buf(32 * spec["cols"])
    base = b"".join(O.fe(x) for c in cols_ints for x in c)
    assert O.lib().oracle_gkr_prove(blob, ctypes.c_size_t(len(blob)), base, slots, O.fe(g) + O.fe(beta),
                                     ctypes.c_size_t(2), s, pr, top) == 0
    proof = [O.fe_int(pr.raw[32 * i:32 * i + 32]) for i in range(proof_elems)]
    return cms, proof, snap, g


def test_shard_pipeline_matches_oracle(env):
    import apogee_gpu as A
    import shard

    ctx, torch, tau = env
    srs = O.toy_srs(tau, 1 << 10)
    for spec in ({"index": 3, "family": 7, "log_rows": 4, "cols": 4},
                 {"index": 11, "family": 2, "log_rows": 6, "cols": 5}):
        cols = shard.device_columns(torch, 1 << spec["log_rows"], spec["cols"], 99 + spec["index"], "cuda:0", ctx)
        torch.cuda.synchronize()
        out = shard.prove_shard(ctx, spec, cols)
        ints = [A.from_mont_bytes(bytes(c.cpu().numpy().tobytes())) for c in cols]
        cms, proof, snap, gamma = oracle_shard(spec, ints, srs, tau)
        assert out["cms"] == cms
        assert out["gkr"] == proof
        # Open with the oracle at the device's base point on the oracle's transcript.
        nv = spec["log_rows"]
        k = spec["cols"]
        s = (ctypes.c_uint8 * O.SNAP).from_buffer(snap)
        ovs, oproof = O.buf(32 * k), O.buf(704)
        assert O.lib().oracle_mercury_batch_open(srs, ctypes.c_size_t(1 << nv),
                                                 b"".join(O.fe(x) for c in ints for x in c), ctypes.c_size_t(k), nv,
                                                 b"".join(cms), b"".join(O.fe(x) for x in out["point"]), s, 4, ovs,
                                                 oproof) == 0
        assert out["vs"] == [O.fe_int(ovs.raw[32 * i:32 * i + 32]) for i in range(k)]
        assert out["opening"] == oproof.raw
        assert out["transcript"] == bytes(snap)
        # The opened values are the columns' evaluations at the point.
        for c, v in zip(ints, out["vs"]):
            t = list(c)
            for r in out["point"]:
                t = [(t[2 * i] + r * (t[2 * i + 1] - t[2 * i])) % O.P_R for i in range(len(t) // 2)]
            assert t[0] == v


def test_alone_equals_batched_equals_served(env):
    import apogee_gpu as A
    import shard

    ctx, torch, _ = env
    rng = random.Random(5)
    specs = [{"index": i, "family": i % 23, "log_rows": rng.choice([2, 4, 6, 8, 10]), "cols": rng.randint(4, 8)}
             for i in range(12)]
    columns = {s["index"]: shard.device_columns(torch, 1 << s["log_rows"], s["cols"], 500 + s["index"], "cuda:0",
                                                ctx) for s in specs}
    torch.cuda.synchronize()
    alone = {s["index"]: shard.prove_shard(ctx, s, columns[s["index"]]) for s in specs}
    extra = [A.Context(0) for _ in range(3)]
    for c in extra:
        c.srs_share(ctx)
    ctxs = [ctx] + extra
    _, batched = shard.prove_batched(ctxs, specs, columns)
    for s in specs:
        assert batched[s["index"]] == alone[s["index"]], f"shard {s['index']} differs in the batch"
    wall, lat, served = shard.serve(ctxs, specs, columns, rate=200.0, budget_bytes=1 << 30)
    assert len(lat) == len(specs)
    for s in specs:
        assert served[s["index"]] == alone[s["index"]], f"shard {s['index']} differs when served"
    for c in extra:
        c.close()
