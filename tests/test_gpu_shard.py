"""End-to-end parity of the library's shard prover (apg_prove_shard: commit
every column, seed the shard transcript, GKR forward + prove, batched Mercury
opening at the GKR base point) against the oracle driving the same schedule
and against the separate entry points, and the server's invariants
(apg_server, apg_submit, apg_poll/apg_wait): a shard's proof is the same
alone, in a concurrent batch and in the served mix; admission holds to the
memory budget; failures stay with their request."""
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


ARTIFACTS = __import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "artifacts")


def oracle_shard(spec, cols_ints, srs, tau):
    import apogee_gpu as A
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
    blob, width, ext = shard.spec_circuit(spec, ARTIFACTS)
    ch = shard.shard_challenges(g, beta, width, ext)
    L = A.lib()
    L.apg_gkr_proof_len.restype = ctypes.c_size_t
    proof_elems = L.apg_gkr_proof_len(blob, ctypes.c_size_t(len(blob))) // 32
    slots = (ctypes.c_uint32 * len(ch))(*sorted(ch))
    s = (ctypes.c_uint8 * O.SNAP).from_buffer(snap)
    pr = O.buf(32 * proof_elems)
    top = O.buf(32 * 128 * (1 << nv))
    base = b"".join(O.fe(x) for c in cols_ints for x in c)
    assert O.lib().oracle_gkr_prove(blob, ctypes.c_size_t(len(blob)), base, slots,
                                     b"".join(O.fe(ch[k]) for k in sorted(ch)), ctypes.c_size_t(len(ch)), s, pr,
                                     top) == 0
    proof = [O.fe_int(pr.raw[32 * i:32 * i + 32]) for i in range(proof_elems)]
    return cms, proof, snap, g


def test_shard_pipeline_matches_oracle(env):
    import apogee_gpu as A
    import shard

    ctx, torch, tau = env
    srs = O.toy_srs(tau, 1 << 10)
    # Two synthetic shards, then the reference's own family circuits (69 and
    # 3 committed columns; add_sub reads the lookup slots and slot 13 with a
    # decoder channel, image_window a window's constant).
    for spec in ({"index": 3, "family": 7, "log_rows": 4, "cols": 4},
                 {"index": 11, "family": 2, "log_rows": 6, "cols": 5},
                 {"index": 40, "family": 0, "log_rows": 6, "artifact": "add_sub"},
                 {"index": 41, "family": 2, "log_rows": 4, "artifact": "image_window"}):
        shard.spec_circuit(spec, ARTIFACTS)  # fills in a family circuit's column count
        cols = shard.device_columns(torch, 1 << spec["log_rows"], spec["cols"], 99 + spec["index"], "cuda:0", ctx)
        torch.cuda.synchronize()
        out = shard.prove_shard(ctx, spec, cols, artifact_dir=ARTIFACTS)
        assert _strip(out) == shard.prove_shard_composed(ctx, spec, cols, artifact_dir=ARTIFACTS)
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


def _strip(out):
    return {k: v for k, v in out.items() if k != "phase_ms"}


def test_shard_prover_equals_the_composed_entry_points(env):
    """apg_prove_shard equals the same schedule driven from the host over the
    separate entry points (commit_batch, the transcript, gkr_forward/prove,
    batch_open), from device and from host columns."""
    import apogee_gpu as A
    import shard

    ctx, torch, _ = env
    spec = {"index": 21, "family": 4, "log_rows": 8, "cols": 6}
    cols = shard.device_columns(torch, 1 << 8, 6, 1234, "cuda:0", ctx)
    torch.cuda.synchronize()
    want = shard.prove_shard_composed(ctx, spec, cols)
    assert _strip(shard.prove_shard(ctx, spec, cols)) == want
    host = [bytes(c.cpu().numpy().tobytes()) for c in cols]
    lo = spec["index"] << 22
    sh = A.Shard(shard.shard_circuit(8, 6), host, 8, shard.statement_digest(spec), spec["family"], spec["index"], lo,
                 lo + 256, on_device=False)
    p = ctx.prove_shard(sh)
    assert (p.cms, p.gkr, p.point, p.values, p.opening, p.transcript) == (
        want["cms"], want["gkr"], want["point"], want["vs"], want["opening"], want["transcript"])


def test_alone_equals_batched_equals_served(env):
    """The server's invariant: each shard's proof is the same alone (one
    shard at a time on the caller's context), when every shard is submitted
    at once, and in a Poisson stream; requests overlap on the device."""
    import apogee_gpu as A
    import shard

    ctx, torch, _ = env
    rng = random.Random(5)
    specs = [{"index": i, "family": i % 23, "log_rows": rng.choice([2, 4, 6, 8, 10]), "cols": rng.randint(4, 8)}
             for i in range(12)]
    # Family circuits in the same mix (each request carries its own
    # statement challenges and decoder width through the server).
    specs += [{"index": 12, "family": 5, "log_rows": 6, "artifact": "mem_word"},
              {"index": 13, "family": 9, "log_rows": 4, "artifact": "memory_frame_reg"},
              {"index": 14, "family": 12, "log_rows": 4, "artifact": "zero_window"}]
    for s in specs:
        shard.spec_circuit(s, ARTIFACTS)
    columns = {s["index"]: shard.device_columns(torch, 1 << s["log_rows"], s["cols"], 500 + s["index"], "cuda:0",
                                                ctx) for s in specs}
    torch.cuda.synchronize()
    alone = {s["index"]: _strip(shard.prove_shard(ctx, s, columns[s["index"]], artifact_dir=ARTIFACTS))
             for s in specs}
    with A.Server(ctx, max_workers=4) as server:
        _, batched, times = shard.prove_batched(server, specs, columns, artifact_dir=ARTIFACTS)
        for s in specs:
            assert _strip(batched[s["index"]]) == alone[s["index"]], f"shard {s['index']} differs in the batch"
        wall, lat, served, _ = shard.serve(server, specs, columns, rate=200.0, artifact_dir=ARTIFACTS)
        assert len(lat) == len(specs)
        for s in specs:
            assert _strip(served[s["index"]]) == alone[s["index"]], f"shard {s['index']} differs when served"
        st = server.stats()
        assert st["completed"] == 2 * len(specs) and st["failed"] == 0 and st["queued"] == 0
        assert st["peak_in_flight"] > 1, "the requests ran side by side"
        assert all(tm["submit_ns"] <= tm["admit_ns"] <= tm["start_ns"] <= tm["done_ns"] for tm in times.values())


def test_server_admits_by_memory(env):
    """With a budget no second request fits in, the server runs one request
    at a time (the first is always admitted), and every request completes."""
    import apogee_gpu as A
    import shard

    ctx, torch, _ = env
    specs = [{"index": 40 + i, "family": i, "log_rows": 6, "cols": 4} for i in range(5)]
    columns = {s["index"]: shard.device_columns(torch, 1 << 6, 4, 900 + s["index"], "cuda:0", ctx) for s in specs}
    torch.cuda.synchronize()
    with A.Server(ctx, hbm_budget=1) as server:
        _, outs, _ = shard.prove_batched(server, specs, columns)
        st = server.stats()
    assert st["peak_in_flight"] == 1 and st["completed"] == len(specs)
    for s in specs:
        assert _strip(outs[s["index"]]) == _strip(shard.prove_shard(ctx, s, columns[s["index"]]))


def test_server_reports_each_requests_failure(env):
    """A malformed circuit is refused at submission; a request whose digest
    is not a field element fails with its own status while the others in the
    same batch complete."""
    import apogee_gpu as A
    import shard

    ctx, torch, _ = env
    cols = shard.device_columns(torch, 1 << 4, 4, 77, "cuda:0", ctx)
    torch.cuda.synchronize()
    good = {"index": 60, "family": 1, "log_rows": 4, "cols": 4}
    with A.Server(ctx) as server:
        bad_blob = A.Shard(b"APGC" + bytes(12), [c.data_ptr() for c in cols], 4, 1, 1, 60, 0, 16)
        with pytest.raises(A.ApogeeError):
            server.submit(bad_blob)
        bad = shard.make_shard(good, cols)
        bad._digest = b"\xff" * 32
        bad.c.statement_digest = bad._digest
        t_bad = server.submit(bad)
        t_good = server.submit(shard.make_shard(good, cols))
        with pytest.raises(A.ApogeeError) as e:
            server.wait(t_bad)
        assert e.value.variant == "NonCanonical"
        p, _ = server.wait(t_good)
        assert p.cms == shard.prove_shard(ctx, good, cols)["cms"]


def test_shard_refuses_bad_external_challenges(env):
    """External challenges may not name a slot the shard draws itself (0,
    6-13), nor one slot twice, nor carry a value that is not a field element;
    the decoder width is at most 7."""
    import apogee_gpu as A
    import shard

    ctx, torch, _ = env
    spec = {"index": 70, "family": 3, "log_rows": 4, "artifact": "memory_frame_reg"}
    blob, width, ext = shard.spec_circuit(spec, ARTIFACTS)
    cols = shard.device_columns(torch, 1 << 4, spec["cols"], 71, "cuda:0", ctx)
    torch.cuda.synchronize()
    lo = spec["index"] << 22
    args = (blob, [c.data_ptr() for c in cols], 4, 5, spec["family"], spec["index"], lo, lo + 16)
    for bad in ({**ext, 6: 1}, {**ext, 0: 1}, {**ext, 13: 1}):
        with pytest.raises(A.ApogeeError) as e:
            ctx.prove_shard(A.Shard(*args, ext=bad))
        assert e.value.variant == "InvalidArgument"
    sh = A.Shard(*args, ext=ext)
    sh._ext_values = b"\xff" * 32 + sh._ext_values[32:]
    sh.c.ext_values = sh._ext_values
    with pytest.raises(A.ApogeeError) as e:
        ctx.prove_shard(sh)
    assert e.value.variant == "NonCanonical"
    with pytest.raises(A.ApogeeError) as e:
        ctx.prove_shard(A.Shard(*args, ext=ext, decoder_width=8))
    assert e.value.variant == "InvalidArgument"
    # Missing statement challenges: the circuit names slots nobody set.
    with pytest.raises(A.ApogeeError):
        ctx.prove_shard(A.Shard(*args))
