"""GPU parity of the Mercury opening and batched opening (crates/pcs/src/lib.rs)
against the reference's committed proofs and the oracle: proof bytes, claimed
values and the transcript state after the opening."""
import ctypes
import random

import pytest

import oracle_lib as O
from oracle_lib import hexb

pytestmark = pytest.mark.gpu

TOY_TAU = 0xABCDEF


@pytest.fixture(scope="module")
def ctx():
    import apogee_gpu as A

    with A.Context(0) as c:
        yield c


def _proof_kat(name):
    rec = {"value": {}, "point": {}}
    for line in O.golden_lines(name):
        f = line.split()
        if f[0] in ("value", "point"):
            rec[f[0]][int(f[1])] = O.fe_int(hexb(f[2]))
        else:
            rec[f[0]] = f[1]
    nv = int(rec["numvars"])
    return rec, nv, [rec["value"][i] for i in range(1 << nv)], [rec["point"][i] for i in range(nv)]


def test_mercury_proof_kat(ctx):
    import apogee_gpu as A

    rec, nv, vals, u = _proof_kat("mercury_proof.txt")
    ctx.srs_generate(TOY_TAU, 1 << nv)
    cm = ctx.commit(A.to_mont_bytes(vals), nv)
    assert cm.hex() == rec["commitment"]
    v, proof, snap = ctx.open(A.to_mont_bytes(vals), nv, cm, u, A.transcript_init())
    assert v == O.fe_int(hexb(rec["claim"]))
    assert proof.hex() == rec["proof"]
    # The terminal sponge state: one raw squeeze after the opening.
    assert O.transcript_op(bytearray(snap), 1).hex() == rec["probe"]


def test_mercury_batch_kat(ctx):
    import apogee_gpu as A

    rec, nv, vals, u = _proof_kat("mercury_batch.txt")
    ctx.srs_generate(TOY_TAU, 1 << nv)
    cm = ctx.commit(A.to_mont_bytes(vals), nv)
    assert cm.hex() == rec["commitment"]
    vs, proof, snap = ctx.batch_open([A.to_mont_bytes(vals)], nv, [cm], u, A.transcript_init())
    assert vs == [O.fe_int(hexb(rec["claim"]))]
    assert proof.hex() == rec["proof"]
    assert O.transcript_op(bytearray(snap), 1).hex() == rec["probe"]


def test_accumulator_three_column_batch(ctx):
    import apogee_gpu as A

    rec = {"batch_value": {}, "batch_point": {}, "batch_claim": {}, "batch_cm": {}}
    for line in O.golden_lines("accumulator.txt"):
        f = line.split()
        if f[0] == "batch_value":
            rec["batch_value"][(int(f[1]), int(f[2]))] = O.fe_int(hexb(f[3]))
        elif f[0] in ("batch_point", "batch_claim"):
            rec[f[0]][int(f[1])] = O.fe_int(hexb(f[2]))
        elif f[0] == "batch_cm":
            rec[f[0]][int(f[1])] = hexb(f[2])
        elif f[0] in ("numvars", "batch_proof"):
            rec[f[0]] = f[1]
    nv = int(rec["numvars"])
    k = len(rec["batch_cm"])
    cols = [[rec["batch_value"][(c, i)] for i in range(1 << nv)] for c in range(k)]
    u = [rec["batch_point"][i] for i in range(nv)]
    ctx.srs_generate(TOY_TAU, 1 << nv)
    cms = [ctx.commit(A.to_mont_bytes(c), nv) for c in cols]
    assert cms == [rec["batch_cm"][c] for c in range(k)]
    vs, proof, _ = ctx.batch_open([A.to_mont_bytes(c) for c in cols], nv, cms, u, A.transcript_init())
    assert vs == [rec["batch_claim"][c] for c in range(k)]
    assert proof.hex() == rec["batch_proof"]


def _oracle_open(srs, vals, nv, cm, u, snap):
    s = (ctypes.c_uint8 * O.SNAP).from_buffer(snap)
    v, proof = O.buf(32), O.buf(704)
    rc = O.lib().oracle_mercury_open(srs, ctypes.c_size_t(len(srs) // 64), b"".join(O.fe(x) for x in vals), nv, cm,
                                      b"".join(O.fe(x) for x in u), s, 8, v, proof)
    assert rc == 0
    return O.fe_int(v.raw), proof.raw


@pytest.mark.parametrize("nv", [2, 4, 6, 8, 10, 12, 18])
def test_open_matches_oracle(ctx, nv):
    """nv = 18 runs the quotient MSMs through the affine pair rounds: q (2^18 - 2^9
    points) and g (2^9) share one group, so g's bucket range is almost empty."""
    import apogee_gpu as A

    rng = random.Random(900 + nv)
    tau = rng.randrange(O.P_R)
    n = 1 << nv
    srs = O.toy_srs(tau, n)
    ctx.srs_upload(srs)
    vals = [rng.choice([0, 1, rng.getrandbits(32), rng.randrange(O.P_R)]) for _ in range(n)]
    u = [rng.randrange(O.P_R) for _ in range(nv)]
    cm = ctx.commit(A.to_mont_bytes(vals), nv)
    snap = A.transcript_append_scalars(A.transcript_init(), 39, [nv])
    osnap = bytearray(snap)
    v, proof, after = ctx.open(A.to_mont_bytes(vals), nv, cm, u, snap)
    ov, oproof = _oracle_open(srs, vals, nv, cm, u, osnap)
    assert v == ov
    assert proof == oproof
    assert after == bytes(osnap)


# 32 and 40 columns: cm* summed on the host up to 32 commitments, through the
# device MSM above that.
@pytest.mark.parametrize("nv,k", [(4, 2), (8, 5), (10, 16), (6, 32), (6, 40)])
def test_batch_open_matches_oracle(ctx, nv, k):
    import apogee_gpu as A

    rng = random.Random(70 + nv * k)
    n = 1 << nv
    tau = rng.randrange(O.P_R)
    srs = O.toy_srs(tau, n)
    ctx.srs_upload(srs)
    cols = [[rng.choice([0, 1, rng.getrandbits(32), rng.randrange(O.P_R)]) for _ in range(n)] for _ in range(k)]
    u = [rng.randrange(O.P_R) for _ in range(nv)]
    cms = [ctx.commit(A.to_mont_bytes(c), nv) for c in cols]
    snap = A.transcript_init()
    osnap = bytearray(snap)
    vs, proof, after = ctx.batch_open([A.to_mont_bytes(c) for c in cols], nv, cms, u, snap)
    s = (ctypes.c_uint8 * O.SNAP).from_buffer(osnap)
    ovs, oproof = O.buf(32 * k), O.buf(704)
    rc = O.lib().oracle_mercury_batch_open(srs, ctypes.c_size_t(n), b"".join(O.fe(x) for c in cols for x in c),
                                            ctypes.c_size_t(k), nv, b"".join(cms), b"".join(O.fe(x) for x in u), s, 8,
                                            ovs, oproof)
    assert rc == 0
    assert vs == [O.fe_int(ovs.raw[32 * i:32 * i + 32]) for i in range(k)]
    assert proof == oproof.raw
    assert after == bytes(osnap)


def test_open_shape_errors(ctx):
    import apogee_gpu as A

    ctx.srs_generate(3, 16)
    with pytest.raises(A.PcsError) as e:
        ctx.open(bytes(32 * 8), 3, bytes(64), [1, 2, 3], A.transcript_init())
    assert e.value.variant == "UnsupportedNumVars"
    with pytest.raises(A.PcsError) as e:
        ctx.open(bytes(32 * 16), 4, bytes(64), [1, 2, 3], A.transcript_init())
    assert e.value.variant == "PointLengthMismatch"
    with pytest.raises(A.PcsError) as e:
        ctx.open(bytes(32 * 64), 6, bytes(64), [1] * 6, A.transcript_init())
    assert e.value.variant == "SrsTooSmall"
    with pytest.raises(A.PcsError) as e:
        ctx.batch_open([], 4, [], [1] * 4, A.transcript_init())
    assert e.value.variant == "EmptyBatch"


@pytest.mark.parametrize("width,sigma,lens", [(4, 2, [4, 3, 1]), (3, 3, [8, 5, 1]), (5, 1, [2, 1]),
                                              (0, 2, [4, 1]), (9, 3, [8, 2, 1, 7])])
def test_batch_open_stacked_matches_oracle(ctx, width, sigma, lens):
    """pcs::batch_open_stacked (crates/pcs/src/lib.rs:705-789): values, proof
    bytes and transcript equal the oracle's; each value is its stack's
    materialised table at u || r, whose commitment is the one opened."""
    import apogee_gpu as A

    rng = random.Random(300 + 17 * width + sigma)
    nv = width + sigma
    n = 1 << nv
    srs = O.toy_srs(rng.randrange(O.P_R), n)
    ctx.srs_upload(srs)
    pick = lambda: rng.choice([0, 1, rng.getrandbits(32), rng.randrange(O.P_R)])  # noqa: E731
    stacks = [[[pick() for _ in range(1 << width)] for _ in range(L)] for L in lens]
    tables = [[x for c in st for x in c] + [0] * (((1 << sigma) - len(st)) << width) for st in stacks]
    cms = [ctx.commit(A.to_mont_bytes(t), nv) for t in tables]
    u = [rng.randrange(O.P_R) for _ in range(width)]
    r = [rng.randrange(O.P_R) for _ in range(sigma)]
    snap = A.transcript_init()
    vs, proof, after = ctx.batch_open_stacked([[A.to_mont_bytes(c) for c in st] for st in stacks], width, cms, u,
                                              r, snap)
    osnap = bytearray(snap)
    rc, ovs, oproof = O.batch_open_stacked(srs, n, stacks, [width] * sum(lens), cms, u, r, osnap)
    assert rc == 0
    assert vs == ovs == [O.mle_eval(t, u + r) for t in tables]
    assert proof == oproof
    assert after == bytes(osnap)


def test_batch_open_stacked_from_device_columns(ctx):
    import torch

    import apogee_gpu as A

    rng = random.Random(41)
    width, sigma, lens = 6, 2, [4, 2]
    nv = width + sigma
    srs = O.toy_srs(rng.randrange(O.P_R), 1 << nv)
    ctx.srs_upload(srs)
    stacks = [[[rng.randrange(O.P_R) for _ in range(1 << width)] for _ in range(L)] for L in lens]
    cms = [ctx.commit_stack([A.to_mont_bytes(c) for c in st], width) for st in stacks]
    u = [rng.randrange(O.P_R) for _ in range(width)]
    r = [rng.randrange(O.P_R) for _ in range(sigma)]
    host = ctx.batch_open_stacked([[A.to_mont_bytes(c) for c in st] for st in stacks], width, cms, u, r,
                                  A.transcript_init())
    dev = [[torch.frombuffer(bytearray(A.to_mont_bytes(c)), dtype=torch.uint8).to("cuda:0") for c in st]
           for st in stacks]
    on_dev = ctx.batch_open_stacked([[t.data_ptr() for t in st] for st in dev], width, cms, u, r,
                                    A.transcript_init(), on_device=True)
    torch.cuda.synchronize()
    assert on_dev == host


def test_batch_open_stacked_refusal_order(ctx):
    """EmptyBatch, BatchLengthMismatch (commitments), MixedColumnSizes,
    UnsupportedNumVars, PointLengthMismatch, BatchLengthMismatch (slots),
    SrsTooSmall: crates/pcs/src/lib.rs:713-754, in that order."""
    import apogee_gpu as A

    ctx.srs_generate(7, 16)
    col = A.to_mont_bytes(list(range(4)))
    col8 = A.to_mont_bytes(list(range(8)))
    cms = [bytes(64)] * 2
    u, r = [1, 2], [3, 4]
    tr = A.transcript_init()

    def refused(stacks, nvs, c, uu, rr):
        with pytest.raises(A.PcsError) as e:
            ctx.batch_open_stacked(stacks, nvs, c, uu, rr, tr)
        return e.value.variant

    assert refused([], 2, [], u, r) == "EmptyBatch"
    assert refused([[col], []], 2, cms, u, r) == "EmptyBatch"
    assert refused([[col], [col]], 2, cms[:1], u, r) == "BatchLengthMismatch"
    assert refused([[col], [col, col8]], [2, 2, 3], cms, u, r) == "MixedColumnSizes"
    assert refused([[col], [col]], 2, cms, u, r[:1]) == "UnsupportedNumVars"
    assert refused([[col], [col]], 2, cms, u[:1], r) == "PointLengthMismatch"
    assert refused([[col] * 5, [col]], 2, cms, u, r) == "BatchLengthMismatch"
    ctx.srs_generate(7, 8)
    assert refused([[col], [col]], 2, cms, u, r) == "SrsTooSmall"


@pytest.mark.parametrize("nv,k", [(12, 0), (18, 0), (10, 16), (6, 40)])
def test_device_openings_pass_the_deferred_verifier(ctx, nv, k):
    """Openings made on the device (k = 0: one column; else a batch of k)
    through the library's deferred verifier on the host: the twelve entries
    satisfy A = tau B under the SRS's tau, and the verifier leaves the
    transcript where the prover left it."""
    import apogee_gpu as A

    rng = random.Random(4400 + nv * 100 + k)
    n = 1 << nv
    tau = rng.randrange(1, O.P_R)
    srs = O.toy_srs(tau, n)
    ctx.srs_upload(srs)
    cols = [[rng.choice([0, 1, rng.getrandbits(32), rng.randrange(O.P_R)]) for _ in range(n)]
            for _ in range(max(k, 1))]
    u = [rng.randrange(O.P_R) for _ in range(nv)]
    cms = [ctx.commit(A.to_mont_bytes(c), nv) for c in cols]
    snap = A.transcript_append_scalars(A.transcript_init(), 39, [nv])
    if k == 0:
        v, proof, after = ctx.open(A.to_mont_bytes(cols[0]), nv, cms[0], u, snap)
        sides, scalars, points, tr = A.mercury_verify_deferred(cms[0], u, v, proof, snap)
    else:
        vs, proof, after = ctx.batch_open([A.to_mont_bytes(c) for c in cols], nv, cms, u, snap)
        sides, scalars, points, tr = A.mercury_batch_verify_deferred(cms, u, vs, proof, snap)
    assert tr == after
    rc, a, b, _, _ = O.accumulator_msms(sides, scalars, points, [12], weights=[1])
    assert rc == 0 and a == O.g1_mul(b, tau)
