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


@pytest.mark.parametrize("nv,k", [(4, 2), (8, 5), (10, 16)])
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
