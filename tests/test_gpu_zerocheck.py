"""GPU parity of the zerocheck prover (crates/sumcheck/src/lib.rs:359-408)
against the oracle: rounds, final evaluations and the transcript state after
the proof, byte for byte, on the same seeded inputs and transcript."""
import ctypes
import random

import pytest

import oracle_lib as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import apogee_gpu as A

    with A.Context(0) as c:
        yield c


def oracle_zerocheck(terms, cols, nv, snap):
    arity = len(cols)
    coefs = b"".join(O.fe(t[0]) for t in terms)
    ta = (ctypes.c_uint32 * max(len(terms), 1))(*[t[1] for t in terms])
    tb = (ctypes.c_uint32 * max(len(terms), 1))(*[0xFFFFFFFF if t[2] is None else t[2] for t in terms])
    polys = b"".join(O.fe(v) for c in cols for v in c)
    s = (ctypes.c_uint8 * O.SNAP).from_buffer(snap)
    rounds = O.buf(128 * max(nv, 1))
    finals = O.buf(32 * arity)
    rc = O.lib().oracle_prove_zerocheck(ctypes.c_size_t(arity), coefs, ta, tb, ctypes.c_size_t(len(terms)), polys,
                                         ctypes.c_size_t(nv), s, rounds, finals)
    assert rc == 0
    rs = [O.fe_int(rounds.raw[32 * i:32 * i + 32]) for i in range(4 * nv)]
    return [rs[4 * i:4 * i + 4] for i in range(nv)], [O.fe_int(finals.raw[32 * i:32 * i + 32]) for i in range(arity)]


def run_case(ctx, terms, cols, nv, seed):
    import apogee_gpu as A

    # Both sides start from the same transcript with some history, absorb the
    # witness digest, then prove.
    snap = A.transcript_init()
    snap = A.transcript_append_scalars(snap, 3, [seed, seed + 1])
    mem = [A.to_mont_bytes(c) for c in cols]
    digest = ctx.witness_digest(mem, nv)
    want_digest = O.buf(32)
    O.lib().oracle_witness_digest(b"".join(O.fe(v) for c in cols for v in c), ctypes.c_size_t(len(cols)),
                                  ctypes.c_size_t(nv), want_digest)
    assert digest == O.fe_int(want_digest.raw)
    snap = A.transcript_append_scalars(snap, 8, [digest])
    osnap = bytearray(snap)
    rounds, finals, after = ctx.prove_zerocheck(terms, mem, nv, snap)
    o_rounds, o_finals = oracle_zerocheck(terms, cols, nv, osnap)
    assert rounds == o_rounds
    assert finals == o_finals
    assert after == bytes(osnap)
    # The prover's final values are the columns' evaluations at the bound point.
    return rounds, finals


@pytest.mark.parametrize("nv", [0, 1, 2, 3, 5, 8, 11, 13, 14])
def test_zerocheck_matches_oracle(ctx, nv):
    rng = random.Random(nv)
    n = 1 << nv
    cols = [[rng.randrange(O.P_R) for _ in range(n)] for _ in range(3)]
    terms = [(rng.randrange(O.P_R), 0, 1), (rng.randrange(O.P_R), 1, None), (5, 2, 2), (O.P_R - 1, 0, 2)]
    run_case(ctx, terms, cols, nv, 40 + nv)


def test_zerocheck_product_gate_config1_shape(ctx):
    """The config-1 shape at a reduced size: Product gate a*b over two columns."""
    rng = random.Random(16)
    nv = 12
    cols = [[rng.randrange(O.P_R) for _ in range(1 << nv)] for _ in range(2)]
    run_case(ctx, [(1, 0, 1)], cols, nv, 7)


def test_zerocheck_edge_gates(ctx):
    """An empty gate (the zero formula), a single-input gate, and a vanishing
    witness (a*b - c with c = a*b), whose round 0 sums to zero."""
    rng = random.Random(3)
    nv = 6
    n = 1 << nv
    a = [rng.randrange(O.P_R) for _ in range(n)]
    b = [rng.randrange(O.P_R) for _ in range(n)]
    c = [x * y % O.P_R for x, y in zip(a, b)]
    rounds, _ = run_case(ctx, [(1, 0, 1), (O.P_R - 1, 2, None)], [a, b, c], nv, 1)
    g0 = rounds[0]
    assert (g0[0] + sum(g0)) % O.P_R == 0  # g(0) + g(1) = 0
    run_case(ctx, [], [a], nv, 2)
    run_case(ctx, [(9, 0, None)], [a], nv, 3)


def test_zerocheck_rejects_bad_terms(ctx):
    import apogee_gpu as A

    with pytest.raises(A.ApogeeError):
        ctx.prove_zerocheck([(1, 0, 5)], [A.to_mont_bytes([1, 2])], 1, A.transcript_init())


WIDTHS = (1, 8, 16, 32, 0)


def _narrow_cols(rng, widths, n):
    cols = []
    for b in widths:
        if b == 0:
            cols.append([rng.randrange(O.P_R) for _ in range(n)])
        else:
            cols.append([rng.getrandbits(b) for _ in range(n)])
    return cols


@pytest.mark.parametrize("nv", [0, 1, 2, 6, 7, 12])
def test_zerocheck_narrow_columns_match_oracle(ctx, nv):
    """Columns in every stored width (bitset, u8, u16, u32, Fr) proved through
    the narrow entry point: the same rounds, finals and transcript as the
    oracle over the lifted values, from host and from device buffers."""
    import apogee_gpu as A
    import torch

    rng = random.Random(300 + nv)
    n = 1 << nv
    cols = _narrow_cols(rng, WIDTHS, n)
    terms = [(rng.randrange(O.P_R), 0, 1), (rng.randrange(O.P_R), 2, 3), (3, 4, None), (O.P_R - 1, 1, 4)]
    snap = A.transcript_append_scalars(A.transcript_init(), 8, [nv])
    osnap = bytearray(snap)
    want_rounds, want_finals = oracle_zerocheck(terms, cols, nv, osnap)
    data = [A.narrow_bytes(c, b) for c, b in zip(cols, WIDTHS)]
    rounds, finals, after = ctx.prove_zerocheck_narrow(terms, data, WIDTHS, nv, snap)
    assert (rounds, finals, after) == (want_rounds, want_finals, bytes(osnap))
    dev = [torch.frombuffer(bytearray(d), dtype=torch.uint8).cuda() for d in data]
    rounds, finals, after = ctx.prove_zerocheck_narrow(terms, [t.data_ptr() for t in dev], WIDTHS, nv, snap,
                                                       on_device=True)
    assert (rounds, finals, after) == (want_rounds, want_finals, bytes(osnap))


def test_zerocheck_narrow_rejects_bad_width(ctx):
    import apogee_gpu as A

    cols = [bytes(8), bytes(8)]
    with pytest.raises(A.ApogeeError) as e:
        ctx.prove_zerocheck_narrow([(1, 0, 1)], cols, [1, 4], 6, A.transcript_init())
    assert e.value.variant == "InvalidArgument"


@pytest.mark.parametrize("nv", [3, 16])
def test_device_proof_of_a_vanishing_gate_verifies(ctx, nv):
    """The device's proof of a gate that vanishes on its columns passes the
    library's verifier (sumcheck::verify_zerocheck on the host), which
    leaves the transcript where the prover left it."""
    import apogee_gpu as A
    from test_verify_zerocheck import _satisfied

    rng = random.Random(80 + nv)
    terms, cols = _satisfied(rng, nv)
    snap = A.transcript_append_scalars(A.transcript_init(), 8, [nv])
    rounds, finals, after = ctx.prove_zerocheck(terms, [A.to_mont_bytes(c) for c in cols], nv, snap)
    point, tr = A.verify_zerocheck(terms, len(cols), nv, rounds, finals, snap)
    assert tr == after and len(point) == nv
    bad = list(finals)
    bad[0] = (bad[0] + 1) % O.P_R
    with pytest.raises(A.SumcheckError):
        A.verify_zerocheck(terms, len(cols), nv, rounds, bad, snap)
