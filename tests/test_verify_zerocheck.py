"""The library's zerocheck verifier (apg_verify_zerocheck,
sumcheck::verify_zerocheck on the host) over proofs the C++ oracle makes on
the CPU: gates that vanish on their columns are accepted with the transcript's
point and the prover's transcript state; a gate that does not vanish fails
round 0; a bumped round fails at that round, a bumped final value the final
check; the count errors come first, in the reference's order. Host only."""
import ctypes
import random

import pytest

import oracle_lib as O

pytestmark = pytest.mark.cpu_host
P = O.P_R


def _A():
    import apogee_gpu as A

    try:
        A.lib()
    except ImportError as e:
        pytest.skip(str(e))
    return A


def oracle_zerocheck(terms, cols, nv, snap):
    k = len(cols)
    coefs = b"".join(O.fe(t[0] % P) for t in terms)
    nt = len(terms)
    ta = (ctypes.c_uint32 * max(nt, 1))(*[t[1] for t in terms])
    tb = (ctypes.c_uint32 * max(nt, 1))(*[0xFFFFFFFF if t[2] is None else t[2] for t in terms])
    rounds_b, finals_b = O.buf(128 * max(nv, 1)), O.buf(32 * k)
    s = (ctypes.c_uint8 * O.SNAP).from_buffer(snap)
    assert O.lib().oracle_prove_zerocheck(ctypes.c_size_t(k), coefs, ta, tb, ctypes.c_size_t(nt),
                                          b"".join(O.fe(v % P) for c in cols for v in c), ctypes.c_size_t(nv), s,
                                          rounds_b, finals_b) == 0
    rounds = [[O.fe_int(rounds_b.raw[128 * i + 32 * j:128 * i + 32 * j + 32]) for j in range(4)] for i in range(nv)]
    finals = [O.fe_int(finals_b.raw[32 * j:32 * j + 32]) for j in range(k)]
    return rounds, finals


def _replay_point(snap0, rounds):
    t = bytearray(snap0)
    for _ in rounds:
        O.transcript_op(t, 4, 5)
    pt = []
    for g in rounds:
        O.transcript_op(t, 2, 4, b"".join(O.fe(x) for x in g), 4)
        pt.append(O.fe_int(O.transcript_op(t, 4, 5)))
    return pt


def _satisfied(rng, nv):
    """Columns and a degree-2 gate that vanishes on every row: a*b - c with
    c = a*b, x*x - x over a bit column, and 3*(a + d) - 3*e with e = a + d."""
    n = 1 << nv
    a = [rng.randrange(P) for _ in range(n)]
    b = [rng.choice([0, 1, rng.getrandbits(32), rng.randrange(P)]) for _ in range(n)]
    c = [x * y % P for x, y in zip(a, b)]
    bits = [rng.getrandbits(1) for _ in range(n)]
    d = [rng.randrange(P) for _ in range(n)]
    e = [(x + y) % P for x, y in zip(a, d)]
    cols = [a, b, c, bits, d, e]
    la, lb, lc = rng.randrange(1, P), rng.randrange(1, P), rng.randrange(1, P)
    terms = [(la, 0, 1), (P - la, 2, None), (lb, 3, 3), (P - lb, 3, None),
             (lc * 3, 0, None), (lc * 3, 4, None), (P - lc * 3 % P, 5, None)]
    return terms, cols


@pytest.mark.parametrize("nv", [1, 2, 5, 9])
def test_vanishing_gates_accepted(nv):
    A = _A()
    rng = random.Random(60 + nv)
    terms, cols = _satisfied(rng, nv)
    snap0 = O.new_snapshot()
    O.transcript_op(snap0, 2, 8, O.fe(nv), 1)
    after = bytearray(snap0)
    rounds, finals = oracle_zerocheck(terms, cols, nv, after)
    point, tr = A.verify_zerocheck(terms, len(cols), nv, rounds, finals, bytes(snap0))
    assert point == _replay_point(snap0, rounds)
    assert tr == bytes(after)


def test_nonvanishing_gate_fails_round_0():
    A = _A()
    rng = random.Random(70)
    nv = 4
    cols = [[rng.randrange(P) for _ in range(1 << nv)] for _ in range(2)]
    terms = [(5, 0, 1), (7, 1, None)]
    snap0 = O.new_snapshot()
    rounds, finals = oracle_zerocheck(terms, cols, nv, bytearray(snap0))
    with pytest.raises(A.SumcheckError) as e:
        A.verify_zerocheck(terms, 2, nv, rounds, finals, bytes(snap0))
    assert e.value.variant == "RoundSumMismatch" and e.value.info == 0


def test_bumps_and_counts():
    A = _A()
    rng = random.Random(71)
    nv = 5
    terms, cols = _satisfied(rng, nv)
    snap0 = O.new_snapshot()
    rounds, finals = oracle_zerocheck(terms, cols, nv, bytearray(snap0))
    k = len(cols)
    for i in range(nv):
        bad = [list(g) for g in rounds]
        bad[i][1] = (bad[i][1] + 1) % P
        with pytest.raises(A.SumcheckError) as e:
            A.verify_zerocheck(terms, k, nv, bad, finals, bytes(snap0))
        assert e.value.variant == "RoundSumMismatch" and e.value.info == i
    for j in range(k):
        bad = list(finals)
        bad[j] = (bad[j] + 1) % P
        with pytest.raises(A.SumcheckError) as e:
            A.verify_zerocheck(terms, k, nv, rounds, bad, bytes(snap0))
        assert e.value.variant == "FinalEvalMismatch"
    # Counts first: a round short, then a final short (with a round short too,
    # the round count is reported).
    with pytest.raises(A.SumcheckError) as e:
        A.verify_zerocheck(terms, k, nv, rounds[:-1], finals[:-1], bytes(snap0))
    assert e.value.variant == "RoundCountMismatch" and e.value.info == nv - 1
    with pytest.raises(A.SumcheckError) as e:
        A.verify_zerocheck(terms, k, nv, rounds, finals[:-1], bytes(snap0))
    assert e.value.variant == "FinalEvalCountMismatch" and e.value.info == k - 1
    # GateError: a term naming an undeclared input.
    with pytest.raises(A.ApogeeError) as e:
        A.verify_zerocheck(terms + [(1, k, None)], k, nv, rounds, finals, bytes(snap0))
    assert e.value.variant == "InvalidArgument"
    # The good proof, after all that, still verifies.
    A.verify_zerocheck(terms, k, nv, rounds, finals, bytes(snap0))
