"""The host verifiers never crash on what a proof, a statement or a circuit
carries: seeded random damage to valid inputs (flipped bytes, truncated and
extended buffers, damaged circuit blobs) only ever returns a status. The
reference's verifiers promise the same (crates/gkr-verify/src/lib.rs:640-646:
never panics on anything a proof or its outputs carry). Host only."""
import random

import pytest

import gkr_definition as D
import oracle_lib as O
from test_gkr_verify import _accepted_case, _outputs
from test_mercury_verify import _proof_kat
from test_verify_zerocheck import _satisfied, oracle_zerocheck

pytestmark = pytest.mark.cpu_host
P = O.P_R


def _A():
    import apogee_gpu as A

    try:
        A.lib()
    except ImportError as e:
        pytest.skip(str(e))
    return A


def _damage(rng, b: bytes) -> bytes:
    b = bytearray(b)
    kind = rng.randrange(4)
    if kind == 0 and b:
        for _ in range(rng.randint(1, 4)):
            b[rng.randrange(len(b))] ^= 1 << rng.randrange(8)
    elif kind == 1 and b:
        del b[rng.randrange(len(b)):]
    elif kind == 2:
        b += bytes(rng.getrandbits(8) for _ in range(rng.choice([1, 31, 32, 64])))
    elif b:
        i = rng.randrange(len(b))
        b[i:i + 32] = bytes([0xFF]) * min(32, len(b) - i)
    return bytes(b)


def test_gkr_verify_survives_damage():
    A = _A()
    circ, top, proof, ch, snap = _accepted_case(11)
    blob, outs, pb = circ.to_blob(), _outputs(A, circ, top), A.to_mont_bytes(proof)
    rng = random.Random(1)
    outcomes = set()
    for i in range(400):
        b, o, p, s = blob, list(outs), pb, bytes(snap)
        what = rng.randrange(4)
        if what == 0:
            b = _damage(rng, blob)
        elif what == 1:
            j = rng.randrange(len(o))
            o[j] = _damage(rng, o[j])
        elif what == 2:
            p = _damage(rng, pb)
        else:
            s = _damage(rng, s)[:A.TRANSCRIPT_BYTES].ljust(A.TRANSCRIPT_BYTES, b"\0")
        try:
            A.gkr_verify(b, o, p, ch, s)
            outcomes.add("Ok")
        except A.ApogeeError as e:
            outcomes.add(e.variant)
    assert "LayerInconsistency" in outcomes and "BadCircuit" in outcomes


def test_zerocheck_verify_survives_damage():
    A = _A()
    rng = random.Random(2)
    nv = 5
    terms, cols = _satisfied(rng, nv)
    snap = O.new_snapshot()
    rounds, finals = oracle_zerocheck(terms, cols, nv, bytearray(snap))
    for _ in range(300):
        r = [list(g) for g in rounds]
        f = list(finals)
        what = rng.randrange(3)
        if what == 0:
            r = r[:rng.randrange(len(r) + 1)] + [[rng.randrange(P) for _ in range(4)]] * rng.randint(0, 2)
        elif what == 1:
            f = f[:rng.randrange(len(f) + 1)]
        else:
            i = rng.randrange(nv)
            r[i][rng.randrange(4)] = rng.randrange(P)
        try:
            A.verify_zerocheck(terms, len(cols), nv, r, f, bytes(snap))
        except A.ApogeeError:
            pass


@pytest.mark.parametrize("batch", [False, True])
def test_mercury_verify_survives_damage(batch):
    A = _A()
    u, v, cm, proof, _ = _proof_kat("mercury_proof.txt")
    rng = random.Random(3 + batch)
    for _ in range(300):
        c, p, uu = cm, proof, list(u)
        what = rng.randrange(3)
        if what == 0:
            c = _damage(rng, cm)[:64].ljust(64, b"\0")
        elif what == 1:
            p = _damage(rng, proof)[:704].ljust(704, b"\0")
        else:
            uu = uu[:rng.randrange(len(uu) + 1)] + [rng.randrange(P)] * rng.randint(0, 3)
        try:
            if batch:
                A.mercury_batch_verify_deferred([c] * rng.randint(1, 3), uu, [v] * rng.randint(1, 3), p,
                                                A.transcript_init())
            else:
                A.mercury_verify_deferred(c, uu, v, p, A.transcript_init())
        except A.ApogeeError:
            pass
