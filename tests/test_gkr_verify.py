"""The library's GKR verifier (apg_gkr_verify, gkr_verify::verify on the
host) against the definition's restatement of the reference verifier
(gkr_definition.verify without enforcing claims, which is the reference's
check exactly), over proofs the C++ oracle makes on the CPU:

* the reference's toy artifacts over its toy columns (oracle.rs), accepted
  with the definition's base point and claims and the same transcript after;
* random circuits without enforcing gates, accepted likewise, their base
  claims discharged against the base columns;
* random circuits whose enforcing gates do not vanish, and the reference's
  family circuits over random rows, rejected at the same gate list as the
  definition rejects them;
* a bumped round coefficient or claim, rejected at its gate list; the
  reference's shape and challenge errors in its order.

Host only: the verifier runs no device code."""
import random

import pytest

import gkr_definition as D
import oracle_lib as O
from test_gkr_definition import every_kind_circuit, oracle_gkr, random_base, toy_bind, toy_circuit, toy_columns

pytestmark = pytest.mark.cpu_host
P = O.P_R


def _A():
    import apogee_gpu as A

    try:
        A.lib()
    except ImportError as e:
        pytest.skip(str(e))
    return A


def _outputs(A, circ, top):
    return [A.to_mont_bytes(top[off]) for off in D.outputs_of(circ)]


def _proof_bytes(A, proof):
    return A.to_mont_bytes(proof)


def _definition(circ, top, proof, ch, snap):
    """(point, values, snapshot after) or the gate list the definition
    rejects at."""
    s = bytearray(snap)
    try:
        point, values = D.verify(circ, top, proof, ch, s)
    except D.DefinitionMismatch as e:
        msg = str(e)
        return int(msg.split("transition ")[1].split()[0].rstrip(":"))
    return point, values, bytes(s)


def _library_snapshot(A, snap):
    """The oracle's snapshot bytes as the library's (the same 226-byte form)."""
    return bytes(snap)


def _check_same(A, circ, top, proof, ch, snap):
    want = _definition(circ, top, proof, ch, snap)
    try:
        got = A.gkr_verify(circ.to_blob(), _outputs(A, circ, top), _proof_bytes(A, proof), ch,
                           _library_snapshot(A, snap))
    except A.GkrError as e:
        assert e.variant == "LayerInconsistency", e
        assert want == e.info, (want, e.info)
        return None
    assert not isinstance(want, int), f"the definition rejects at {want}, the library accepts"
    point, values, after = got
    assert point == want[0] and values == want[1]
    assert after == want[2]
    return got


@pytest.mark.parametrize("name", ["toy_cached.bin", "toy_cache_free.bin"])
def test_toys_accepted(name):
    A = _A()
    circ = toy_circuit(name)
    for seed in range(3):
        cols = toy_columns(0x53131200 + seed)
        _, probe, gamma = toy_bind(cols)
        after = bytearray(probe)
        proof, top = oracle_gkr(circ, list(cols), {0: gamma}, after)
        got = _check_same(A, circ, top, proof, {0: gamma}, probe)
        assert got is not None, "the reference's toy proof is rejected"
        assert got[2] == bytes(after)
        D.discharge([[x % P for x in c] for c in cols], got[0], got[1])


def _without_enforcing(circ):
    for i, L in enumerate(circ.layers):
        circ.layers[i] = L[:5] + ([],)
    return circ


@pytest.mark.parametrize("seed", range(6))
def test_random_circuits_accepted(seed):
    import circuits as C

    A = _A()
    rng = random.Random(4100 + seed)
    circ = _without_enforcing(C.random_circuit(rng, rng.choice([2, 3, 4]), rng.randint(1, 3), rng.randint(1, 4),
                                               list(range(7)), slots=(0, 1, 2)))
    base = random_base(rng, circ)
    ch = {s: rng.randrange(P) for s in (0, 1, 2)}
    snap = O.new_snapshot()
    O.transcript_op(snap, 2, 39, O.fe(seed), 1)
    after = bytearray(snap)
    proof, top = oracle_gkr(circ, base, ch, after)
    got = _check_same(A, circ, top, proof, ch, snap)
    assert got is not None and got[2] == bytes(after)
    D.discharge([[x % P for x in c] for c in base], got[0], got[1])


@pytest.mark.parametrize("seed", range(4))
def test_unsatisfied_enforcing_rejected_like_the_definition(seed):
    A = _A()
    rng = random.Random(4200 + seed)
    circ = every_kind_circuit(4200 + seed, rng.choice([2, 3, 4]))
    base = random_base(rng, circ)
    ch = {s: rng.randrange(P) for s in (0, 1, 2)}
    snap = O.new_snapshot()
    proof, top = oracle_gkr(circ, base, ch, bytearray(snap))
    assert isinstance(_definition(circ, top, proof, ch, snap), int)
    assert _check_same(A, circ, top, proof, ch, snap) is None


@pytest.mark.parametrize("name", ["lookup_toy.bin", "add_sub.bin", "mul_div.bin"])
def test_artifacts_like_the_definition(name):
    import artifact

    A = _A()
    art = artifact.decode(O.golden_artifacts()[name])
    circ = artifact.to_circuit(art, min(3, art["trace_vars"]))
    rng = random.Random(sum(name.encode()) + 1)
    base = random_base(rng, circ)
    slots = sorted({c[1] for L in art["layers"] for grp in ("cached", "producing", "enforcing")
                    for e in L[grp] for c in e[-1]["coeffs"] if c[0] == "ch"} | {0})
    ch = {s: rng.randrange(P) for s in slots}
    snap = O.new_snapshot()
    proof, top = oracle_gkr(circ, base, ch, bytearray(snap))
    _check_same(A, circ, top, proof, ch, snap)


def _accepted_case(seed=7):
    import circuits as C

    rng = random.Random(4300 + seed)
    circ = _without_enforcing(C.random_circuit(rng, 3, 2, 3, list(range(7)), slots=(0, 1)))
    base = random_base(rng, circ)
    ch = {0: rng.randrange(P), 1: rng.randrange(P)}
    snap = O.new_snapshot()
    proof, top = oracle_gkr(circ, base, ch, bytearray(snap))
    return circ, top, proof, ch, snap


def test_bumped_values_rejected_at_their_gate_list():
    A = _A()
    circ, top, proof, ch, snap = _accepted_case()
    parts = D.split_proof(circ, proof)
    off = 0
    for k, (rounds, evals) in enumerate(parts):
        for where in ([off + 1] if rounds else []) + [off + 4 * len(rounds)]:
            bad = list(proof)
            bad[where] = (bad[where] + 1) % P
            with pytest.raises(A.GkrError) as e:
                A.gkr_verify(circ.to_blob(), _outputs(A, circ, top), _proof_bytes(A, bad), ch, bytes(snap))
            assert e.value.variant == "LayerInconsistency"
            # A bumped claim of list k fails its final check; a bumped round of
            # list k fails there or at a later round of the same list.
            assert e.value.info == k
            assert _definition(circ, top, bad, ch, snap) == k
        off += 4 * len(rounds) + len(evals)
    # A bumped output value moves the whole top claim.
    bad_top = [list(t) for t in top]
    first = D.outputs_of(circ)[0]
    bad_top[first][0] = (bad_top[first][0] + 1) % P
    with pytest.raises(A.GkrError) as e:
        A.gkr_verify(circ.to_blob(), _outputs(A, circ, bad_top), _proof_bytes(A, proof), ch, bytes(snap))
    assert e.value.info == circ.depth() - 1


def test_shape_and_challenge_errors_in_the_reference_order():
    A = _A()
    circ, top, proof, ch, snap = _accepted_case()
    blob, outs, pb = circ.to_blob(), _outputs(A, circ, top), _proof_bytes(A, proof)
    # MissingChallenge comes first, naming the slot.
    with pytest.raises(A.GkrError) as e:
        A.gkr_verify(blob, outs[:-1], pb[:-32], {0: ch[0]}, bytes(snap))
    assert e.value.variant == "MissingChallenge" and e.value.info == 1
    # Then OutputShape: a table too few, or a table of the wrong size.
    with pytest.raises(A.GkrError) as e:
        A.gkr_verify(blob, outs[:-1], pb[:-32], ch, bytes(snap))
    assert e.value.variant == "OutputShape"
    with pytest.raises(A.GkrError) as e:
        A.gkr_verify(blob, [o[:len(o) // 2] for o in outs], pb[:-32], ch, bytes(snap))
    assert e.value.variant == "OutputShape"
    # Then ProofShape: the first list that does not fit, or depth for extra bytes.
    parts = D.split_proof(circ, proof)
    first_len = 32 * (4 * len(parts[0][0]) + len(parts[0][1]))
    with pytest.raises(A.GkrError) as e:
        A.gkr_verify(blob, outs, pb[:first_len - 32], ch, bytes(snap))
    assert e.value.variant == "ProofShape" and e.value.info == 0
    with pytest.raises(A.GkrError) as e:
        A.gkr_verify(blob, outs, pb[:-32], ch, bytes(snap))
    assert e.value.variant == "ProofShape" and e.value.info == circ.depth() - 1
    with pytest.raises(A.GkrError) as e:
        A.gkr_verify(blob, outs, pb + bytes(32), ch, bytes(snap))
    assert e.value.variant == "ProofShape" and e.value.info == circ.depth()
    # A value at or above p is refused before any check.
    with pytest.raises(A.ApogeeError) as e:
        A.gkr_verify(blob, outs, pb[:-32] + b"\xff" * 32, ch, bytes(snap))
    assert e.value.variant == "NonCanonical"
    # And the good proof still passes with the same inputs.
    A.gkr_verify(blob, outs, pb, ch, bytes(snap))
