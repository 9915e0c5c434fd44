"""The library's GKR proofs (apg_gkr_prove, on the device) through the
library's verifier (apg_gkr_verify, gkr_verify::verify on the host):
accepted, the base point the prover reports, every base claim the committed
column's multilinear extension at that point, the transcript left where the
prover left it; and a bumped claim rejected at its gate list."""
import ctypes
import random

import pytest

import gkr_definition as D
import oracle_lib as O

pytestmark = pytest.mark.gpu
P = O.P_R


@pytest.fixture(scope="module")
def ctx():
    import apogee_gpu as A

    with A.Context(0) as c:
        yield c


def _without_enforcing(circ):
    for i, L in enumerate(circ.layers):
        circ.layers[i] = L[:5] + ([],)
    return circ


def _mle(table, point):
    if len(point) <= 12:
        return D.mle(table, point)
    out = O.buf(32)
    assert O.lib().oracle_evaluate(b"".join(O.fe(x) for x in table), ctypes.c_size_t(len(point)),
                                   b"".join(O.fe(x) for x in point), out) == 0
    return O.fe_int(out.raw)


def _prove_and_verify(ctx, circ, seed, slots=(0, 1, 2)):
    import apogee_gpu as A

    rng = random.Random(seed)
    n = 1 << circ.trace_vars
    base = [[rng.choice([0, 1, rng.getrandbits(32), rng.randrange(P)]) for _ in range(n)]
            for _ in range(circ.n_committed)]
    ch = {s: rng.randrange(P) for s in slots}
    blob = circ.to_blob()
    snap = A.transcript_append_scalars(A.transcript_init(), 39, [seed])
    values = ctx.gkr_forward(blob, [A.to_mont_bytes(c) for c in base], ch)
    top = [values.read(circ.depth(), off) for off in D.outputs_of(circ)]
    proof, after, point = ctx.gkr_prove(blob, values, ch, snap, with_point=True)
    values.free()
    outs = [A.to_mont_bytes(t) for t in top]
    got_point, got_values, got_after = A.gkr_verify(blob, outs, A.to_mont_bytes(proof), ch, snap)
    assert got_point == A.from_mont_bytes(point)
    assert got_after == after
    for j, col in enumerate(base):
        assert got_values[j] == _mle([x % P for x in col], got_point), f"base claim {j}"
    return blob, outs, proof, ch, snap


@pytest.mark.parametrize("seed", range(4))
def test_device_proofs_of_random_circuits_verify(ctx, seed):
    import circuits as C

    rng = random.Random(5100 + seed)
    circ = _without_enforcing(C.random_circuit(rng, rng.choice([3, 5, 8]), rng.randint(1, 4), rng.randint(1, 5),
                                               rng.sample(range(7), rng.randint(0, 4)), slots=(0, 1, 2)))
    _prove_and_verify(ctx, circ, 5100 + seed)


def test_device_proof_of_the_shard_circuit_verifies(ctx):
    import apogee_gpu as A
    import circuits as C

    circ = _without_enforcing(C.shard_circuit(12, 8))
    blob, outs, proof, ch, snap = _prove_and_verify(ctx, circ, 5200)
    # A bumped claim of the base list fails its final check.
    parts = D.split_proof(circ, proof)
    bad = list(proof)
    where = 4 * len(parts[0][0])
    bad[where] = (bad[where] + 1) % P
    with pytest.raises(A.GkrError) as e:
        A.gkr_verify(blob, outs, A.to_mont_bytes(bad), ch, snap)
    assert e.value.variant == "LayerInconsistency" and e.value.info == 0
