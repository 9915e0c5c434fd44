"""The GPU's GKR forward pass and proofs held to the definition and to what
the reference itself holds (the CPU side of the same checks, against the C++
oracle, is tests/test_gkr_definition.py):

* the literal gate known answers of the reference's crates/gkr/tests/kernel.rs
  through the device forward pass, one-gate circuits with the operands as
  columns, and their proofs by definition;
* the reference's toy artifacts against crates/gkr/tests/oracle.rs's hand
  formulas at every node of every round;
* random circuits over all seven gate shapes and all seven virtual tables, and
  all sixteen of the reference's committed circuits, every round by definition,
  the reference verifier's final checks and the discharge of the base claims;
* the virtual tables at 20 variables (Range19's mask, RamLive's bit 14 and the
  bytes of Xor8 all inside) through the reference verifier alone, which reads
  them in closed form."""
import ctypes
import random

import pytest

import gkr_definition as D
import oracle_lib as O
from test_gkr_definition import (Hand, as_gate, check_toy_by_hand, every_kind_circuit, gate_kats, kat_circuit,
                                 random_base, toy_bind, toy_circuit, toy_columns)

pytestmark = pytest.mark.gpu
P = O.P_R


@pytest.fixture(scope="module")
def ctx():
    import apogee_gpu as A

    with A.Context(0) as c:
        yield c


def gpu_prove(ctx, circ, base, challenges, snap):
    """Forward and prove on the device; returns (proof, top layer, transcript after)."""
    import apogee_gpu as A

    blob = circ.to_blob()
    values = ctx.gkr_forward(blob, [A.to_mont_bytes(c) for c in base], challenges)
    try:
        top = [values.read(circ.depth(), j) for j in range(circ.width(circ.depth()))]
        proof, after = ctx.gkr_prove(blob, values, challenges, bytes(snap))
    finally:
        values.free()
    return proof, top, after


def test_gate_kats_on_gpu(ctx):
    kats = gate_kats()
    ch = {kats["slot"]: kats["gamma"]}
    for case in kats["cases"]:
        circ, base = kat_circuit(case)
        snap = O.new_snapshot()
        proof, top, after = gpu_prove(ctx, circ, base, ch, snap)
        assert top[0][0] == case["expect"], case["name"]
        for bad in case["not"]:
            assert top[0][0] != bad, case["name"]
        D.check_proof(circ, base, ch, snap, proof, top=top, after=after)


@pytest.mark.parametrize("name", ["toy_cached.bin", "toy_cache_free.bin"])
def test_toy_by_hand_gpu(ctx, name):
    circ = toy_circuit(name)
    for seed in range(3):
        cols = toy_columns(0x53131200 + seed)
        _snap, probe, gamma = toy_bind(cols)
        h = Hand(cols, gamma)
        proof, top, after = gpu_prove(ctx, circ, list(cols), {0: gamma}, probe)
        assert top[1] == h.fingerprint3_product and top[0] == h.abm_product
        t = check_toy_by_hand(h, proof, probe)
        assert bytes(t) == after
        D.check_proof(circ, list(cols), {0: gamma}, probe, proof, top=top, after=after)


@pytest.mark.parametrize("seed", range(6))
def test_random_circuits_by_definition_gpu(ctx, seed):
    rng = random.Random(1900 + seed)
    circ = every_kind_circuit(1900 + seed, [2, 3, 4, 6, 8, 9][seed])
    base = random_base(rng, circ)
    ch = {s: rng.randrange(P) for s in (0, 1, 2)}
    snap = O.new_snapshot()
    O.transcript_op(snap, 2, 39, O.fe(seed), 1)
    proof, top, after = gpu_prove(ctx, circ, base, ch, snap)
    n = D.check_proof(circ, base, ch, snap, proof, top=top, after=after)
    assert n == 4 * sum(L[1] for L in circ.layers)


@pytest.mark.parametrize("name", sorted(O.golden_artifacts()))
def test_reference_circuits_by_definition_gpu(ctx, name):
    import artifact

    art = artifact.decode(O.golden_artifacts()[name])
    circ = artifact.to_circuit(art, min(6, art["trace_vars"]))
    rng = random.Random(sum(name.encode()) + 7)
    base = random_base(rng, circ)
    slots = sorted({c[1] for L in art["layers"] for grp in ("cached", "producing", "enforcing")
                    for e in L[grp] for c in e[-1]["coeffs"] if c[0] == "ch"} | {0})
    ch = {s: rng.randrange(P) for s in slots}
    snap = O.new_snapshot()
    proof, top, after = gpu_prove(ctx, circ, base, ch, snap)
    D.check_proof(circ, base, ch, snap, proof, top=top, after=after)


def test_virtual_tables_at_20_vars_verify(ctx):
    """A list reading all seven virtual tables over 2^20 rows, then a
    product tree down to one row: the GPU's proof passes the reference
    verifier (closed-form virtual tables at the bound point, pinned against
    the tables' extensions on the CPU) and its base claims discharge."""
    import numpy as np

    import apogee_gpu as A
    import circuits as C

    nv = 20
    circ = C.Circuit(nv, 2, list(range(7)))
    gates = [C.linear([(3 + v, C.virt(v)), (1, C.col(v % 2))], 11 + v) for v in range(7)]
    gates.append(C.product(5, C.virt(1), C.col(0)))  # RamLive times a column
    cac = [C.linear([(2, C.virt(2)), (("ch", 0), C.virt(6))], 1)]
    gates.append(C.quadratic(7, [(1, C.cached(0))], [(1, C.virt(5), C.virt(4))]))
    circ.add_layer(gates, cached=cac)
    for _ in range(nv):
        circ.add_layer([C.tree_product(C.col(j)) for j in range(len(gates))], halving=True)
    n = 1 << nv
    rng = np.random.Generator(np.random.PCG64(20))
    base_u32 = [rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32) for _ in range(2)]
    ch = {0: 0xC0FFEE}
    blob = circ.to_blob()
    values = ctx.gkr_forward_narrow(blob, [c.tobytes() for c in base_u32], [32, 32], ch)
    try:
        top = [values.read(circ.depth(), j) for j in range(circ.width(circ.depth()))]
        snap = O.new_snapshot()
        proof, after = ctx.gkr_prove(blob, values, ch, bytes(snap))
    finally:
        values.free()
    t = bytearray(snap)
    point, claims = D.verify(circ, top, proof, ch, t)
    assert bytes(t) == after
    assert len(point) == nv
    for j, col in enumerate(base_u32):
        canon = np.zeros((n, 8), dtype=np.uint32)
        canon[:, 0] = col
        out = O.buf(32)
        assert O.lib().oracle_evaluate(canon.tobytes(), ctypes.c_size_t(nv), b"".join(O.fe(x) for x in point),
                                       out) == 0
        assert O.fe_int(out.raw) == claims[j], f"base column {j}"
    # A wrong closed form anywhere would have failed a final check; make sure
    # the check bites: a bumped claim of the row-wise list is rejected.
    bad = list(proof)
    bad[4 * nv] = (bad[4 * nv] + 1) % P
    with pytest.raises(D.DefinitionMismatch):
        D.verify(circ, top, bad, ch, bytearray(snap))
