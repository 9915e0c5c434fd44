"""GPU parity of the GKR forward pass and layer prover (crates/gkr/src/lib.rs)
against the oracle: every layer's values, every round polynomial and claim,
and the transcript state after the proof, on seeded circuits that exercise
all seven gate shapes, cached entries, enforcing gates, all seven virtual
tables and halving lists."""
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


def oracle_gkr(blob, base_cols, challenges, snap, circuit):
    slots = sorted(challenges)
    sarr = (ctypes.c_uint32 * max(len(slots), 1))(*slots)
    vals = b"".join(O.fe(challenges[s]) for s in slots)
    base = b"".join(O.fe(v) for c in base_cols for v in c)
    s = (ctypes.c_uint8 * O.SNAP).from_buffer(snap)
    n_proof = circuit.proof_elems()
    top_w = circuit.width(circuit.depth())
    top_n = 1 << circuit.vars(circuit.depth())
    proof = O.buf(32 * max(n_proof, 1))
    top = O.buf(32 * max(top_w * top_n, 1))
    rc = O.lib().oracle_gkr_prove(blob, ctypes.c_size_t(len(blob)), base, sarr, vals, ctypes.c_size_t(len(slots)),
                                   s, proof, top)
    assert rc == 0
    p = [O.fe_int(proof.raw[32 * i:32 * i + 32]) for i in range(n_proof)]
    t = [O.fe_int(top.raw[32 * i:32 * i + 32]) for i in range(top_w * top_n)]
    return p, [t[j * top_n:(j + 1) * top_n] for j in range(top_w)]


def run_case(ctx, circuit, seed, slots=(0, 1, 2)):
    import apogee_gpu as A

    rng = random.Random(seed)
    n = 1 << circuit.trace_vars
    base = [[rng.choice([0, 1, rng.getrandbits(32), rng.randrange(O.P_R)]) for _ in range(n)]
            for _ in range(circuit.n_committed)]
    challenges = {s: rng.randrange(O.P_R) for s in slots}
    blob = circuit.to_blob()
    snap = A.transcript_append_scalars(A.transcript_init(), 39, [seed])
    values = ctx.gkr_forward(blob, [A.to_mont_bytes(c) for c in base], challenges)
    for j in range(circuit.n_committed):
        assert values.read(0, j) == base[j]
    osnap = bytearray(snap)
    want_proof, want_top = oracle_gkr(blob, base, challenges, osnap, circuit)
    top = circuit.depth()
    for j in range(circuit.width(top)):
        assert values.read(top, j) == want_top[j], f"forward layer {top} column {j}"
    proof, after = ctx.gkr_prove(blob, values, challenges, snap)
    assert proof == want_proof
    assert after == bytes(osnap)
    values.free()


@pytest.mark.parametrize("seed", range(6))
def test_random_circuits_match_oracle(ctx, seed):
    import circuits as C

    rng = random.Random(100 + seed)
    virtuals = rng.sample(range(7), rng.randint(0, 3))
    trace_vars = rng.choice([2, 3, 5, 7, 9])
    c = C.random_circuit(rng, trace_vars, rng.randint(1, 4), rng.randint(1, 5), virtuals, slots=(0, 1, 2))
    run_case(ctx, c, seed)


def test_every_virtual_table_at_16_vars(ctx):
    """Range16/Xor8 tables need >= 16 variables to be full tables; RamLive's
    high bits start at variable 14."""
    import circuits as C

    c = C.Circuit(16, 2, list(range(7)))
    gates = [C.linear([(1, C.virt(v)), (3, C.col(v % 2))], v) for v in range(7)]
    c.add_layer(gates, enforcing=[C.product(2, C.virt(6), C.col(0))])
    c.add_layer([C.tree_product(C.col(0)), C.tree_cross(C.col(1), C.col(2))], halving=True)
    run_case(ctx, c, 77)


def test_wide_layers(ctx):
    """40 committed columns: the halving list's 80 tables need narrower
    thread blocks to keep every thread's operand slots in shared memory."""
    import circuits as C

    c = C.Circuit(5, 40)
    c.add_layer([C.product(2, C.col(j), C.col((j + 1) % 40)) for j in range(40)],
                enforcing=[C.linear([(1, C.col(j)) for j in range(40)], 3)])
    c.add_layer([C.tree_product(C.col(j)) for j in range(40)], halving=True)
    run_case(ctx, c, 41)


def test_shard_circuit_reduced(ctx):
    """The single-execution-shard circuit shape at 2^10 rows."""
    import circuits as C

    run_case(ctx, C.shard_circuit(10, 8), 5)


def test_bad_circuits_are_refused(ctx):
    import apogee_gpu as A
    import circuits as C

    c = C.Circuit(3, 1)
    c.add_layer([C.product(1, C.col(0), C.col(5))])  # operand outside the layer
    with pytest.raises(A.ApogeeError) as e:
        ctx.gkr_forward(c.to_blob(), [A.to_mont_bytes([1] * 8)], {})
    assert e.value.variant == "BadCircuit"
    with pytest.raises(A.ApogeeError):
        ctx.gkr_forward(b"APGC" + bytes(8), [A.to_mont_bytes([1] * 8)], {})
    good = C.Circuit(3, 1)
    good.add_layer([C.product(("ch", 9), C.col(0), C.col(0))])
    with pytest.raises(A.ApogeeError):  # slot 9 has no value
        ctx.gkr_forward(good.to_blob(), [A.to_mont_bytes([1] * 8)], {})


@pytest.mark.parametrize("name", sorted(O.golden_artifacts()))
def test_reference_family_circuits(ctx, name):
    """The reference's own committed circuit artifacts (its family circuits
    and toy circuits, decoded from their wire form) over 2^6 rows: every
    gate list, cached entry, virtual table and fraction tree of a real
    circuit, forward values and proof equal to the oracle's."""
    import artifact

    art = artifact.decode(O.golden_artifacts()[name])
    circuit = artifact.to_circuit(art, min(6, art["trace_vars"]))
    slots = sorted({c[1] for L in art["layers"] for grp in ("cached", "producing", "enforcing")
                    for e in L[grp] for c in e[-1]["coeffs"] if c[0] == "ch"} | {0})
    run_case(ctx, circuit, sum(name.encode()), slots)


@pytest.mark.parametrize("seed", range(3))
def test_narrow_base_matches_oracle(ctx, seed):
    """A random circuit over a base in every stored width (bitset, u8, u16,
    u32, Fr): the forward values, the proof and the transcript equal the
    oracle's over the lifted base; reading the base back lifts it."""
    import apogee_gpu as A
    import circuits as C

    rng = random.Random(500 + seed)
    circ = C.random_circuit(rng, 6 + seed, 5 + seed, 3, rng.sample(range(7), 2), slots=(0, 1, 2))
    n = 1 << circ.trace_vars
    widths = [(1, 8, 16, 32, 0)[j % 5] for j in range(circ.n_committed)]
    base = [[rng.getrandbits(b) for _ in range(n)] if b else [rng.randrange(O.P_R) for _ in range(n)]
            for b in widths]
    challenges = {s: rng.randrange(O.P_R) for s in (0, 1, 2)}
    blob = circ.to_blob()
    snap = A.transcript_append_scalars(A.transcript_init(), 39, [seed])
    values = ctx.gkr_forward_narrow(blob, [A.narrow_bytes(c, b) for c, b in zip(base, widths)], widths, challenges)
    osnap = bytearray(snap)
    want_proof, want_top = oracle_gkr(blob, base, challenges, osnap, circ)
    top = circ.depth()
    for j in range(circ.width(top)):
        assert values.read(top, j) == want_top[j]
    proof, after = ctx.gkr_prove(blob, values, challenges, snap)
    assert proof == want_proof
    assert after == bytes(osnap)
    for j in range(circ.n_committed):
        assert values.read(0, j) == base[j]
    values.free()


def test_narrow_base_family_circuit(ctx):
    """The reference's add_sub artifact over a base of bitsets and u32 columns
    (its committed columns are trace values), forward + proof against the
    oracle."""
    import apogee_gpu as A
    import artifact

    art = artifact.decode(O.golden_artifacts()["add_sub.bin"])
    circ = artifact.to_circuit(art, 6)
    rng = random.Random(8)
    n = 1 << circ.trace_vars
    widths = [1 if j % 3 == 0 else 32 for j in range(circ.n_committed)]
    base = [[rng.getrandbits(b) for _ in range(n)] for b in widths]
    slots = sorted({c[1] for L in art["layers"] for grp in ("cached", "producing", "enforcing")
                    for e in L[grp] for c in e[-1]["coeffs"] if c[0] == "ch"} | {0})
    challenges = {s: rng.randrange(O.P_R) for s in slots}
    blob = circ.to_blob()
    snap = A.transcript_init()
    values = ctx.gkr_forward_narrow(blob, [A.narrow_bytes(c, b) for c, b in zip(base, widths)], widths, challenges)
    osnap = bytearray(snap)
    want_proof, _ = oracle_gkr(blob, base, challenges, osnap, circ)
    proof, after = ctx.gkr_prove(blob, values, challenges, snap)
    assert proof == want_proof and after == bytes(osnap)
    values.free()



def test_linearized_wide_lists_match_oracle(ctx):
    """Wide summed lists are re-linearised into one merged quadratic form:
    a row-wise list of every gate shape over shared operands (products,
    masks, affine products, linear forms with a challenge, quadratics) and a
    halving list whose tree gates repeat products; the proof equals the
    oracle's, gate by gate."""
    import circuits as C

    rng = random.Random(77)

    def r():
        return rng.randrange(O.P_R)

    circ = C.Circuit(8, 5, [C.V_ROW])
    prod = []
    for j in range(24):
        a, b = C.col(j % 5), C.col((3 * j + 1) % 5)
        kind = j % 6
        if kind == 0:
            prod.append(C.product(r(), a, b))
        elif kind == 1:
            prod.append(C.mask(a, b))
        elif kind == 2:
            prod.append(C.affine([(r(), a), (1, C.virt(0))], r(), [(r(), b), (O.P_R - 1, a)], r()))
        elif kind == 3:
            prod.append(C.linear([(r(), a), (1, b), (("ch", 1), C.virt(0))], r()))
        elif kind == 4:
            prod.append(C.quadratic(r(), [(r(), a)], [(1, a, b), (r(), b, b)]))
        else:
            prod.append(C.product(1, b, a))
    enf = [C.quadratic(0, [(1, C.col(0))], [(O.P_R - 1, C.col(0), C.col(0))]) for _ in range(3)]
    circ.add_layer(prod, enforcing=enf)
    circ.add_layer([C.tree_product(C.col(j % 8)) for j in range(20)]
                   + [C.tree_cross(C.col(0), C.col(1)), C.tree_cross(C.col(1), C.col(0))], halving=True)
    run_case(ctx, circ, 77, slots=(0, 1, 2))
