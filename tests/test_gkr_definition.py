"""The GKR semantics pinned to what the reference itself holds, on the CPU:

* the gate kernel against the literal known answers of the reference's
  crates/gkr/tests/kernel.rs (golden/gkr_gate_kats.json), both the
  definition module's and the C++ oracle's;
* the virtual tables' closed forms against the multilinear extension of the
  tables they stand for, at every size around their bit boundaries;
* the toy circuit's rounds against the hand-written formulas of the
  reference's crates/gkr/tests/oracle.rs, restated here;
* the oracle's whole proofs (every round at every node, every claim, the
  reference verifier's final checks, the discharge of the base claims) on
  random circuits over all seven gate shapes and all seven virtual tables,
  on the reference's toy and lookup circuits and on its family circuits.

The GPU side of the same checks is tests/test_gpu_gkr_definition.py."""
import ctypes
import json
import os
import random

import pytest

import gkr_definition as D
import oracle_lib as O

P = O.P_R


def gate_kats():
    with open(os.path.join(O.GOLDEN, "gkr_gate_kats.json")) as f:
        return json.load(f)


def as_gate(g):
    shape, t, u, ops, cs = g
    return (shape, t, u, [(0, x) for x in ops], [tuple(c) if isinstance(c, list) else c for c in cs])


def kat_circuit(case):
    """A one-gate circuit computing the case over its columns: a row-wise
    list over one row pair (row 0 holds the case, row 1 other values), or a
    halving list whose two rows are the case's children."""
    import circuits as C

    shape = case["gate"][0]
    tree = shape in (D.TREE_PRODUCT, D.TREE_CROSS)
    ncols = max(1, len(case["columns"]))
    c = C.Circuit(1, ncols)
    c.add_layer([as_gate(case["gate"])], halving=tree)
    if tree:
        base = [list(v) for v in case["columns"]]
    else:
        base = [[v, 1000 + 7 * j] for j, v in enumerate(case["columns"])] or [[5, 6]]
    return c, base


def test_gate_kats_pin_the_definition():
    kats = gate_kats()
    assert kats["gamma"] == 0x9E3779B97F4A7C15 * 0x0123456789ABCDEF % P
    ch = {kats["slot"]: kats["gamma"]}
    shapes = set()
    for case in kats["cases"]:
        g = as_gate(case["gate"])
        cols = case["columns"]
        if g[0] in (D.TREE_PRODUCT, D.TREE_CROSS):
            v = [x for col in g[3] for x in cols[col[1]]]
        else:
            v = [cols[x] for _, x in g[3]]
        got = D.eval_gate(g, v, ch)
        assert got == case["expect"], case["name"]
        for bad in case["not"]:
            assert got != bad, case["name"]
        shapes.add(g[0])
    assert shapes == set(range(7)), "every gate variant has a known answer"


def oracle_gkr(circ, base, challenges, snap):
    slots = sorted(challenges)
    sarr = (ctypes.c_uint32 * max(len(slots), 1))(*slots)
    vals = b"".join(O.fe(challenges[s]) for s in slots)
    blob = circ.to_blob()
    s = (ctypes.c_uint8 * O.SNAP).from_buffer(snap)
    n_proof = circ.proof_elems()
    top_w, top_n = circ.width(circ.depth()), 1 << circ.vars(circ.depth())
    proof, top = O.buf(32 * max(n_proof, 1)), O.buf(32 * max(top_w * top_n, 1))
    rc = O.lib().oracle_gkr_prove(blob, ctypes.c_size_t(len(blob)), b"".join(O.fe(v) for c in base for v in c),
                                   sarr, vals, ctypes.c_size_t(len(slots)), s, proof, top)
    assert rc == 0, rc
    p = [O.fe_int(proof.raw[32 * i:32 * i + 32]) for i in range(n_proof)]
    t = [O.fe_int(top.raw[32 * i:32 * i + 32]) for i in range(top_w * top_n)]
    return p, [t[j * top_n:(j + 1) * top_n] for j in range(top_w)]


def test_gate_kats_through_the_oracle():
    """The C++ oracle's forward pass computes every known answer, and its
    one-gate proofs hold by definition."""
    kats = gate_kats()
    ch = {kats["slot"]: kats["gamma"]}
    for case in kats["cases"]:
        circ, base = kat_circuit(case)
        snap0 = O.new_snapshot()
        snap = bytearray(snap0)
        proof, top = oracle_gkr(circ, base, ch, snap)
        assert top[0][0] == case["expect"], case["name"]
        D.check_proof(circ, base, ch, snap0, proof, top=top, after=snap)


# ---- the virtual tables ---------------------------------------------------------

def test_virtual_closed_forms_are_the_tables_extensions():
    """virtual_at_point is the multilinear extension of virtual_at_row's
    table, at every size from 0 to 20 variables (RamLive's bit 14, the bytes
    of Xor8 at 8 and 16, Range16 and Range19's masks all fall inside)."""
    rng = random.Random(3)
    for nv in list(range(0, 12)) + [13, 14, 15, 16, 17, 19, 20]:
        for kind in range(7):
            table = [D.virtual_at_row(kind, y) for y in range(1 << nv)]
            point = [rng.randrange(P) for _ in range(nv)]
            if nv <= 12:
                want = D.mle(table, point)
            else:
                out = O.buf(32)
                assert O.lib().oracle_evaluate(b"".join(O.fe(x) for x in table), ctypes.c_size_t(nv),
                                               b"".join(O.fe(x) for x in point), out) == 0
                want = O.fe_int(out.raw)
            assert D.virtual_at_point(kind, point) == want, (kind, nv)


# ---- the toy, by hand (crates/gkr/tests/oracle.rs) ----------------------------

TOY_ROWS = 16


def toy_columns(seed):
    """crates/gkr/tests/common/mod.rs toy_columns: m, a, b, c, e random u32,
    s random bits, e = a wherever s = 1 (splitmix64 draws, low 32 bits)."""
    rng = O.Rng(seed)
    draw = [[rng.next_u64() & 0xFFFFFFFF for _ in range(TOY_ROWS)] for _ in range(6)]
    m, a, b, c, e, s = draw
    s = [x & 1 for x in s]
    e = [a[y] if s[y] else e[y] for y in range(TOY_ROWS)]
    return m, a, b, c, e, s


def toy_bind(cols):
    """common/mod.rs bind: absorb the base's witness digest, then draw the
    toy's challenge (slot TOY) after it."""
    out = O.buf(32)
    assert O.lib().oracle_witness_digest(b"".join(O.fe(v) for c in cols for v in c), ctypes.c_size_t(len(cols)),
                                         ctypes.c_size_t(4), out) == 0
    snap = O.new_snapshot()
    O.transcript_op(snap, 2, 8, out.raw, 1)  # WITNESS_DIGEST
    probe = bytearray(snap)
    gamma = O.fe_int(O.transcript_op(probe, 4, 5))  # SUMCHECK_CHALLENGE
    return snap, probe, gamma


class Hand:
    """oracle.rs's Hand: the toy's layers from its description."""

    def __init__(self, cols, gamma):
        m, a, b, c, e, s = cols
        rows = range(TOY_ROWS)
        self.base = [list(x) for x in cols]
        self.ab = [a[y] * b[y] % P for y in rows]
        self.fingerprint = [(gamma * a[y] + y) * c[y] % P for y in rows]
        self.masked_m = [(m[y] * s[y] + 1 - s[y]) % P for y in rows]
        self.abm = [self.ab[y] * self.masked_m[y] % P for y in rows]
        self.fingerprint3 = [(self.fingerprint[y] + 3) % P for y in rows]
        half = TOY_ROWS // 2
        self.abm_product = [self.abm[i] * self.abm[i + half] % P for i in range(half)]
        self.fingerprint3_product = [self.fingerprint3[i] * self.fingerprint3[i + half] % P for i in range(half)]
        self.gamma = gamma

    def summand(self, which, lam, y):
        if which == 2:
            def child(t, bit):
                return D.mle(t, y + [bit])
            return (child(self.abm, 0) * child(self.abm, 1)
                    + lam * child(self.fingerprint3, 0) * child(self.fingerprint3, 1)) % P
        if which == 1:
            return (D.mle(self.ab, y) * D.mle(self.masked_m, y) + lam * (D.mle(self.fingerprint, y) + 3)) % P
        m, a, b, c, e, s = [D.mle(t, y) for t in self.base]
        row = sum((1 << j) * yj for j, yj in enumerate(y))
        l2 = lam * lam
        return (a * b + lam * (self.gamma * a + row) * c + l2 * (m * s + 1 - s) + l2 * lam * (e - a) * s) % P

    def naive(self, which, lam, p, bound, x):
        rest = len(p) - len(bound) - 1
        total = 0
        for i in range(1 << rest):
            pt = bound + [x] + [(i >> j) & 1 for j in range(rest)]
            total += D.eq(p, pt) * self.summand(which, lam, pt)
        return total % P


def check_toy_by_hand(h, proof, snap):
    """Replay oracle.rs's every_round_of_every_transition_matches_the_definition
    over a proof in the documented layout (transitions 0, 1, 2 in order)."""
    t = bytearray(snap)
    L0, L1, L2 = 4 * 4 + 6, 4 * 4 + 3, 4 * 3 + 4
    p0, p1, p2 = proof[:L0], proof[L0:L0 + L1], proof[L0 + L1:L0 + L1 + L2]
    assert len(proof) == L0 + L1 + L2
    outputs = h.fingerprint3_product + h.abm_product  # the output map: L3[1], L3[0]
    O.transcript_op(t, 2, 25, b"".join(O.fe(x) for x in outputs), len(outputs))
    r = [O.fe_int(O.transcript_op(t, 4, 26)) for _ in range(3)]
    compared = 0

    def rounds(which, lam, p, rs):
        nonlocal compared
        bound = []
        for i in range(len(rs) // 4):
            g = rs[4 * i:4 * i + 4]
            for node in range(4):
                assert D.cubic(g, node) == h.naive(which, lam, p, bound, node), (which, i, node)
                compared += 1
            O.transcript_op(t, 2, 4, b"".join(O.fe(x) for x in g), 4)
            bound.append(O.fe_int(O.transcript_op(t, 4, 5)))
        return bound

    lam = O.fe_int(O.transcript_op(t, 4, 27))
    rho = rounds(2, lam, r, p2[:12])
    claims = [D.mle(h.abm, rho + [0]), D.mle(h.abm, rho + [1]), D.mle(h.fingerprint3, rho + [0]),
              D.mle(h.fingerprint3, rho + [1])]
    assert p2[12:] == claims, "the child claims"
    O.transcript_op(t, 2, 28, b"".join(O.fe(x) for x in claims), 4)
    p = rho + [O.fe_int(O.transcript_op(t, 4, 29))]
    lam = O.fe_int(O.transcript_op(t, 4, 27))
    rho = rounds(1, lam, p, p1[:16])
    claims = [D.mle(h.ab, rho), D.mle(h.fingerprint, rho), D.mle(h.masked_m, rho)]
    assert p1[16:] == claims, "layer 1's claims"
    O.transcript_op(t, 2, 28, b"".join(O.fe(x) for x in claims), 3)
    lam = O.fe_int(O.transcript_op(t, 4, 27))
    rho = rounds(0, lam, rho, p0[:16])
    claims = [D.mle(c, rho) for c in h.base]
    assert p0[16:] == claims, "the base claims"
    O.transcript_op(t, 2, 28, b"".join(O.fe(x) for x in claims), 6)
    assert compared == 4 * (3 + 4 + 4), "every node of every round"
    return t


def toy_circuit(name):
    import artifact

    art = artifact.decode(O.golden_artifacts()[name])
    return artifact.to_circuit(art)


@pytest.mark.parametrize("name", ["toy_cached.bin", "toy_cache_free.bin"])
def test_toy_by_hand_oracle(name):
    """The oracle's proofs of the reference's toy artifacts, decoded from
    their committed bytes, equal oracle.rs's hand formulas at every node of
    every round, for the three seeds oracle.rs uses."""
    circ = toy_circuit(name)
    for seed in range(3):
        cols = toy_columns(0x53131200 + seed)
        snap, probe, gamma = toy_bind(cols)
        h = Hand(cols, gamma)
        after = bytearray(probe)
        proof, top = oracle_gkr(circ, list(cols), {0: gamma}, after)
        assert top[1] == h.fingerprint3_product and top[0] == h.abm_product
        t = check_toy_by_hand(h, proof, probe)
        assert bytes(t) == bytes(after)
        # The same proof through the generic definition and the reference verifier.
        D.check_proof(circ, list(cols), {0: gamma}, probe, proof, top=top, after=after)


def test_hand_check_rejects_a_perturbed_round():
    """oracle.rs the_oracle_rejects_a_perturbed_round: one bumped X
    coefficient of transition 2's first round agrees with the definition at
    X = 0 only; the generic check rejects it too."""
    circ = toy_circuit("toy_cached.bin")
    cols = toy_columns(0x53131300)
    snap, probe, gamma = toy_bind(cols)
    h = Hand(cols, gamma)
    proof, top = oracle_gkr(circ, list(cols), {0: gamma}, bytearray(probe))
    t = bytearray(probe)
    outputs = h.fingerprint3_product + h.abm_product
    O.transcript_op(t, 2, 25, b"".join(O.fe(x) for x in outputs), len(outputs))
    r = [O.fe_int(O.transcript_op(t, 4, 26)) for _ in range(3)]
    lam = O.fe_int(O.transcript_op(t, 4, 27))
    off = 4 * 4 + 6 + 4 * 4 + 3
    g = proof[off:off + 4]
    assert D.cubic(g, 2) == h.naive(2, lam, r, [], 2)
    broken = [g[0], (g[1] + 1) % P, g[2], g[3]]
    assert sum(D.cubic(broken, x) != h.naive(2, lam, r, [], x) for x in range(4)) == 3
    bad = list(proof)
    bad[off + 1] = (bad[off + 1] + 1) % P
    with pytest.raises(D.DefinitionMismatch):
        D.check_proof(circ, list(cols), {0: gamma}, probe, bad, top=top)
    with pytest.raises(D.DefinitionMismatch):
        D.check_proof(circ, list(cols), {0: gamma}, probe, bad, top=top, rounds=False)
    # A bumped claim fails the claims check and the verifier's final check.
    bad = list(proof)
    bad[4 * 4] = (bad[4 * 4] + 1) % P
    with pytest.raises(D.DefinitionMismatch):
        D.check_proof(circ, list(cols), {0: gamma}, probe, bad, top=top)
    with pytest.raises(D.DefinitionMismatch):
        D.check_proof(circ, list(cols), {0: gamma}, probe, bad, top=top, rounds=False)


# ---- whole proofs by definition -------------------------------------------------

def random_base(rng, circ):
    n = 1 << circ.trace_vars
    return [[rng.choice([0, 1, rng.getrandbits(32), rng.randrange(P)]) for _ in range(n)]
            for _ in range(circ.n_committed)]


def every_kind_circuit(seed, trace_vars):
    """A random circuit that reads all seven virtual tables and uses all seven
    gate shapes (random_circuit's lists plus one list of every shape)."""
    import circuits as C

    rng = random.Random(seed)
    c = C.random_circuit(rng, trace_vars, rng.randint(2, 3), rng.randint(1, 3), list(range(7)), slots=(0, 1, 2))
    w = c.width(c.depth())
    r = lambda: rng.randrange(P)  # noqa: E731
    col = lambda: C.col(rng.randrange(w))  # noqa: E731
    cac = [C.linear([(r(), C.virt(v)) for v in range(7)] + [(("ch", 1), col())], r())]
    prod = [C.linear([(r(), col()), (("ch", 0), C.cached(0))], r()), C.product(r(), col(), C.virt(2)),
            C.mask(col(), C.virt(1)), C.affine([(r(), col())], r(), [(("ch", 2), C.virt(6))], r()),
            C.quadratic(r(), [(r(), C.virt(4))], [(r(), col(), C.virt(5)), (r(), C.cached(0), col())])]
    enf = [C.product(r(), C.virt(3), col())]
    c.add_layer(prod, cached=cac, enforcing=enf)
    c.add_layer([C.tree_product(C.col(0)), C.tree_cross(C.col(1), C.col(2))], halving=True)
    return c


@pytest.mark.parametrize("seed", range(4))
def test_oracle_random_circuits_by_definition(seed):
    rng = random.Random(900 + seed)
    circ = every_kind_circuit(900 + seed, rng.choice([2, 3, 4, 5]))
    base = random_base(rng, circ)
    ch = {s: rng.randrange(P) for s in (0, 1, 2)}
    snap0 = O.new_snapshot()
    O.transcript_op(snap0, 2, 39, O.fe(seed), 1)
    after = bytearray(snap0)
    proof, top = oracle_gkr(circ, base, ch, after)
    n = D.check_proof(circ, base, ch, snap0, proof, top=top, after=after)
    assert n == 4 * sum(L[1] for L in circ.layers)


@pytest.mark.parametrize("name", ["lookup_toy.bin", "add_sub.bin", "memory_frame_mem.bin", "mul_div.bin"])
def test_oracle_artifacts_by_definition(name):
    """The reference's committed circuits (its lookup toy and family
    circuits) over 2^3 rows: the oracle's proofs by definition."""
    import artifact

    art = artifact.decode(O.golden_artifacts()[name])
    circ = artifact.to_circuit(art, min(3, art["trace_vars"]))
    rng = random.Random(sum(name.encode()))
    base = random_base(rng, circ)
    slots = sorted({c[1] for L in art["layers"] for grp in ("cached", "producing", "enforcing")
                    for e in L[grp] for c in e[-1]["coeffs"] if c[0] == "ch"} | {0})
    ch = {s: rng.randrange(P) for s in slots}
    snap0 = O.new_snapshot()
    after = bytearray(snap0)
    proof, top = oracle_gkr(circ, base, ch, after)
    D.check_proof(circ, base, ch, snap0, proof, top=top, after=after)
