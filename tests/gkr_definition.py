"""The GKR prover's semantics by definition, in Python integers: test
infrastructure, written from the reference's specification and independent
of both the C++ oracle (oracle/prover.hpp) and the CUDA library.

It restates, for a circuit in the APGC form of circuits.py:

* the gate kernel `eval_gate` (crates/gkr-verify/src/lib.rs:142-202) and the
  virtual tables at a row (`virtual_at_row`, :205-232) and at a point
  (`virtual_at_point`, :245-286);
* the resolved gate list (`ResolvedList`, :300-480): cached entries first,
  then producing, then enforcing gates; a halving list reads every column
  operand at child 0 then child 1;
* the forward pass (`gkr::forward`, crates/gkr/src/lib.rs:279-336);
* the verifier (`gkr_verify::verify`, lib.rs:640-748), including the final
  check of every transition and the child merge of halving lists, and the
  discharge of its base claims against the base columns
  (crates/gkr/tests/common/mod.rs `discharge`);
* and, in the manner of crates/gkr/tests/oracle.rs, every round polynomial of
  every transition recomputed at its four nodes X = 0..3 as the direct sum
  over the rest of the cube of eq(p, (c, X, rest)) * S(c, X, rest), each
  column and each virtual table read as the multilinear extension of its
  table (not through a closed form).

The transcript (Poseidon2 duplex) is the one shared primitive; it comes from
oracle_lib, pinned by the reference's 128 permutation vectors and transcript
scripts.
"""
import oracle_lib as O

P = O.P_R
RAM_LIVE_BIT = 14  # crates/constants/src/lib.rs:1922

# Shape and virtual-kind numbers of the APGC form (circuits.py).
LINEAR, PRODUCT, MASK, AFFINE, TREE_PRODUCT, TREE_CROSS, QUADRATIC = range(7)
V_ROW, V_RAM_LIVE, V_RANGE19, V_RANGE16, V_XOR8A, V_XOR8B, V_XOR8OUT = range(7)

# Transcript tags (crates/constants/src/lib.rs transcript_tags).
T_SUMCHECK_ROUND, T_SUMCHECK_CHALLENGE = 4, 5
T_GKR_OUTPUTS, T_GKR_OUTPUT_POINT, T_GKR_BATCH, T_GKR_LAYER_CLAIMS, T_GKR_CHILD = 25, 26, 27, 28, 29


class DefinitionMismatch(AssertionError):
    pass


# ---- the kernel --------------------------------------------------------------

def coefficient(c, challenges):
    """A literal or an external challenge slot's value (lib.rs:127-134)."""
    if isinstance(c, tuple):
        return challenges[c[1]] % P
    return c % P


def eval_gate(gate, v, challenges):
    """`eval_gate` (lib.rs:142-202): one gate at one point, `v` holding one
    value per operand in operand order (two per column for a halving gate)."""
    shape, t, u, ops, cs = gate
    c = [coefficient(x, challenges) for x in cs]
    if shape == LINEAR:
        # terms zip values, starting from the constant (the last coefficient).
        acc = c[len(ops)]
        for i in range(len(ops)):
            acc += c[i] * v[i]
        return acc % P
    if shape == PRODUCT:
        return c[0] * v[0] * v[1] % P
    if shape == MASK:
        return (v[0] * v[1] + 1 - v[1]) % P
    if shape == AFFINE:
        # coefficients: left terms, left constant, right terms, right constant.
        left = c[t] + sum(c[i] * v[i] for i in range(t))
        right = c[t + 1 + u] + sum(c[t + 1 + j] * v[t + j] for j in range(u))
        return left * right % P
    if shape == TREE_PRODUCT:
        return v[0] * v[1] % P
    if shape == TREE_CROSS:
        # p(.,0) q(.,1) + p(.,1) q(.,0): operands p then q, each at child 0 then 1.
        return (v[0] * v[3] + v[1] * v[2]) % P
    if shape == QUADRATIC:
        # coefficients: constant, linear terms, product terms.
        acc = c[0] + sum(c[1 + i] * v[i] for i in range(t))
        for j in range(u):
            acc += c[1 + t + j] * v[t + 2 * j] * v[t + 2 * j + 1]
        return acc % P
    raise ValueError(f"gate shape {shape}")


def virtual_at_row(kind, row):
    """lib.rs:205-232."""
    if kind == V_ROW:
        return row
    if kind == V_RAM_LIVE:
        return 1 if row >= 1 << RAM_LIVE_BIT else 0
    if kind == V_RANGE19:
        return row & ((1 << 19) - 1)
    if kind == V_RANGE16:
        return row & ((1 << 16) - 1)
    if kind == V_XOR8A:
        return row & 0xFF
    if kind == V_XOR8B:
        return (row >> 8) & 0xFF
    if kind == V_XOR8OUT:
        return (row & 0xFF) ^ ((row >> 8) & 0xFF)
    raise ValueError(f"virtual kind {kind}")


def virtual_at_point(kind, point):
    """The closed forms of lib.rs:245-286 (what the verifier uses)."""
    def horner(lo, hi):
        acc = 0
        for j in reversed(range(lo, hi)):
            acc = (2 * acc + (point[j] if j < len(point) else 0)) % P
        return acc

    n = len(point)
    if kind == V_ROW:
        return horner(0, n)
    if kind == V_RAM_LIVE:
        prod = 1
        for y in point[min(n, RAM_LIVE_BIT):]:
            prod = prod * (1 - y) % P
        return (1 - prod) % P
    if kind == V_RANGE19:
        return horner(0, min(n, 19))
    if kind == V_RANGE16:
        return horner(0, min(n, 16))
    if kind == V_XOR8A:
        return horner(0, 8)
    if kind == V_XOR8B:
        return horner(8, 16)
    if kind == V_XOR8OUT:
        acc = 0
        for j in reversed(range(8)):
            y = point[j] if j < n else 0
            z = point[j + 8] if j + 8 < n else 0
            acc = (2 * acc + y + z - 2 * y * z) % P
        return acc
    raise ValueError(f"virtual kind {kind}")


# ---- multilinear helpers -------------------------------------------------------

def bind(table, r):
    """Fix variable 0 (the low bit of the index) to r (crates/poly/src/lib.rs:156-185)."""
    return [(table[2 * i] + r * (table[2 * i + 1] - table[2 * i])) % P for i in range(len(table) // 2)]


def mle(table, point):
    t = [x % P for x in table]
    for r in point:
        t = bind(t, r)
    assert len(t) == 1
    return t[0]


def eq(p, y):
    acc = 1
    for a, b in zip(p, y):
        acc = acc * (a * b + (1 - a) * (1 - b)) % P
    return acc


def cubic(g, x):
    return (((g[3] * x + g[2]) * x + g[1]) * x + g[0]) % P


def powers(x, n):
    out, acc = [], 1
    for _ in range(n):
        out.append(acc)
        acc = acc * x % P
    return out


# ---- gate lists ------------------------------------------------------------------

def gate_values(circ, k, lower, upper, virtuals, challenges):
    """Every producing then enforcing gate of list k at one point, cached
    entries evaluated first and substituted (`ResolvedList`, lib.rs:300-480)."""
    halving, _nv, _w, cac, prod, enf = circ.layers[k]
    if halving:
        out = []
        for g in prod:
            v = []
            for src, x in g[3]:
                assert src == 0, "a halving gate reads columns only"
                v += [lower[x], upper[x]]
            out.append(eval_gate(g, v, challenges))
        return out
    cached = []

    def read(op):
        src, x = op
        return lower[x] if src == 0 else virtuals[x] if src == 1 else cached[x]

    for g in cac:
        cached.append(eval_gate(g, [read(op) for op in g[3]], challenges))
    return [eval_gate(g, [read(op) for op in g[3]], challenges) for g in prod + enf]


def summand(circ, k, weights, lower, upper, virtuals, challenges):
    vals = gate_values(circ, k, lower, upper, virtuals, challenges)
    assert len(vals) == len(weights)
    return sum(w * v for w, v in zip(weights, vals)) % P


def forward(circ, base, challenges, enforcing=None):
    """`gkr::forward`: layers[0] = the base, layers[k + 1] = list k's
    producing gates at every row (a halving list's row y reads rows y and
    y + rows of the layer below). With a list `enforcing`, also appends per
    gate list the value tables of its enforcing gates over its rows."""
    layers = [[[x % P for x in col] for col in base]]
    for k, (halving, _nv, width, _c, _p, _e) in enumerate(circ.layers):
        cols = layers[k]
        rows_in = 1 << circ.vars(k)
        rows = rows_in // 2 if halving else rows_in
        kinds = circ.virtuals
        n_enf = 0 if halving else len(circ.layers[k][5])
        out = [[0] * rows for _ in range(width + n_enf)]
        for y in range(rows):
            lower = [c[y] for c in cols]
            upper = [c[y + rows] for c in cols] if halving else []
            virt = [] if halving else [virtual_at_row(kd, y) for kd in kinds]
            vals = gate_values(circ, k, lower, upper, virt, challenges)
            for j in range(width + n_enf):
                out[j][y] = vals[j]
        layers.append(out[:width])
        if enforcing is not None:
            enforcing.append(out[width:])
    return layers


def outputs_of(circ):
    return circ.outputs if circ.outputs is not None else list(range(circ.width(circ.depth())))


def split_proof(circ, proof):
    """The proof's documented layout: per gate list k, its rounds (4 values
    each) then its claims (two per column for a halving list)."""
    parts, off = [], 0
    for k, (halving, nv, _w, _c, _p, _e) in enumerate(circ.layers):
        rounds = [proof[off + 4 * i:off + 4 * i + 4] for i in range(nv)]
        off += 4 * nv
        nclaims = (2 if halving else 1) * circ.width(k)
        parts.append((rounds, proof[off:off + nclaims]))
        off += nclaims
    if off != len(proof):
        raise DefinitionMismatch(f"proof has {len(proof)} values, the circuit's layout {off}")
    return parts


# ---- the verifier --------------------------------------------------------------

def verify(circ, top, proof, challenges, snap, enforcing=None):
    """`gkr_verify::verify` (lib.rs:640-748) with the outputs `top` (the top
    layer's columns) as the claimed output tables: returns the base point
    and the base claim values; advances `snap` (a bytearray) in place.
    Raises DefinitionMismatch where the reference verifier rejects.

    The reference verifier takes every enforcing gate's claim to be zero (a
    satisfied circuit). A random circuit's enforcing gates need not vanish,
    so `enforcing` (per gate list, the enforcing gates' value tables over its
    rows, from `forward`) adds their weighted values at the point to the
    claim; without it the check is the reference's exactly."""
    depth = circ.depth()
    parts = split_proof(circ, proof)
    outs = outputs_of(circ)
    msg = b"".join(O.fe(x) for off in outs for x in top[off])
    O.transcript_op(snap, 2, T_GKR_OUTPUTS, msg, sum(len(top[off]) for off in outs))
    point = [O.fe_int(O.transcript_op(snap, 4, T_GKR_OUTPUT_POINT)) for _ in range(circ.vars(depth))]
    values = [0] * len(outs)
    for off in outs:
        values[off] = mle(top[off], point)
    for k in reversed(range(depth)):
        halving, _nv, _w, _c, prod, enf = circ.layers[k]
        rounds, evals = parts[k]
        lam = O.fe_int(O.transcript_op(snap, 4, T_GKR_BATCH))
        weights = powers(lam, len(prod) + len(enf))
        claim = sum(v * w for v, w in zip(values, weights)) % P
        if enforcing is not None:
            for e, table in enumerate(enforcing[k]):
                claim = (claim + weights[len(prod) + e] * mle(table, point)) % P
        rho = []
        for i, g in enumerate(rounds):
            if (cubic(g, 0) + cubic(g, 1)) % P != claim:
                raise DefinitionMismatch(f"transition {k} round {i}: g(0) + g(1) is not the claim")
            O.transcript_op(snap, 2, T_SUMCHECK_ROUND, b"".join(O.fe(x) for x in g), 4)
            r = O.fe_int(O.transcript_op(snap, 4, T_SUMCHECK_CHALLENGE))
            claim = cubic(g, r)
            rho.append(r)
        O.transcript_op(snap, 2, T_GKR_LAYER_CLAIMS, b"".join(O.fe(x) for x in evals), len(evals))
        if halving:
            s = summand(circ, k, weights, evals[0::2], evals[1::2], [], challenges)
        else:
            virt = [virtual_at_point(kd, rho) for kd in circ.virtuals]
            s = summand(circ, k, weights, evals, [], virt, challenges)
        if claim != eq(point, rho) * s % P:
            raise DefinitionMismatch(f"transition {k}: the final check fails")
        if halving:
            tau = O.fe_int(O.transcript_op(snap, 4, T_GKR_CHILD))
            values = [(evals[2 * i] + tau * (evals[2 * i + 1] - evals[2 * i])) % P for i in range(len(evals) // 2)]
            point = rho + [tau]
        else:
            values = list(evals)
            point = rho
    return point, values


def discharge(base, point, values):
    """Every base claim against the column it names (the opening's job)."""
    for j, (col, v) in enumerate(zip(base, values)):
        if mle(col, point) != v:
            raise DefinitionMismatch(f"base column {j}: the claim is not the column's value at the point")


# ---- every round by definition -------------------------------------------------

def check_rounds_by_definition(circ, layers, proof, challenges, snap):
    """crates/gkr/tests/oracle.rs generalised to any circuit: replay the
    transcript schedule (docs/spec/gkr.md 5.2) and hold every round of every
    transition to the direct sum of eq * S over the remaining cube at its
    four nodes; hold every transition's claims to the columns' values at the
    bound point, and round 0 of every transition to the batched claim
    sum_y eq(p, y) S(y) over the cube. Returns the number of nodes compared.
    Advances `snap` (a bytearray) in place."""
    depth = circ.depth()
    parts = split_proof(circ, proof)
    top = layers[depth]
    outs = outputs_of(circ)
    msg = b"".join(O.fe(x) for off in outs for x in top[off])
    O.transcript_op(snap, 2, T_GKR_OUTPUTS, msg, sum(len(top[off]) for off in outs))
    p = [O.fe_int(O.transcript_op(snap, 4, T_GKR_OUTPUT_POINT)) for _ in range(circ.vars(depth))]
    compared = 0
    for k in reversed(range(depth)):
        halving, nk, _w, _c, prod, enf = circ.layers[k]
        rounds, evals = parts[k]
        lam = O.fe_int(O.transcript_op(snap, 4, T_GKR_BATCH))
        weights = powers(lam, len(prod) + len(enf))
        cols = layers[k]
        if halving:
            half = len(cols[0]) // 2
            lo = [c[:half] for c in cols]
            up = [c[half:] for c in cols]
            vt = []
        else:
            lo, up = [list(c) for c in cols], []
            vt = [[virtual_at_row(kd, y) for y in range(1 << nk)] for kd in circ.virtuals]
        # The batched claim over the cube, by definition.
        claim = 0
        for y in range(1 << nk):
            yb = [(y >> j) & 1 for j in range(nk)]
            s = summand(circ, k, weights, [c[y] for c in lo], [c[y] for c in up], [c[y] for c in vt], challenges)
            claim += eq(p, yb) * s
        claim %= P
        if rounds and (cubic(rounds[0], 0) + cubic(rounds[0], 1)) % P != claim:
            raise DefinitionMismatch(f"transition {k}: round 0 does not sum to the batched claim")
        bound = []
        for i, g in enumerate(rounds):
            rest = nk - i - 1
            for x in range(4):
                total = 0
                for r in range(1 << rest):
                    def line(t):
                        return (t[2 * r] + x * (t[2 * r + 1] - t[2 * r])) % P
                    pt = bound + [x] + [(r >> j) & 1 for j in range(rest)]
                    s = summand(circ, k, weights, [line(t) for t in lo], [line(t) for t in up],
                                [line(t) for t in vt], challenges)
                    total += eq(p, pt) * s
                if total % P != cubic(g, x):
                    raise DefinitionMismatch(f"transition {k} round {i} differs from the definition at X = {x}")
                compared += 1
            O.transcript_op(snap, 2, T_SUMCHECK_ROUND, b"".join(O.fe(v) for v in g), 4)
            c = O.fe_int(O.transcript_op(snap, 4, T_SUMCHECK_CHALLENGE))
            bound.append(c)
            lo = [bind(t, c) for t in lo]
            up = [bind(t, c) for t in up]
            vt = [bind(t, c) for t in vt]
        if halving:
            want = [v for a, b in zip(lo, up) for v in (a[0], b[0])]
        else:
            want = [t[0] for t in lo]
        if list(evals) != want:
            raise DefinitionMismatch(f"transition {k}: the claims are not the columns at the bound point")
        O.transcript_op(snap, 2, T_GKR_LAYER_CLAIMS, b"".join(O.fe(v) for v in evals), len(evals))
        p = bound
        if halving:
            p = p + [O.fe_int(O.transcript_op(snap, 4, T_GKR_CHILD))]
    return compared


def check_proof(circ, base, challenges, snap, proof, top=None, after=None, rounds=True):
    """The whole pin for one proof: forward by definition (and the top layer
    against `top` if given), every round by definition (if `rounds`), the
    reference verifier, the discharge of the base claims, and the transcript
    state after the proof against `after` if given."""
    enforcing = []
    layers = forward(circ, base, challenges, enforcing)
    if top is not None:
        want = layers[circ.depth()]
        for j, col in enumerate(top):
            if [x % P for x in col] != want[j]:
                raise DefinitionMismatch(f"top layer column {j} is not the forward pass by definition")
    compared = 0
    if rounds:
        s1 = bytearray(snap)
        compared = check_rounds_by_definition(circ, layers, proof, challenges, s1)
    s2 = bytearray(snap)
    point, values = verify(circ, layers[circ.depth()], proof, challenges, s2, enforcing)
    discharge(layers[0], point, values)
    if rounds:
        assert s1 == s2
    if after is not None and bytes(s2) != bytes(after):
        raise DefinitionMismatch("the transcript after the proof differs from the schedule's")
    return compared
