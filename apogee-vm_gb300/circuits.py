"""Circuits as data for the GKR entry points: a small builder for the APGC
blob (the resolved gate-list form include/apogee_gpu.h documents) and the
synthetic shard circuits the workloads use.

Gate shapes follow constraints::GateDef (crates/constraints/src/lib.rs:310-358)
with operands in GateDef::operands order and coefficients in
GateDef::coefficients order. A coefficient is an int literal (canonical Fr)
or ("ch", slot) for an external challenge slot.
"""
import random
import struct

P_R = 21888242871839275222246405745257275088548364400416034343698204186575808495617

LINEAR, PRODUCT, MASK, AFFINE, TREE_PRODUCT, TREE_CROSS, QUADRATIC = range(7)
V_ROW, V_RAM_LIVE, V_RANGE19, V_RANGE16, V_XOR8A, V_XOR8B, V_XOR8OUT = range(7)


def col(i):
    return (0, i)


def virt(i):
    return (1, i)


def cached(j):
    return (2, j)


def linear(terms, const=0):
    return (LINEAR, len(terms), 0, [op for _, op in terms], [c for c, _ in terms] + [const])


def product(coef, x, y):
    return (PRODUCT, 0, 0, [x, y], [coef])


def mask(x, m):
    return (MASK, 0, 0, [x, m], [])


def affine(left, left_const, right, right_const):
    return (AFFINE, len(left), len(right), [op for _, op in left] + [op for _, op in right],
            [c for c, _ in left] + [left_const] + [c for c, _ in right] + [right_const])


def tree_product(x):
    return (TREE_PRODUCT, 0, 0, [x], [])


def tree_cross(p, q):
    return (TREE_CROSS, 0, 0, [p, q], [])


def quadratic(const, lin, prods):
    ops = [op for _, op in lin]
    for _, y, z in prods:
        ops += [y, z]
    return (QUADRATIC, len(lin), len(prods), ops, [const] + [c for c, _ in lin] + [c for c, _, _ in prods])


class Circuit:
    def __init__(self, trace_vars: int, n_committed: int, virtuals=()):
        self.trace_vars = trace_vars
        self.n_committed = n_committed
        self.virtuals = list(virtuals)
        self.layers = []  # (halving, num_vars, width, cached, producing, enforcing)
        self.outputs = None

    def vars(self, k):
        return self.trace_vars if k == 0 else self.layers[k - 1][1]

    def width(self, k):
        return self.n_committed if k == 0 else self.layers[k - 1][2]

    def add_layer(self, producing, cached=(), enforcing=(), halving=False):
        k = len(self.layers)
        nv = self.vars(k) - (1 if halving else 0)
        self.layers.append((halving, nv, len(producing), list(cached), list(producing), list(enforcing)))
        return self

    def depth(self):
        return len(self.layers)

    def to_blob(self) -> bytes:
        out = [struct.pack("<5I", 0x43475041, 1, self.trace_vars, self.n_committed, len(self.virtuals))]
        out.append(b"".join(struct.pack("<I", v) for v in self.virtuals))
        outs = self.outputs if self.outputs is not None else list(range(self.width(self.depth())))
        out.append(struct.pack("<I", len(outs)) + b"".join(struct.pack("<I", o) for o in outs))
        out.append(struct.pack("<I", len(self.layers)))
        for halving, nv, width, cac, prod, enf in self.layers:
            out.append(struct.pack("<6I", 1 if halving else 0, nv, width, len(cac), len(prod), len(enf)))
            for kind, p1, p2, ops, coeffs in cac + prod + enf:
                out.append(struct.pack("<4I", kind, p1, p2, len(ops)))
                out.append(b"".join(struct.pack("<2I", s, i) for s, i in ops))
                out.append(struct.pack("<I", len(coeffs)))
                for c in coeffs:
                    if isinstance(c, tuple):
                        out.append(struct.pack("<2I", 1, c[1]))
                    else:
                        out.append(struct.pack("<I", 0) + (int(c) % P_R).to_bytes(32, "little"))
        return b"".join(out)

    def proof_elems(self):
        n = 0
        for k, (halving, nv, _w, _c, _p, _e) in enumerate(self.layers):
            n += 4 * nv + (2 if halving else 1) * self.width(k)
        return n


def random_circuit(rng: random.Random, trace_vars: int, n_committed: int, depth: int, virtuals=(),
                   slots=(1, 2)) -> Circuit:
    """A circuit exercising every gate shape: row-wise lists with cached
    entries, enforcing gates, virtual tables and challenge coefficients,
    and halving lists of TreeProduct / TreeCross."""
    c = Circuit(trace_vars, n_committed, virtuals)

    def coeff():
        return ("ch", rng.choice(slots)) if rng.random() < 0.2 else rng.randrange(P_R)

    for k in range(depth):
        w = c.width(k)
        if c.vars(k) >= 1 and rng.random() < 0.35:
            gates = []
            for j in range(rng.randint(1, 4)):
                if rng.random() < 0.5:
                    gates.append(tree_product(col(rng.randrange(w))))
                else:
                    gates.append(tree_cross(col(rng.randrange(w)), col(rng.randrange(w))))
            c.add_layer(gates, halving=True)
            continue
        nv = len(virtuals)
        cac = []
        for j in range(rng.randint(0, 2)):
            srcs = [col(rng.randrange(w))] + ([virt(rng.randrange(nv))] if nv else [])
            srcs += [cached(rng.randrange(j))] if j else []
            cac.append(linear([(coeff(), rng.choice(srcs)) for _ in range(rng.randint(1, 3))], coeff()))

        def operand():
            pool = [col(rng.randrange(w))]
            if nv:
                pool.append(virt(rng.randrange(nv)))
            if cac:
                pool.append(cached(rng.randrange(len(cac))))
            return rng.choice(pool)

        def gate():
            kind = rng.randrange(5)
            if kind == 0:
                return linear([(coeff(), operand()) for _ in range(rng.randint(1, 3))], coeff())
            if kind == 1:
                return product(coeff(), operand(), operand())
            if kind == 2:
                return mask(operand(), operand())
            if kind == 3:
                return affine([(coeff(), operand()) for _ in range(rng.randint(1, 2))], coeff(),
                              [(coeff(), operand()) for _ in range(rng.randint(1, 2))], coeff())
            return quadratic(coeff(), [(coeff(), operand()) for _ in range(rng.randint(0, 2))],
                             [(coeff(), operand(), operand()) for _ in range(rng.randint(1, 2))])

        prod = [gate() for _ in range(rng.randint(1, 4))]
        enf = [gate() for _ in range(rng.randint(0, 2))]
        c.add_layer(prod, cached=cac, enforcing=enf)
    return c


def shard_circuit(vars_: int = 20, width: int = 8) -> Circuit:
    """The single-execution-shard circuit: 12 gate lists over `width`
    committed columns at 2^vars rows -- lists 0-3 row-wise at vars, list 4
    halving, lists 5-7 row-wise at vars-1, list 8 halving, lists 9-11
    row-wise at vars-2 -- so the layer sumchecks run over vars, vars, vars,
    vars, vars-1, vars-1, vars-1, vars-1, vars-2, ... variables. Row-wise
    lists mix degree-2 gates (Product, AffineProduct, MaskIntoIdentity,
    Quadratic, Linear) with a cached sub-expression over the row index and
    one enforcing gate; the top list narrows to one output column."""
    c = Circuit(vars_, width, [V_ROW])
    gamma = ("ch", 0)
    for k in range(12):
        w = c.width(k)
        if k in (4, 8):
            gates = []
            for j in range(width):
                if j % 2 == 0:
                    gates.append(tree_product(col(j)))
                else:
                    gates.append(tree_cross(col(j), col((j + 1) % w)))
            c.add_layer(gates, halving=True)
            continue
        cac = [linear([(gamma, col(0)), (1, virt(0))], 0)]  # gamma * x_0 + row
        out_w = 1 if k == 11 else width
        prod = []
        for j in range(out_w):
            a, b = col(j % w), col((j + 1) % w)
            kind = (j + k) % 5
            if kind == 0:
                prod.append(product(3, a, b))
            elif kind == 1:
                prod.append(affine([(1, a), (2, cached(0))], 5, [(1, b)], 7))
            elif kind == 2:
                prod.append(mask(a, b))
            elif kind == 3:
                prod.append(quadratic(1, [(4, a)], [(gamma, b, cached(0)), (P_R - 1, a, b)]))
            else:
                prod.append(linear([(1, a), (9, b), (2, cached(0))], 11))
        enf = [quadratic(0, [(1, col(0)), (P_R - 1, col(1 % w))], [(1, col(0), col(1 % w))])]
        c.add_layer(prod, cached=cac, enforcing=enf)
    return c
