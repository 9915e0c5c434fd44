"""Definition oracles for the sumcheck provers (the reference's own approach,
crates/sumcheck/tests/oracle.rs and crates/gkr/tests/oracle.rs: recompute every
round polynomial by brute force). Round and final values have no committed
golden vectors, so the CPU oracle is pinned here against the definition:

    g_i(X) = sum_{y} eq(r, (c_0..c_{i-1}, X, y)) * G(f(c_0..c_{i-1}, X, y)),

with every multilinear extension evaluated directly in Python integers."""
import ctypes
import random

import oracle_lib as O

P = O.P_R


def mle(table, point):
    t = list(table)
    for r in point:
        t = [(t[2 * i] + r * (t[2 * i + 1] - t[2 * i])) % P for i in range(len(t) // 2)]
    return t[0]


def eq(r, pt):
    acc = 1
    for a, b in zip(r, pt):
        acc = acc * (a * b + (1 - a) * (1 - b)) % P
    return acc


def cubic(g, x):
    return (((g[3] * x + g[2]) * x + g[1]) * x + g[0]) % P


def test_zerocheck_rounds_are_the_definition(oracle):
    rng = random.Random(8)
    for nv in (1, 2, 3, 4):
        n = 1 << nv
        cols = [[rng.randrange(P) for _ in range(n)] for _ in range(3)]
        terms = [(rng.randrange(P), 0, 1), (rng.randrange(P), 2, None), (3, 1, 1)]

        def gate(v):
            return (terms[0][0] * v[0] * v[1] + terms[1][0] * v[2] + terms[2][0] * v[1] * v[1]) % P

        snap0 = O.new_snapshot()
        O.transcript_op(snap0, 2, 8, O.fe(nv), 1)
        snap = bytearray(snap0)
        coefs = b"".join(O.fe(t[0]) for t in terms)
        ta = (ctypes.c_uint32 * 3)(*[t[1] for t in terms])
        tb = (ctypes.c_uint32 * 3)(*[0xFFFFFFFF if t[2] is None else t[2] for t in terms])
        rounds_b, finals_b = O.buf(128 * nv), O.buf(96)
        s = (ctypes.c_uint8 * O.SNAP).from_buffer(snap)
        assert oracle.oracle_prove_zerocheck(ctypes.c_size_t(3), coefs, ta, tb, ctypes.c_size_t(3),
                                             b"".join(O.fe(v) for c in cols for v in c), ctypes.c_size_t(nv), s,
                                             rounds_b, finals_b) == 0
        rounds = [[O.fe_int(rounds_b.raw[128 * i + 32 * j:128 * i + 32 * j + 32]) for j in range(4)]
                  for i in range(nv)]
        finals = [O.fe_int(finals_b.raw[32 * k:32 * k + 32]) for k in range(3)]
        # Replay the transcript to recover r and the challenges.
        t = bytearray(snap0)
        r = [O.fe_int(O.transcript_op(t, 4, 5)) for _ in range(nv)]
        chal = []
        for g in rounds:
            O.transcript_op(t, 2, 4, b"".join(O.fe(x) for x in g), 4)
            chal.append(O.fe_int(O.transcript_op(t, 4, 5)))
        for i, g in enumerate(rounds):
            for X in range(4):
                total = 0
                rest = nv - i - 1
                for y in range(1 << rest):
                    pt = chal[:i] + [X] + [(y >> j) & 1 for j in range(rest)]
                    total += eq(r, pt) * gate([mle(c, pt) for c in cols])
                assert total % P == cubic(g, X), f"nv={nv} round {i} X={X}"
        assert finals == [mle(c, chal) for c in cols]
        O.transcript_op(t, 2, 9, b"".join(O.fe(x) for x in finals), 3)
        assert bytes(t) == bytes(snap)


def test_gkr_rounds_chain(oracle):
    """Every layer sumcheck of the oracle's GKR proof is internally
    consistent: g_i(0) + g_i(1) = g_{i-1}(c_{i-1}) for each round."""
    import sys
    import os

    sys.path.insert(0, os.path.join(O.ROOT, "apogee-vm_gb300"))
    import circuits as C

    for seed in range(4):
        rng = random.Random(seed)
        c = C.random_circuit(rng, rng.choice([3, 4, 5]), rng.randint(1, 3), rng.randint(2, 4),
                             rng.sample(range(7), 2), slots=(0, 1, 2))
        blob = c.to_blob()
        n = 1 << c.trace_vars
        base = b"".join(O.fe(rng.randrange(P)) for _ in range(n * c.n_committed))
        slots = (ctypes.c_uint32 * 3)(0, 1, 2)
        vals = b"".join(O.fe(v) for v in (11, 12, 13))
        snap = bytearray(O.new_snapshot())
        sb = (ctypes.c_uint8 * O.SNAP).from_buffer(snap)
        pr = O.buf(32 * c.proof_elems())
        top = O.buf(32 * c.width(c.depth()) * (1 << c.vars(c.depth())))
        assert oracle.oracle_gkr_prove(blob, ctypes.c_size_t(len(blob)), base, slots, vals, ctypes.c_size_t(3), sb,
                                       pr, top) == 0
        proof = [O.fe_int(pr.raw[32 * i:32 * i + 32]) for i in range(c.proof_elems())]
        # Replay the transcript schedule to recover each round's challenge.
        t = O.new_snapshot()
        t = bytearray(t)
        topw, topn = c.width(c.depth()), 1 << c.vars(c.depth())
        outs = [O.fe_int(top.raw[32 * i:32 * i + 32]) for i in range(topw * topn)]
        O.transcript_op(t, 2, 25, b"".join(O.fe(x) for x in outs), len(outs))
        for _ in range(c.vars(c.depth())):
            O.transcript_op(t, 4, 26)
        offs = []
        off = 0
        for k in range(c.depth()):
            nk = c.vars(k + 1)
            claims = (2 if c.layers[k][0] else 1) * c.width(k)
            offs.append((off, nk, claims))
            off += 4 * nk + claims
        for k in reversed(range(c.depth())):
            o, nk, claims = offs[k]
            O.transcript_op(t, 4, 27)
            prev = None
            for i in range(nk):
                g = proof[o + 4 * i:o + 4 * i + 4]
                if prev is not None:
                    assert (cubic(g, 0) + cubic(g, 1)) % P == prev
                O.transcript_op(t, 2, 4, b"".join(O.fe(x) for x in g), 4)
                ci = O.fe_int(O.transcript_op(t, 4, 5))
                prev = cubic(g, ci)
            cl = proof[o + 4 * nk:o + 4 * nk + claims]
            O.transcript_op(t, 2, 28, b"".join(O.fe(x) for x in cl), claims)
            if c.layers[k][0]:
                O.transcript_op(t, 4, 29)
        assert bytes(t) == bytes(snap)
