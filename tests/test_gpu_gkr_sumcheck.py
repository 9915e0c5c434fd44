"""apg_gkr_prove_sumcheck, gkr::prove_sumcheck on its own
(crates/gkr/src/lib.rs:792): one gate list's sumcheck over the caller's
device tables with the caller's weights, eq point, challenges and
transcript. Every round, the bound point, the tables' bound values and the
transcript after it equal the oracle's restatement of the same function, for
every gate list of seeded random circuits (all gate shapes, cached entries,
enforcing gates, virtual tables, halving lists) and of the reference's own
add_sub artifact; the reference's refusal cases map to InvalidArgument."""
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


def _device(torch, vals):
    import apogee_gpu as A

    return torch.frombuffer(bytearray(A.to_mont_bytes(vals)), dtype=torch.uint8).to("cuda:0")


def oracle_sumcheck(blob, k, weights, challenges, point, lower, upper, snap):
    slots = sorted(challenges)
    sarr = (ctypes.c_uint32 * max(len(slots), 1))(*slots)
    vals = b"".join(O.fe(challenges[s]) for s in slots)
    n, width = len(point), len(lower)
    s = (ctypes.c_uint8 * O.SNAP).from_buffer(snap)
    rounds, pt, finals = O.buf(128 * max(n, 1)), O.buf(32 * max(n, 1)), O.buf(64 * max(width, 1))
    rc = O.lib().oracle_gkr_prove_sumcheck(
        blob, ctypes.c_size_t(len(blob)), ctypes.c_size_t(k), b"".join(O.fe(w) for w in weights),
        ctypes.c_size_t(len(weights)), sarr, vals, ctypes.c_size_t(len(slots)), b"".join(O.fe(x) for x in point),
        ctypes.c_size_t(n), b"".join(O.fe(v) for t in lower for v in t),
        b"".join(O.fe(v) for t in upper for v in t) if upper else None, ctypes.c_size_t(width), s, rounds, pt, finals)
    assert rc == 0
    r = [O.fe_int(rounds.raw[32 * i:32 * i + 32]) for i in range(4 * n)]
    nf = width * (2 if upper else 1)
    return ([tuple(r[4 * i:4 * i + 4]) for i in range(n)], [O.fe_int(pt.raw[32 * i:32 * i + 32]) for i in range(n)],
            [O.fe_int(finals.raw[32 * i:32 * i + 32]) for i in range(nf)])


def check_circuit(ctx, circuit, seed, slots):
    import torch

    import apogee_gpu as A

    rng = random.Random(seed)
    blob = circuit.to_blob()
    challenges = {s: rng.randrange(O.P_R) for s in slots}
    for k, (halving, n, _w, _cac, prod, enf) in enumerate(circuit.layers):
        width = circuit.width(k)
        draw = lambda: [rng.choice([0, 1, rng.getrandbits(32), rng.randrange(O.P_R)]) for _ in range(1 << n)]  # noqa: E731
        lower = [draw() for _ in range(width)]
        upper = [draw() for _ in range(width)] if halving else []
        weights = [rng.randrange(O.P_R) for _ in range(len(prod) + len(enf))]
        point = [rng.randrange(O.P_R) for _ in range(n)]
        snap = A.transcript_append_scalars(A.transcript_init(), 41, [seed, k])
        d_lo = [_device(torch, t) for t in lower]
        d_up = [_device(torch, t) for t in upper]
        got = ctx.gkr_prove_sumcheck(blob, k, weights, challenges, point, [t.data_ptr() for t in d_lo],
                                     [t.data_ptr() for t in d_up] if halving else None, snap)
        osnap = bytearray(snap)
        want = oracle_sumcheck(blob, k, weights, challenges, point, lower, upper, osnap)
        assert got[0] == want[0], f"list {k}: rounds"
        assert got[1] == want[1], f"list {k}: point"
        assert got[2] == want[2], f"list {k}: bound tables"
        assert got[3] == bytes(osnap), f"list {k}: transcript"
        # The caller's tables are read, not bound.
        assert bytes(d_lo[0].cpu().numpy().tobytes()) == A.to_mont_bytes(lower[0])


@pytest.mark.parametrize("seed", range(4))
def test_random_circuit_lists_match_oracle(ctx, seed):
    import circuits as C

    rng = random.Random(300 + seed)
    virtuals = rng.sample(range(7), rng.randint(0, 3))
    c = C.random_circuit(rng, rng.choice([3, 5, 8, 11]), rng.randint(1, 4), rng.randint(2, 4), virtuals,
                         slots=(0, 1, 2))
    check_circuit(ctx, c, seed, (0, 1, 2))


def test_shard_circuit_lists_match_oracle(ctx):
    """The shard circuit's row-wise list (cached row-index term, enforcing
    gate, virtual row table) and its halving tree-product lists at 2^9 rows:
    the generic, pair-term and small-round kernels all run."""
    import circuits as C

    check_circuit(ctx, C.shard_circuit(9, 4), 9, (0,))


def test_reference_add_sub_lists_match_oracle(ctx):
    import artifact

    art = artifact.decode(O.golden_artifacts()["add_sub.bin"])
    circuit = artifact.to_circuit(art, 5)
    slots = sorted({c[1] for L in art["layers"] for grp in ("cached", "producing", "enforcing")
                    for e in L[grp] for c in e[-1]["coeffs"] if c[0] == "ch"} | {0})
    check_circuit(ctx, circuit, 11, slots)


def test_refusals(ctx):
    import torch

    import apogee_gpu as A
    import circuits as C

    c = C.Circuit(4, 2)
    c.add_layer([C.product(1, C.col(0), C.col(1))])
    blob = c.to_blob()
    t = [_device(torch, [1] * 16), _device(torch, [2] * 16)]
    ptrs = [x.data_ptr() for x in t]
    snap = A.transcript_init()
    point = [3, 4, 5, 6]
    assert ctx.gkr_prove_sumcheck(blob, 0, [1], {}, point, ptrs, None, snap)[0]  # the valid call
    for layer, weights, pt, tables in ((1, [1], point, ptrs),      # no such list
                                       (0, [1, 2], point, ptrs),   # one weight a gate
                                       (0, [1], point[:3], ptrs),  # eq point of the wrong length
                                       (0, [1], point, ptrs[:1]),   # a column missing
                                       (0, [1], point, [ptrs[0], 0])):  # a null table
        with pytest.raises(A.ApogeeError) as e:
            ctx.gkr_prove_sumcheck(blob, layer, weights, {}, pt, tables, None, snap)
        assert e.value.variant == "InvalidArgument"
