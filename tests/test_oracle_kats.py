"""Pin the CPU oracle against the reference's committed known-answer vectors
(tests/golden/, extracted by tests/golden/make_golden.py).

Each test replays one fixture the way the reference's own suite does:
crates/field/tests, crates/curve/tests/{fq,g1,msm}.rs, crates/poly/tests,
crates/transcript/tests/{poseidon2,cases}.rs and crates/pcs/tests/kats.rs.
"""
import ctypes
import random

import pytest

import oracle_lib as O
from oracle_lib import buf, fe, hexb


def _field_kats(fn, fname, kinds):
    n = 0
    for line in O.golden_lines(fname):
        f = line.split()
        kind = f[0]
        if kind not in kinds:
            continue
        n += 1
        yield kind, f


def test_fr_kats(oracle):
    ops = {"add": 0, "sub": 1, "mul": 2}
    checked = 0
    for line in O.golden_lines("fr_kats.txt"):
        f = line.split()
        out = buf(32)
        if f[0] in ops:
            assert oracle.oracle_fr_op(ops[f[0]], hexb(f[1]), hexb(f[2]), out) == 0
            assert out.raw.hex() == f[3], line
        elif f[0] == "square":
            assert oracle.oracle_fr_op(3, hexb(f[1]), None, out) == 0
            assert out.raw.hex() == f[2]
        elif f[0] == "inv":
            rc = oracle.oracle_fr_op(4, hexb(f[1]), None, out)
            if f[2] == "none":
                assert rc == 1
            else:
                assert rc == 0 and out.raw.hex() == f[2]
        elif f[0] == "pow":
            assert oracle.oracle_fr_op(5, hexb(f[1]), hexb(f[2]), out) == 0
            assert out.raw.hex() == f[3]
        else:
            continue
        checked += 1
    assert checked == 536


def test_fq_kats(oracle):
    checked = 0
    for line in O.golden_lines("fq_kats.txt"):
        f = line.split()
        out = buf(32)
        if f[0] == "fq_ops":
            a, b = hexb(f[1]), hexb(f[2])
            for op, want in ((0, f[3]), (1, f[4]), (2, f[5])):
                assert oracle.oracle_fq_op(op, a, b, out) == 0
                assert out.raw.hex() == want, line
            assert oracle.oracle_fq_op(3, a, None, out) == 0 and out.raw.hex() == f[6]
            rc = oracle.oracle_fq_op(4, a, None, out)
            assert (rc == 1) if f[7] == "none" else (rc == 0 and out.raw.hex() == f[7])
        elif f[0] == "fq_pow":
            assert oracle.oracle_fq_op(5, hexb(f[1]), hexb(f[2]), out) == 0
            assert out.raw.hex() == f[3]
        elif f[0] == "fq_bytes":
            v = int.from_bytes(hexb(f[1]), "little")
            assert (v < O.P_Q) == (f[2] == "ok")
        else:
            continue
        checked += 1
    assert checked > 400


def test_g1_kats(oracle):
    checked = 0
    for line in O.golden_lines("g1_kats.txt"):
        f = line.split()
        out = buf(64)
        if f[0] == "g1_generator":
            assert f[1] == O.G1_GEN.hex()
        elif f[0] == "g1_ops":
            p, q, k = hexb(f[1]), hexb(f[2]), hexb(f[3])
            assert oracle.oracle_g1_op(0, p, q, out) == 0 and out.raw.hex() == f[4]
            assert oracle.oracle_g1_op(1, p, None, out) == 0 and out.raw.hex() == f[5]
            assert oracle.oracle_g1_op(2, p, k, out) == 0 and out.raw.hex() == f[6]
            assert oracle.oracle_g1_op(3, p, None, out) == 0 and out.raw.hex() == f[7]
        elif f[0] == "g1_add_edge":
            assert oracle.oracle_g1_op(0, hexb(f[2]), hexb(f[3]), out) == 0
            assert out.raw.hex() == f[4], line
        elif f[0] == "g1_madd_edge":
            # acc = 2P at Z != 1; acc + 2P through the mixed add is 4P and
            # acc + (-2P) is infinity (crates/curve/tests/kats.rs:454-475).
            p = hexb(f[1])
            assert oracle.oracle_g1_op(1, p, None, out) == 0 and out.raw.hex() == f[2]
            assert oracle.oracle_g1_op(4, p, hexb(f[2]), out) == 0 and out.raw.hex() == f[3]
            assert oracle.oracle_g1_op(4, p, hexb(f[4]), out) == 0 and out.raw == bytes(64)
        elif f[0] == "g1_scalar_edge":
            assert oracle.oracle_g1_op(2, hexb(f[2]), hexb(f[3]), out) == 0
            assert out.raw.hex() == f[4], line
        elif f[0] == "g1_reject":
            assert oracle.oracle_g1_check(hexb(f[1])) != 0
        else:
            continue
        checked += 1
    assert checked > 100


def test_msm_kats(oracle):
    checked = 0
    for line in O.golden_lines("msm_kats.txt"):
        f = line.split()
        pattern, n, seed, want = f[1], int(f[2]), int(f[3]), f[4]
        bases, scalars = O.msm_case(pattern, n, seed)
        got = O.msm(bases, scalars, n, threads=8)
        assert got.hex() == want, f"{pattern} n={n}"
        checked += 1
    assert checked == 13


def test_msm_thread_count_independent(oracle):
    bases, scalars = O.msm_case("random", 300, 7)
    outs = {O.msm(bases, scalars, 300, threads=t) for t in (1, 3, 16)}
    assert len(outs) == 1


def test_poseidon2_perm(oracle):
    checked = 0
    for line in O.golden_lines("poseidon2_perm.txt"):
        f = line.split()
        out = buf(96)
        assert oracle.oracle_poseidon2(b"".join(hexb(x) for x in f[1:4]), out) == 0
        assert out.raw.hex() == "".join(f[4:7])
        checked += 1
    assert checked == 128


def test_transcript_cases(oracle):
    snap = None
    cases = 0
    for line in O.golden_lines("transcript_cases.txt"):
        f = line.split()
        if f[0] == "case":
            snap = O.new_snapshot()
        elif f[0] == "end":
            cases += 1
        elif f[0] == "observe":
            O.transcript_op(snap, 0, data=hexb(f[1]))
        elif f[0] == "sample":
            assert O.transcript_op(snap, 1).hex() == f[1]
        elif f[0] == "append_scalar":
            O.transcript_op(snap, 2, O.TAG_NAMES[f[1]], hexb(f[2]), 1)
        elif f[0] == "append_scalars":
            n = int(f[2])
            O.transcript_op(snap, 2, O.TAG_NAMES[f[1]], b"".join(hexb(x) for x in f[3:3 + n]), n)
        elif f[0] == "append_bytes":
            data = b"" if f[3] == "-" else hexb(f[3])
            assert len(data) == int(f[2])
            O.transcript_op(snap, 3, O.TAG_NAMES[f[1]], data, len(data))
        elif f[0] == "challenge":
            assert O.transcript_op(snap, 4, O.TAG_NAMES[f[1]]).hex() == f[2]
        else:
            raise AssertionError(line)
    assert cases > 5


def test_g1_absorb_kats(oracle):
    for line in O.golden_lines("g1_absorb_kats.txt"):
        f = line.split()
        if f[0] == "single":
            out = buf(128)
            oracle.oracle_g1_limbs(hexb(f[1]), out)
            assert out.raw.hex() == "".join(f[2:6])
        elif f[0] == "pair":
            for i, p in enumerate(f[1:3]):
                out = buf(128)
                oracle.oracle_g1_limbs(hexb(p), out)
                assert out.raw.hex() == "".join(f[3 + 4 * i:7 + 4 * i])


def test_poly_kats(oracle):
    lines = [l.split() for l in O.golden_lines("poly_kats.txt")]
    src = [l for l in lines if l[0] == "source"][0]
    assert src[1] == "u32"
    nv = int(src[2])
    values = [int(l[2], 16) for l in lines if l[0] == "value"]
    chals = [hexb(l[2]) for l in lines if l[0] == "challenge"]
    table = bytearray(b"".join(fe(v) for v in values))
    # bind k index value: the table after binding the first k challenges.
    binds = {}
    for l in lines:
        if l[0] == "bind":
            binds.setdefault(int(l[1]), {})[int(l[2])] = l[3]
    for k, entries in binds.items():
        t = (ctypes.c_uint8 * len(table)).from_buffer_copy(table)
        assert oracle.oracle_bind(t, nv, b"".join(chals[:k]), k) == 0
        raw = bytes(t)
        for idx, want in entries.items():
            assert raw[32 * idx:32 * idx + 32].hex() == want
    # eq k index value: eq_table(challenges[..k]).
    eqs = {}
    for l in lines:
        if l[0] == "eq":
            eqs.setdefault(int(l[1]), {})[int(l[2])] = l[3]
    for k, entries in eqs.items():
        out = buf(32 << k)
        assert oracle.oracle_eq_table(b"".join(chals[:k]), k, out) == 0
        for idx, want in entries.items():
            assert out.raw[32 * idx:32 * idx + 32].hex() == want
    # point case index value / result case value.
    points = {}
    for l in lines:
        if l[0] == "point":
            points.setdefault(int(l[1]), {})[int(l[2])] = hexb(l[3])
    results = {int(l[1]): l[2] for l in lines if l[0] == "result"}
    for case, want in results.items():
        pt = b"".join(points[case][i] for i in range(nv))
        out = buf(32)
        assert oracle.oracle_evaluate(bytes(table), nv, pt, out) == 0
        assert out.raw.hex() == want
    assert results and binds and eqs


def _parse_proof_kat(name):
    rec = {"value": {}, "point": {}}
    for line in O.golden_lines(name):
        f = line.split()
        if f[0] in ("value", "point"):
            rec[f[0]][int(f[1])] = hexb(f[2])
        else:
            rec[f[0]] = f[1]
    nv = int(rec["numvars"])
    evals = b"".join(rec["value"][i] for i in range(1 << nv))
    u = b"".join(rec["point"][i] for i in range(nv))
    return rec, nv, evals, u


TOY_TAU = 0xABCDEF


def test_mercury_proof_kat(oracle):
    rec, nv, evals, u = _parse_proof_kat("mercury_proof.txt")
    assert O.fe_int(hexb(rec["tau"])) == TOY_TAU
    srs = O.toy_srs(TOY_TAU, 1 << nv)
    cm = buf(64)
    assert oracle.oracle_commit(srs, ctypes.c_size_t(1 << nv), evals, nv, 4, cm) == 0
    assert cm.raw.hex() == rec["commitment"]
    snap = O.new_snapshot()
    s = (ctypes.c_uint8 * O.SNAP).from_buffer(snap)
    v, proof = buf(32), buf(704)
    rc = oracle.oracle_mercury_open(srs, ctypes.c_size_t(1 << nv), evals, nv, cm.raw, u, s, 4, v, proof)
    assert rc == 0
    assert v.raw.hex() == rec["claim"]
    assert proof.raw.hex() == rec["proof"]
    assert O.transcript_op(snap, 1).hex() == rec["probe"]


def test_mercury_batch_kat(oracle):
    rec, nv, evals, u = _parse_proof_kat("mercury_batch.txt")
    srs = O.toy_srs(TOY_TAU, 1 << nv)
    cm = buf(64)
    assert oracle.oracle_commit(srs, ctypes.c_size_t(1 << nv), evals, nv, 4, cm) == 0
    assert cm.raw.hex() == rec["commitment"]
    snap = O.new_snapshot()
    s = (ctypes.c_uint8 * O.SNAP).from_buffer(snap)
    vs, proof = buf(32), buf(704)
    rc = oracle.oracle_mercury_batch_open(srs, ctypes.c_size_t(1 << nv), evals, 1, nv, cm.raw, u, s, 4, vs, proof)
    assert rc == 0
    assert vs.raw.hex() == rec["claim"]
    assert proof.raw.hex() == rec["proof"]
    assert O.transcript_op(snap, 1).hex() == rec["probe"]


def test_accumulator_batch_proof(oracle):
    """The three-column batch opening recorded in accumulator.txt replays."""
    rec = {"batch_value": {}, "batch_point": {}, "batch_claim": {}, "batch_cm": {}}
    for line in O.golden_lines("accumulator.txt"):
        f = line.split()
        if f[0] == "batch_value":
            rec["batch_value"][(int(f[1]), int(f[2]))] = hexb(f[3])
        elif f[0] in ("batch_point", "batch_claim", "batch_cm"):
            rec[f[0]][int(f[1])] = hexb(f[2])
        elif f[0] in ("numvars", "batch_proof"):
            rec[f[0]] = f[1]
    nv = int(rec["numvars"])
    k = len(rec["batch_cm"])
    cols = b"".join(rec["batch_value"][(c, i)] for c in range(k) for i in range(1 << nv))
    u = b"".join(rec["batch_point"][i] for i in range(nv))
    srs = O.toy_srs(TOY_TAU, 1 << nv)
    for c in range(k):
        cm = buf(64)
        assert oracle.oracle_commit(srs, ctypes.c_size_t(1 << nv), cols[32 * c << nv:32 * (c + 1) << nv], nv, 4, cm) == 0
        assert cm.raw == rec["batch_cm"][c]
    snap = O.new_snapshot()
    s = (ctypes.c_uint8 * O.SNAP).from_buffer(snap)
    vs, proof = buf(32 * k), buf(704)
    cms = b"".join(rec["batch_cm"][c] for c in range(k))
    rc = oracle.oracle_mercury_batch_open(srs, ctypes.c_size_t(1 << nv), cols, k, nv, cms, u, s, 4, vs, proof)
    assert rc == 0
    assert vs.raw == b"".join(rec["batch_claim"][c] for c in range(k))
    assert proof.raw.hex() == rec["batch_proof"]


def test_known_tau_commitment(oracle):
    """cm == [f(tau)] G for a commitment over a seeded-tau SRS."""
    rng = O.Rng(99)
    nv = 6
    tau = rng.next_fr()
    srs = O.toy_srs(tau, 1 << nv)
    coeffs = [rng.next_fr() for _ in range(1 << nv)]
    cm = buf(64)
    assert oracle.oracle_commit(srs, ctypes.c_size_t(1 << nv), b"".join(fe(c) for c in coeffs), nv, 4, cm) == 0
    f_tau = sum(c * pow(tau, i, O.P_R) for i, c in enumerate(coeffs)) % O.P_R
    assert cm.raw == O.g1_mul(O.G1_GEN, f_tau)


def test_accumulator_words_and_digest(oracle):
    """The oracle rebuilds the concatenated accumulator's 146 words (two
    deferred checks of twelve entries) and their digest from the entries
    accumulator.txt records (crates/pcs/tests/vectors/accumulator.txt)."""
    tau, words, digest = O.golden_accumulator()
    sides, scalars, points, checks = O.entries_from_words(words)
    assert checks == [12, 12]
    assert O.accumulator_words(sides, scalars, points, checks) == words
    rc, _, _, _, dg = O.accumulator_msms(sides, scalars, points, checks)
    assert rc == 0 and dg == digest


def test_accumulator_discharge_relation(oracle):
    """With the toy SRS's known tau, e(A, [1]_2) = e(B, [x]_2) is A = tau * B:
    the recorded deferred verifications hold, merged and one by one, and a
    changed scalar breaks the relation."""
    tau, words, _ = O.golden_accumulator()
    sides, scalars, points, checks = O.entries_from_words(words)
    rc, a, b, _, _ = O.accumulator_msms(sides, scalars, points, checks)
    assert rc == 0 and O.g1_mul(b, tau) == a
    for j in range(2):
        s = slice(12 * j, 12 * j + 12)
        rc, a1, b1, _, _ = O.accumulator_msms(sides[s], scalars[s], points[s], [12], weights=[1])
        assert rc == 0 and O.g1_mul(b1, tau) == a1
    bad = list(scalars)
    bad[3] = (bad[3] + 1) % O.P_R
    rc, a2, b2, _, _ = O.accumulator_msms(sides, bad, points, checks)
    assert rc == 0 and O.g1_mul(b2, tau) != a2


def test_accumulator_refusal_order(oracle):
    """discharge validates points before the partition; check_pairings checks
    the partition first (crates/pcs/src/accumulator.rs:151, :177-185)."""
    _, words, _ = O.golden_accumulator()
    sides, scalars, points, checks = O.entries_from_words(words)
    off = bytearray(points[0])
    off[0] ^= 1
    pts = [bytes(off)] + points[1:]
    assert O.accumulator_msms(sides, scalars, points, [12, 11])[0] == 10
    assert O.accumulator_msms(sides, scalars, pts, checks)[0] == 9
    assert O.accumulator_msms(sides, scalars, pts, [12, 13])[0] == 9
    assert O.accumulator_msms(sides, scalars, pts, [12, 13], weights=[1, 1])[0] == 10


def _accumulator_batch():
    rec = {"batch_value": {}, "batch_point": {}, "batch_claim": {}, "batch_cm": {}}
    for line in O.golden_lines("accumulator.txt"):
        f = line.split()
        if f[0] == "batch_value":
            rec["batch_value"][(int(f[1]), int(f[2]))] = hexb(f[3])
        elif f[0] in ("batch_point", "batch_claim", "batch_cm"):
            rec[f[0]][int(f[1])] = hexb(f[2])
        elif f[0] in ("numvars", "batch_proof"):
            rec[f[0]] = f[1]
    return rec


def test_stacked_opening_at_empty_r_replays_the_golden_batch(oracle):
    """batch_open is batch_open_stacked at r = [] with one column a stack
    (crates/pcs/src/lib.rs:688-703): the stacked entry point replays the
    committed three-column batch proof byte for byte."""
    rec = _accumulator_batch()
    nv = int(rec["numvars"])
    k = len(rec["batch_cm"])
    stacks = [[[O.fe_int(rec["batch_value"][(c, i)]) for i in range(1 << nv)]] for c in range(k)]
    u = [O.fe_int(rec["batch_point"][i]) for i in range(nv)]
    srs = O.toy_srs(TOY_TAU, 1 << nv)
    snap = O.new_snapshot()
    rc, vs, proof = O.batch_open_stacked(srs, 1 << nv, stacks, [nv] * k, [rec["batch_cm"][c] for c in range(k)],
                                         u, [], snap)
    assert rc == 0
    assert [O.fe(v) for v in vs] == [rec["batch_claim"][c] for c in range(k)]
    assert proof.hex() == rec["batch_proof"]


def _stacked_case(seed, width, sigma, lens):
    rng = random.Random(seed)
    stacks = [[[rng.randrange(O.P_R) for _ in range(1 << width)] for _ in range(L)] for L in lens]
    tables = [[x for c in st for x in c] + [0] * (((1 << sigma) - len(st)) << width) for st in stacks]
    u = [rng.randrange(O.P_R) for _ in range(width)]
    r = [rng.randrange(O.P_R) for _ in range(sigma)]
    return stacks, tables, u, r


def test_stacked_values_are_the_stacks_at_u_r(oracle):
    """v_j = sum_s eq(r, s) col_{j,s}(u) is stack j's table at u || r
    (crates/pcs/tests/batch.rs:650-660), for a full, a short and a
    one-column stack; the commitments are the materialised stacks'."""
    width, sigma = 3, 3
    stacks, tables, u, r = _stacked_case(5, width, sigma, [8, 5, 1])
    nv = width + sigma
    srs = O.toy_srs(TOY_TAU, 1 << nv)
    cms = []
    for t in tables:
        cm = buf(64)
        assert oracle.oracle_commit(srs, ctypes.c_size_t(1 << nv), b"".join(fe(x) for x in t), nv, 4, cm) == 0
        cms.append(cm.raw)
    rc, vs, proof = O.batch_open_stacked(srs, 1 << nv, stacks, [width] * 14, cms, u, r, O.new_snapshot())
    assert rc == 0 and len(proof) == 704
    assert vs == [O.mle_eval(t, u + r) for t in tables]


def test_stacked_refusal_order(oracle):
    """The refusals of batch_open_stacked in order (crates/pcs/src/lib.rs:713-754):
    EmptyBatch, BatchLengthMismatch (commitments), MixedColumnSizes,
    UnsupportedNumVars, PointLengthMismatch, BatchLengthMismatch (slots),
    SrsTooSmall; the oracle returns 10 + its status."""
    stacks, _, u, r = _stacked_case(6, 2, 2, [4, 2])
    srs = O.toy_srs(TOY_TAU, 16)
    cms = [bytes(64)] * 2

    def run(st, nvs, c, uu, rr, srs_n=16):
        return O.batch_open_stacked(srs, srs_n, st, nvs, c, uu, rr, O.new_snapshot())[0]

    assert run([], [], [], u, r) == 15
    assert run([stacks[0], []], [2] * 4, cms, u, r) == 15
    assert run(stacks, [2] * 6, cms[:1], u, r) == 16
    mixed = [stacks[0], [stacks[1][0], stacks[1][1] + stacks[1][1]]]
    assert run(mixed, [2] * 5 + [3], cms, u, r) == 17
    assert run(stacks, [2] * 6, cms, u, r[:1]) == 11
    assert run(stacks, [2] * 6, cms, u[:1], r) == 12
    long = [stacks[0] + [stacks[1][0]], stacks[1]]
    assert run(long, [2] * 7, cms, u, r) == 16
    assert run(stacks, [2] * 6, cms, u, r, srs_n=8) == 13


def test_evaluate_diff(oracle):
    """crates/poly/tests/vectors/evaluate_diff.txt: 100 evaluate cases against
    ark-poly. Case i has i % 13 variables and backing BACKINGS[i % 5]; its
    table is drawn from splitmix64 seeded 20260908 + i (u1/u8/u16/u32 take
    the low bits of one draw, fr four draws read mod p) and pinned by a
    SHA-256 over the lifted entries before the oracle evaluates it."""
    import hashlib

    cases, points, results = {}, {}, {}
    for line in O.golden_lines("evaluate_diff.txt"):
        f = line.split()
        if f[0] == "case":
            cases[int(f[1])] = (f[2], int(f[3]), f[4])
        elif f[0] == "point":
            points.setdefault(int(f[1]), {})[int(f[2])] = O.fe_int(hexb(f[3]))
        elif f[0] == "result":
            results[int(f[1])] = f[2]
    assert len(cases) == 100
    masks = {"u1": 1, "u8": 0xFF, "u16": 0xFFFF, "u32": 0xFFFFFFFF}
    for i, (backing, nv, digest) in cases.items():
        rng = O.Rng(20260908 + i)
        if backing == "fr":
            table = [O.fe_int(rng.next_le32()) % O.P_R for _ in range(1 << nv)]
        else:
            table = [rng.next_u64() & masks[backing] for _ in range(1 << nv)]
        raw = b"".join(O.fe(x) for x in table)
        assert hashlib.sha256(raw).hexdigest() == digest, f"case {i}: table"
        pt = [points[i][j] for j in range(nv)] if nv else []
        out = buf(32)
        assert oracle.oracle_evaluate(raw, ctypes.c_size_t(nv), b"".join(O.fe(x) for x in pt), out) == 0
        assert out.raw.hex() == results[i], f"case {i}"


def test_io_digest(oracle):
    """crates/transcript/tests/vectors/io_digest.txt through the oracle's
    duplex: append_bytes of each stream under its tag, then one squeeze."""
    n = 0
    for line in O.golden_lines("io_digest.txt"):
        f = line.split()
        snap = O.new_snapshot()
        for tag, stream in ((O.TAG_NAMES["PUBLIC_INPUT_STREAM"], f[2]), (O.TAG_NAMES["PUBLIC_OUTPUT_STREAM"], f[3])):
            data = b"" if stream == "-" else hexb(stream)
            O.transcript_op(snap, 3, tag, data, len(data))
        assert O.transcript_op(snap, 1).hex() == f[4], f[1]
        n += 1
    assert n >= 10
