"""GPU parity of the deferred-pairing accumulator's group side
(crates/pcs/src/accumulator.rs:146-218, everything before the pairing)
against the oracle and the reference's committed accumulator: A, B and the
merge challenge byte for byte, the pairing relation through the known toy
tau (e(A, [1]_2) = e(B, [x]_2) is A = tau * B), and the refusals in the
reference's order."""
import random

import pytest

import oracle_lib as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import apogee_gpu as A

    with A.Context(0) as c:
        yield c


def _mont(xs):
    import apogee_gpu as A

    return A.to_mont_bytes(xs)


def _nu(b: bytes) -> int:
    import apogee_gpu as A

    return A.from_mont_bytes(b)[0]


def _golden():
    tau, words, _ = O.golden_accumulator()
    sides, scalars, points, checks = O.entries_from_words(words)
    return tau, sides, scalars, points, checks


def test_golden_accumulator_discharges(ctx):
    tau, sides, scalars, points, checks = _golden()
    a, b, nu = ctx.discharge_msms(sides, _mont(scalars), b"".join(points), checks)
    rc, oa, ob, onu, _ = O.accumulator_msms(sides, scalars, points, checks)
    assert rc == 0
    assert (a, b, _nu(nu)) == (oa, ob, onu)
    assert O.g1_mul(b, tau) == a


def test_golden_checks_one_by_one(ctx):
    tau, sides, scalars, points, checks = _golden()
    for j in range(2):
        s = slice(12 * j, 12 * j + 12)
        a, b = ctx.pairing_msms(sides[s], _mont(scalars[s]), b"".join(points[s]), [12], _mont([1]))
        assert O.g1_mul(b, tau) == a


def _synthetic(n_checks: int, seed: int, tau: int):
    """Deferred checks that hold under tau, shaped like Mercury's (ten A terms,
    two B terms), over SRS-like points k_i * G with known k_i: the B terms'
    points reappear on the A side times tau, eight more A terms sum to zero.
    Some checks are empty, some points are infinity or the generator."""
    rng = random.Random(seed)
    s_base = rng.randrange(2, O.P_R)
    pool = 512
    pts = O.toy_srs(s_base, pool)
    ks = [pow(s_base, i, O.P_R) for i in range(pool)]
    sides, scalars, points, checks = bytearray(), [], [], []
    for j in range(n_checks):
        if j % 97 == 5:
            checks.append(0)
            continue
        idx = [rng.randrange(pool) for _ in range(10)]
        a = [rng.randrange(O.P_R) for _ in range(8)]
        # sum_{i<8} a_i k_i = 0: solve for the last one (k != 0 for SRS points)
        acc = sum(a[i] * ks[idx[i]] for i in range(7)) % O.P_R
        a[7] = (-acc * pow(ks[idx[7]], -1, O.P_R)) % O.P_R
        b = [rng.randrange(O.P_R) for _ in range(2)]
        ents = [(0, a[i], pts[64 * idx[i]:64 * idx[i] + 64]) for i in range(8)]
        ents += [(0, tau * b[t] % O.P_R, pts[64 * idx[8 + t]:64 * idx[8 + t] + 64]) for t in range(2)]
        ents += [(1, b[t], pts[64 * idx[8 + t]:64 * idx[8 + t] + 64]) for t in range(2)]
        if j % 13 == 3:
            ents.append((0, rng.randrange(O.P_R), bytes(64)))
            ents.append((1, 0, O.G1_GEN))
        rng.shuffle(ents)
        for sd, sc, pt in ents:
            sides.append(sd)
            scalars.append(sc)
            points.append(pt)
        checks.append(len(ents))
    return bytes(sides), scalars, points, checks


@pytest.mark.parametrize("n_checks", [1, 7, 300, 2000])
def test_synthetic_accumulators(ctx, n_checks):
    tau = 0xABCDEF
    sides, scalars, points, checks = _synthetic(n_checks, 11 + n_checks, tau)
    a, b, nu = ctx.discharge_msms(sides, _mont(scalars), b"".join(points), checks)
    rc, oa, ob, onu, _ = O.accumulator_msms(sides, scalars, points, checks)
    assert rc == 0
    assert (a, b, _nu(nu)) == (oa, ob, onu)
    assert O.g1_mul(b, tau) == a
    # one changed scalar breaks the relation
    bad = list(scalars)
    bad[len(bad) // 2] = (bad[len(bad) // 2] + 1) % O.P_R
    a2, b2, _ = ctx.discharge_msms(sides, _mont(bad), b"".join(points), checks)
    assert O.g1_mul(b2, tau) != a2


def test_explicit_weights_match_the_oracle(ctx):
    sides, scalars, points, checks = _synthetic(40, 3, 0xABCDEF)
    rng = random.Random(9)
    w = [rng.randrange(O.P_R) for _ in checks]
    a, b = ctx.pairing_msms(sides, _mont(scalars), b"".join(points), checks, _mont(w))
    rc, oa, ob, _, _ = O.accumulator_msms(sides, scalars, points, checks, weights=w)
    assert rc == 0 and (a, b) == (oa, ob)


def test_empty_accumulators(ctx):
    for checks in ([], [0], [0, 0, 0]):
        a, b, nu = ctx.discharge_msms(b"", b"", b"", checks)
        rc, oa, ob, onu, _ = O.accumulator_msms(b"", [], [], checks)
        assert rc == 0 and a == b == bytes(64) == oa == ob
        assert _nu(nu) == onu


def test_refusals_in_the_reference_order(ctx):
    import apogee_gpu as A

    tau, sides, scalars, points, checks = _golden()
    off = bytearray(points[1])
    off[0] ^= 1
    bad_pts = b"".join([points[0], bytes(off)] + points[2:])
    good_pts = b"".join(points)
    sc = _mont(scalars)
    with pytest.raises(A.PcsError) as e:
        ctx.discharge_msms(sides, sc, good_pts, [12, 11])
    assert e.value.variant == "MalformedAccumulator"
    with pytest.raises(A.PcsError) as e:
        ctx.discharge_msms(sides, sc, bad_pts, [12, 13])
    assert e.value.variant == "InvalidPoint"
    with pytest.raises(A.PcsError) as e:
        ctx.pairing_msms(sides, sc, bad_pts, [12, 13], _mont([1, 1]))
    assert e.value.variant == "MalformedAccumulator"
    with pytest.raises(A.ApogeeError) as e:
        ctx.discharge_msms(bytes([2]) + sides[1:], sc, good_pts, checks)
    assert e.value.variant == "InvalidArgument"
    # the context is clean afterwards
    a, b, _ = ctx.discharge_msms(sides, sc, good_pts, checks)
    assert O.g1_mul(b, tau) == a


def test_discharge_with_its_pairing(ctx):
    """pcs::discharge end to end: the golden accumulator's MSMs on the device
    and the pairing e(A, [1]_2) e(-B, [tau]_2) on the host under the toy
    tau's verifier points; a bumped scalar fails with VerificationFailed."""
    import apogee_gpu as A
    from test_host_pairing import _toy_vsrs

    tau, sides, scalars, points, checks = _golden()
    vsrs = _toy_vsrs(A)
    ctx.discharge(vsrs, sides, _mont(scalars), b"".join(points), checks)
    bad = list(scalars)
    bad[3] = (bad[3] + 1) % O.P_R
    with pytest.raises(A.PcsError) as e:
        ctx.discharge(vsrs, sides, _mont(bad), b"".join(points), checks)
    assert e.value.variant == "VerificationFailed"
