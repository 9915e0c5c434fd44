"""GPU parity of the MSM and commit paths against the oracle and the
reference's committed MSM corpus (crates/curve/tests/vectors/msm_kats.txt).

Every comparison is on the canonical affine bytes, which are
representation-independent, so the device's XYZZ buckets and windows need
not match the reference's Jacobian ones.
"""
import random

import pytest

import oracle_lib as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import apogee_gpu as A

    with A.Context(0) as c:
        yield c


def mont(scalars_bytes: bytes) -> bytes:
    import apogee_gpu as A

    xs = [int.from_bytes(scalars_bytes[i:i + 32], "little") for i in range(0, len(scalars_bytes), 32)]
    return A.to_mont_bytes(xs)


def test_msm_kats(ctx):
    checked = 0
    for line in O.golden_lines("msm_kats.txt"):
        f = line.split()
        pattern, n, seed, want = f[1], int(f[2]), int(f[3]), f[4]
        bases, scalars = O.msm_case(pattern, n, seed)
        assert ctx.msm(bases, mont(scalars)).hex() == want, f"{pattern} n={n}"
        checked += 1
    assert checked == 13


@pytest.mark.parametrize("n", [1, 2, 3, 31, 32, 33, 100, 257, 1025, 5000])
def test_msm_random_sizes_against_oracle(ctx, n):
    bases, scalars = O.msm_case("random", n, 1000 + n)
    assert ctx.msm(bases, mont(scalars)) == O.msm(bases, scalars, n, threads=8)


def test_msm_length_mismatch_and_empty(ctx):
    import apogee_gpu as A

    bases, scalars = O.msm_case("random", 4, 5)
    with pytest.raises(A.MsmError):
        ctx.msm(bases, mont(scalars)[:96])
    assert ctx.msm(b"", b"") == bytes(64)


def test_msm_edge_scalars(ctx):
    """0, 1, p-1 and top-window carries: scalars just below 2^254 and
    values whose every window reaches the signed-digit threshold."""
    n = 64
    bases, _ = O.msm_case("random", n, 77)
    edge = [0, 1, 2, O.P_R - 1, O.P_R - 2, (1 << 253), (1 << 253) + (1 << 252)]
    edge += [int("8" * 63, 16) % O.P_R, int("7fff" * 16, 16) % O.P_R, int("ffff" * 15 + "0fff", 16) % O.P_R]
    rng = random.Random(3)
    scalars = edge + [rng.randrange(O.P_R) for _ in range(n - len(edge))]
    sb = b"".join(O.fe(s) for s in scalars)
    assert ctx.msm(bases, mont(sb)) == O.msm(bases, sb, n)


def test_msm_rejects_noncanonical(ctx):
    import apogee_gpu as A

    bases, scalars = O.msm_case("random", 4, 6)
    bad = bytearray(bases)
    bad[64:96] = O.fe(O.P_Q)  # x = q is not a canonical coordinate
    with pytest.raises(A.ApogeeError):
        ctx.msm(bytes(bad), mont(scalars))
    off = bytearray(bases)
    off[0] ^= 1  # breaks the curve equation
    with pytest.raises(A.PcsError):
        ctx.msm(bytes(off), mont(scalars))
    # and the context stays usable afterwards
    assert ctx.msm(bases, mont(scalars)) == O.msm(bases, scalars, 4)


def test_msm_small_u32(ctx):
    n = 3000
    bases, _ = O.msm_case("random", n, 8)
    rng = random.Random(9)
    vals = [rng.choice([0, 1, rng.getrandbits(8), rng.getrandbits(16), rng.getrandbits(32)]) for _ in range(n)]
    vals[:4] = [0xFFFFFFFF, 0x80000000, 0x7FFFFFFF, 0]
    sb = b"".join(O.fe(v) for v in vals)
    assert ctx.msm_small_u32(bases, vals) == O.msm(bases, sb, n)


def test_srs_generate_matches_oracle(ctx):
    tau = 0xABCDEF
    n = 300
    ctx.srs_generate(tau, n)
    assert ctx.srs_download(n) == O.toy_srs(tau, n)


def test_commit_against_oracle_and_known_tau(ctx):
    import ctypes

    rng = O.Rng(2026)
    tau = rng.next_fr()
    nv = 10
    n = 1 << nv
    srs = O.toy_srs(tau, n)
    ctx.srs_upload(srs)
    coeffs = [rng.next_fr() for _ in range(n)]
    cb = b"".join(O.fe(c) for c in coeffs)
    cm = ctx.commit(mont(cb), nv)
    want = O.buf(64)
    assert O.lib().oracle_commit(srs, ctypes.c_size_t(n), cb, nv, 8, want) == 0
    assert cm == want.raw
    f_tau = sum(c * pow(tau, i, O.P_R) for i, c in enumerate(coeffs)) % O.P_R
    assert cm == O.g1_mul(O.G1_GEN, f_tau)


def test_commit_shape_errors(ctx):
    import apogee_gpu as A

    ctx.srs_generate(5, 64)
    with pytest.raises(A.PcsError) as e:
        ctx.commit(bytes(32 * 8), 3)
    assert e.value.variant == "UnsupportedNumVars"
    with pytest.raises(A.PcsError) as e:
        ctx.commit(bytes(32 * 256), 8)
    assert e.value.variant == "SrsTooSmall"


def test_commit_u32_and_batch(ctx):
    tau = 0x1234567
    nv = 8
    n = 1 << nv
    ctx.srs_generate(tau, n)
    rng = random.Random(11)
    vals = [rng.getrandbits(32) for _ in range(n)]
    f_tau = sum(v * pow(tau, i, O.P_R) for i, v in enumerate(vals)) % O.P_R
    assert ctx.commit_u32(vals, nv) == O.g1_mul(O.G1_GEN, f_tau)
    cols = [[rng.randrange(O.P_R) for _ in range(n)] for _ in range(3)]
    import apogee_gpu as A

    cms = ctx.commit_batch([A.to_mont_bytes(c) for c in cols], nv)
    for c, cm in zip(cols, cms):
        f_tau = sum(v * pow(tau, i, O.P_R) for i, v in enumerate(c)) % O.P_R
        assert cm == O.g1_mul(O.G1_GEN, f_tau)


@pytest.mark.parametrize("kind", ["ones", "bits", "mixed", "identical"])
def test_commit_skewed_digits(ctx, kind):
    """Skewed scalars pile most digits into a few buckets (a column of ones
    puts every entry in bucket 1): the edge-run folding must still write each
    bucket exactly once. Checked by the known-tau identity at 2^14."""
    import apogee_gpu as A
    import synth

    tau = 0xC0FFEE
    nv = 14
    n = 1 << nv
    ctx.srs_generate(tau, n)
    rng = random.Random(hash(kind) & 0xFFFF)
    if kind == "ones":
        coeffs = [1] * n
    elif kind == "bits":
        coeffs = [rng.getrandbits(1) for _ in range(n)]
    elif kind == "identical":
        coeffs = [rng.randrange(O.P_R)] * n
    else:
        coeffs = synth.to_ints(synth.mixed_column(n, 5))
    cm = ctx.commit(A.to_mont_bytes(coeffs), nv)
    acc = 0
    for c in reversed(coeffs):
        acc = (acc * tau + c) % O.P_R
    assert cm == O.g1_mul(O.G1_GEN, acc)


def test_msm_identical_large_against_oracle(ctx):
    bases, scalars = O.msm_case("identical", 4096, 31)
    assert ctx.msm(bases, mont(scalars)) == O.msm(bases, scalars, 4096, threads=8)


def test_commit_large_known_tau(ctx):
    """2^16 points through the wide-window table: the known-tau identity."""
    import apogee_gpu as A

    tau = 0x5EED
    nv = 16
    n = 1 << nv
    ctx.srs_generate(tau, n)
    rng = random.Random(12)
    coeffs = [rng.randrange(O.P_R) for _ in range(n)]
    cm = ctx.commit(A.to_mont_bytes(coeffs), nv)
    # f(tau) by Horner
    acc = 0
    for c in reversed(coeffs):
        acc = (acc * tau + c) % O.P_R
    assert cm == O.g1_mul(O.G1_GEN, acc)


def _f_tau(coeffs, tau):
    acc = 0
    for c in reversed(coeffs):
        acc = (acc * tau + c) % O.P_R
    return acc


def _column(kind, n, rng):
    import synth

    if kind == "zeros":
        return [0] * n
    if kind == "ones":
        return [1] * n
    if kind == "bits":
        return [rng.getrandbits(1) for _ in range(n)]
    if kind == "u32":
        return [rng.getrandbits(32) for _ in range(n)]
    if kind == "identical":
        return [rng.randrange(O.P_R)] * n
    if kind == "mixed":
        return synth.to_ints(synth.mixed_column(n, rng.getrandbits(32)))
    return [rng.randrange(O.P_R) for _ in range(n)]


@pytest.mark.parametrize("nv", [12, 16, 20])
def test_commit_batch_groups_known_tau(ctx, nv):
    """Columns of every digit shape committed together share one sort,
    accumulation and bucket reduction per group (nine columns: three groups
    over both lanes; at 2^20 the 20-bit window table); each commitment must
    equal [f(tau)]G, and single commits must agree with the batch."""
    import apogee_gpu as A

    tau = 0xBA7C4 + nv
    n = 1 << nv
    ctx.srs_generate(tau, n)
    rng = random.Random(nv)
    kinds = ["zeros", "ones", "bits", "u32", "identical", "mixed", "uniform", "mixed", "ones"]
    if nv >= 20:
        kinds = ["mixed", "uniform", "u32", "ones", "bits"]
    cols = [_column(k, n, rng) for k in kinds]
    blobs = [A.to_mont_bytes(c) for c in cols]
    cms = ctx.commit_batch(blobs, nv)
    for kind, c, cm in zip(kinds, cols, cms):
        assert cm == O.g1_mul(O.G1_GEN, _f_tau(c, tau)), kind
    assert [ctx.commit(b, nv) for b in blobs[:3]] == cms[:3]


def test_commit_batch_many_small_columns(ctx):
    """130 columns of 4 values: groups of 33 split at the 32-column limit."""
    import apogee_gpu as A

    tau = 0x77
    nv = 2
    ctx.srs_generate(tau, 1 << nv)
    rng = random.Random(130)
    cols = [_column(["uniform", "u32", "bits", "zeros"][j % 4], 4, rng) for j in range(130)]
    cms = ctx.commit_batch([A.to_mont_bytes(c) for c in cols], nv)
    for c, cm in zip(cols, cms):
        assert cm == O.g1_mul(O.G1_GEN, _f_tau(c, tau))


def test_autotune_choice_keeps_commitments(ctx):
    """The window-width autotuner only changes speed: after it records a
    width per size class, commits (alone and batched) still equal [f(tau)]G,
    and every chosen width is one of the candidates."""
    import numpy as np
    import torch

    import apogee_gpu as A
    import synth

    tau = 0xA070
    nv = 12
    n = 1 << nv
    ctx.srs_generate(tau, n)
    sample = torch.from_numpy(synth.mixed_column(n, 3).view(np.int32).reshape(-1)).to("cuda:0")
    ctx.fr_to_mont_device(sample.data_ptr(), n)
    chosen = ctx.msm_autotune(sample.data_ptr(), n, 8, 13, cands=(8, 12, 16))
    assert set(chosen) == set(range(8, 14))
    assert chosen[13] == 0  # beyond the sample and the SRS
    assert all(chosen[k] in (8, 12, 16) for k in range(8, 13))
    rng = random.Random(77)
    for k in (8, 10, 12):
        cols = [_column(kind, 1 << k, rng) for kind in ("mixed", "uniform", "u32")]
        cms = ctx.commit_batch([A.to_mont_bytes(c) for c in cols], k)
        for c, cm in zip(cols, cms):
            assert cm == O.g1_mul(O.G1_GEN, _f_tau(c, tau))
        assert ctx.commit(A.to_mont_bytes(cols[0]), k) == cms[0]


def test_commit_stack_known_tau(ctx):
    """pcs::commit_stack: the stack's commitment is [F(tau)]G for F the
    concatenation of the columns, read as coefficients; 40 columns of 4 take
    two groups whose partial sums are added; the reference's refusal order."""
    import apogee_gpu as A

    tau = 0x57AC
    ctx.srs_generate(tau, 1 << 10)
    rng = random.Random(5)
    for nv, k, kinds in ((8, 3, ("mixed", "uniform", "bits")), (2, 40, ("uniform", "u32", "zeros", "ones"))):
        cols = [_column(kinds[j % len(kinds)], 1 << nv, rng) for j in range(k)]
        concat = [v for c in cols for v in c]
        cm = ctx.commit_stack([A.to_mont_bytes(c) for c in cols], nv)
        assert cm == O.g1_mul(O.G1_GEN, _f_tau(concat, tau)), (nv, k)
    one = A.to_mont_bytes([1, 2, 3, 4])
    with pytest.raises(A.PcsError) as e:
        ctx.commit_stack([], 2)
    assert e.value.variant == "EmptyBatch"
    with pytest.raises(A.PcsError) as e:  # needs 3 * 2^9 > 2^10 powers: checked before the sizes
        ctx.commit_stack([one, one, one], [9, 2, 2])
    assert e.value.variant == "SrsTooSmall"
    with pytest.raises(A.PcsError) as e:
        ctx.commit_stack([one, A.to_mont_bytes([1] * 8)], [2, 3])
    assert e.value.variant == "MixedColumnSizes"


@pytest.mark.parametrize("bits", [1, 8, 16, 32])
def test_commit_narrow_backings(ctx, bits):
    """A narrow column commits through the small-scalar path, never lifted to
    Fr, and equals the commitment of the same values as Fr: [f(tau)]G."""
    import struct

    import apogee_gpu as A

    tau = 0xB175 + bits
    nv = 12
    n = 1 << nv
    ctx.srs_generate(tau, n)
    rng = random.Random(bits)
    vals = [rng.getrandbits(bits) for _ in range(n)]
    if bits == 1:
        limbs = [0] * (n // 64)
        for i, v in enumerate(vals):
            limbs[i // 64] |= v << (i % 64)
        data = struct.pack(f"<{len(limbs)}Q", *limbs)
    else:
        data = struct.pack({8: f"<{n}B", 16: f"<{n}H", 32: f"<{n}I"}[bits], *vals)
    cm = ctx.commit_narrow(data, bits, nv)
    assert cm == O.g1_mul(O.G1_GEN, _f_tau(vals, tau))
    assert cm == ctx.commit(A.to_mont_bytes(vals), nv)


@pytest.mark.parametrize("scalars_kind", ["uniform", "equal", "small"])
def test_msm_large_degenerate_bases(ctx, scalars_kind):
    """2^18 generic bases drawn from {infinity, G, -G, 2G, 3G, 7G}: inside a
    bucket, adjacent points collide (P + P, P + (-P), infinity) in every way
    the affine pair rounds classify. The value is (sum s_i k_i) * G."""
    import apogee_gpu as A

    rng = random.Random(77 + len(scalars_kind))
    n = 1 << 18
    ks = [0, 1, O.P_R - 1, 2, 3, 7]
    pts = {k: (bytes(64) if k == 0 else O.g1_mul(O.G1_GEN, k)) for k in ks}
    kk = [rng.choice(ks) for _ in range(n)]
    if scalars_kind == "uniform":
        ss = [rng.randrange(O.P_R) for _ in range(n)]
    elif scalars_kind == "equal":
        ss = [rng.randrange(O.P_R)] * n
    else:
        ss = [rng.randrange(1, 9) for _ in range(n)]
    want = O.g1_mul(O.G1_GEN, sum(s * k for s, k in zip(ss, kk)) % O.P_R)
    got = ctx.msm(b"".join(pts[k] for k in kk), A.to_mont_bytes(ss))
    assert got == want


def test_msm_large_one_point_all_doublings(ctx):
    """Every base G and one scalar: each window's digit puts all 2^18 points in
    one bucket, so every affine pair round is doublings only."""
    import apogee_gpu as A

    n = 1 << 18
    s = random.Random(5).randrange(O.P_R)
    got = ctx.msm(O.G1_GEN * n, A.to_mont_bytes([s] * n))
    assert got == O.g1_mul(O.G1_GEN, s * n % O.P_R)


def test_pair_round_fallback_agrees(ctx):
    """16 uniform 2^22 columns commit as four groups of four: about 4 x 15 x 2^22
    references, whose first affine pair round would exceed its scratch cap, so
    the groups take the XYZZ path from the references (the device flag). Each
    column committed alone runs the pair rounds. Both give the same points."""
    import torch

    nv = 22
    n = 1 << nv
    ctx.srs_generate(0x1234567, n)
    ctx.srs_prepare()
    g = torch.Generator(device="cuda").manual_seed(5)
    cols = []
    for _ in range(16):
        t = torch.randint(0, 1 << 31, (n, 8), dtype=torch.int64, device="cuda", generator=g)
        t[:, 7] &= 0x0FFFFFFF  # below 2^252 < r
        t = t.to(torch.int32).contiguous()
        ctx.fr_to_mont_device(t.data_ptr(), n)
        cols.append(t)
    ptrs = [t.data_ptr() for t in cols]
    batch = ctx.commit_batch_device(ptrs, nv)
    alone = [ctx.commit_device(p, nv) for p in ptrs]
    assert batch == alone
