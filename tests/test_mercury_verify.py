"""The library's deferred Mercury verifier (apg_mercury_verify_deferred and
apg_mercury_batch_verify_deferred: pcs::verify_deferred and
batch_verify_deferred on the host) against what the reference holds:

* accumulator.txt (crates/pcs/tests/vectors): the single and the three-column
  batch instance, each verified from a fresh transcript, give the twelve
  entries whose concatenation is the committed word array, word for word,
  and its digest;
* mercury_proof.txt and mercury_batch.txt: the golden proofs verify to
  entries whose pairing relation A = tau B holds under the toy tau (the
  group side through the oracle's MSMs), and the transcript after the
  verification draws the committed probe;
* a bumped proof value or claim breaks the relation; off-curve points and
  shapes are refused in the reference's order.

Host only: the verifier runs no device code."""
import random

import pytest

import oracle_lib as O
from oracle_lib import hexb

pytestmark = pytest.mark.cpu_host
P = O.P_R
TOY_TAU = 0xABCDEF


def _A():
    import apogee_gpu as A

    try:
        A.lib()
    except ImportError as e:
        pytest.skip(str(e))
    return A


def _accumulator_kat():
    rec = {"single_point": {}, "batch_point": {}, "batch_claim": {}, "batch_cm": {}}
    for line in O.golden_lines("accumulator.txt"):
        f = line.split()
        if f[0] in rec:
            rec[f[0]][int(f[1])] = hexb(f[2])
        elif f[0] in ("single_claim", "single_cm", "single_proof", "batch_proof"):
            rec[f[0]] = hexb(f[1])
    s = {"u": [O.fe_int(rec["single_point"][i]) for i in range(len(rec["single_point"]))],
         "v": O.fe_int(rec["single_claim"]), "cm": rec["single_cm"], "proof": rec["single_proof"]}
    k = len(rec["batch_cm"])
    b = {"u": [O.fe_int(rec["batch_point"][i]) for i in range(len(rec["batch_point"]))],
         "vs": [O.fe_int(rec["batch_claim"][i]) for i in range(k)],
         "cms": [rec["batch_cm"][i] for i in range(k)], "proof": rec["batch_proof"]}
    return s, b


def _proof_kat(name):
    rec = {"point": {}}
    for line in O.golden_lines(name):
        f = line.split()
        if f[0] == "point":
            rec["point"][int(f[1])] = O.fe_int(hexb(f[2]))
        elif f[0] != "value":
            rec[f[0]] = f[1]
    u = [rec["point"][i] for i in range(int(rec["numvars"]))]
    return u, O.fe_int(hexb(rec["claim"])), hexb(rec["commitment"]), hexb(rec["proof"]), rec["probe"]


def _limbs(point):
    out = O.buf(128)
    assert O.lib().oracle_g1_limbs(point, out) == 0
    return out.raw


def _holds(entries):
    """A = tau B for one deferred check (check_pairings with weight one)."""
    sides, scalars, points, _ = entries
    rc, a, b, _, _ = O.accumulator_msms(sides, scalars, points, [12], weights=[1])
    assert rc == 0, rc
    return a == O.g1_mul(b, TOY_TAU)


def test_accumulator_words_replay():
    A = _A()
    s, b = _accumulator_kat()
    first = A.mercury_verify_deferred(s["cm"], s["u"], s["v"], s["proof"], A.transcript_init())
    second = A.mercury_batch_verify_deferred(b["cms"], b["u"], b["vs"], b["proof"], A.transcript_init())
    sides = first[0] + second[0]
    scalars = first[1] + second[1]
    points = first[2] + second[2]
    assert sides == bytes([0] * 10 + [1, 1]) * 2
    tau, words, digest = O.golden_accumulator()
    assert tau == TOY_TAU
    assert O.accumulator_words(sides, scalars, points, [12, 12]) == words
    rc, _, _, _, dg = O.accumulator_msms(sides, scalars, points, [12, 12])
    assert rc == 0 and dg == digest
    assert _holds(first) and _holds(second)


@pytest.mark.parametrize("name", ["mercury_proof.txt", "mercury_batch.txt"])
def test_golden_proofs_verify(name):
    A = _A()
    u, v, cm, proof, probe = _proof_kat(name)
    if name == "mercury_proof.txt":
        got = A.mercury_verify_deferred(cm, u, v, proof, A.transcript_init())
    else:
        got = A.mercury_batch_verify_deferred([cm], u, [v], proof, A.transcript_init())
    assert _holds(got)
    snap = bytearray(got[3])
    assert O.transcript_op(snap, 1).hex() == probe


def test_bumped_values_break_the_relation():
    A = _A()
    u, v, cm, proof, _ = _proof_kat("mercury_proof.txt")
    assert not _holds(A.mercury_verify_deferred(cm, u, (v + 1) % P, proof, A.transcript_init()))
    for i in range(6):
        bad = bytearray(proof)
        x = (O.fe_int(bytes(bad[512 + 32 * i:544 + 32 * i])) + 1) % P
        bad[512 + 32 * i:544 + 32 * i] = O.fe(x)
        assert not _holds(A.mercury_verify_deferred(cm, u, v, bytes(bad), A.transcript_init())), i
    # Another valid point in place of one of the proof's: on the curve, so
    # accepted by the deferred checks, but the relation fails.
    g = bytes(O.g1_mul(bytes([1] + [0] * 31 + [2] + [0] * 31), 7))
    for i in range(8):
        bad = bytearray(proof)
        bad[64 * i:64 * i + 64] = g
        assert not _holds(A.mercury_verify_deferred(cm, u, v, bytes(bad), A.transcript_init())), i


def test_refusals_in_the_reference_order():
    A = _A()
    u, v, cm, proof, _ = _proof_kat("mercury_proof.txt")
    snap = A.transcript_init()
    off = bytearray(cm)
    off[0] ^= 1  # leaves the curve
    with pytest.raises(A.VerifyPcsError) as e:
        A.mercury_verify_deferred(cm, u[:-1], v, proof, snap)
    assert e.value.variant == "UnsupportedNumVars"
    for i in range(8):
        bad = bytearray(proof)
        bad[64 * i] ^= 1
        with pytest.raises(A.VerifyPcsError) as e:
            A.mercury_verify_deferred(bytes(off), u, v, bytes(bad), snap)
        assert e.value.variant == "InvalidPoint" and e.value.info == i  # proof points before cm
    with pytest.raises(A.VerifyPcsError) as e:
        A.mercury_verify_deferred(bytes(off), u, v, proof, snap)
    assert e.value.variant == "InvalidPoint" and e.value.info == 8
    bad = bytearray(proof)
    bad[512:544] = P.to_bytes(32, "little")
    with pytest.raises(A.ApogeeError) as e:
        A.mercury_verify_deferred(cm, u, v, bytes(bad), snap)
    assert e.value.variant == "NonCanonical"
    # Batches: EmptyBatch, then BatchLengthMismatch, then the instance rule,
    # then the commitments.
    with pytest.raises(A.VerifyPcsError) as e:
        A.mercury_batch_verify_deferred([], u[:-1], [], proof, snap)
    assert e.value.variant == "EmptyBatch"
    with pytest.raises(A.VerifyPcsError) as e:
        A.mercury_batch_verify_deferred([cm, cm], u[:-1], [v], proof, snap)
    assert e.value.variant == "BatchLengthMismatch"
    with pytest.raises(A.VerifyPcsError) as e:
        A.mercury_batch_verify_deferred([bytes(off)], u[:-1], [v], proof, snap)
    assert e.value.variant == "UnsupportedNumVars"
    with pytest.raises(A.VerifyPcsError) as e:
        A.mercury_batch_verify_deferred([cm, bytes(off)], u, [v, v], proof, snap)
    assert e.value.variant == "InvalidPoint" and e.value.info == 8


def test_batches_of_many_commitments_sum_on_the_host():
    """A batch's cm* over 40 commitments: the verifier's host sum against the
    oracle's MSM, seen through the first entry's point."""
    A = _A()
    u, v, cm, proof, _ = _proof_kat("mercury_proof.txt")
    rng = random.Random(5)
    gen = bytes([1] + [0] * 31 + [2] + [0] * 31)
    cms = [O.g1_mul(gen, rng.randrange(1, P)) for _ in range(40)]
    vs = [rng.randrange(P) for _ in range(40)]
    got = A.mercury_batch_verify_deferred(cms, u, vs, proof, A.transcript_init())
    # rho from the preamble, replayed on the oracle's transcript.
    snap = O.new_snapshot()
    limbs = b"".join(_limbs(c) for c in cms)
    O.transcript_op(snap, 2, 3, limbs, 4 * len(cms))
    O.transcript_op(snap, 2, 6, b"".join(O.fe(x) for x in u + vs), len(u) + len(vs))
    rho = O.fe_int(O.transcript_op(snap, 4, 17))
    w = [pow(rho, i, P) for i in range(40)]
    want = O.msm(b"".join(cms), b"".join(O.fe(x) for x in w), 40)
    assert got[2][0] == want


@pytest.mark.parametrize("nv,k", [(2, 0), (6, 0), (8, 0), (4, 3), (6, 9)])
def test_oracle_openings_verify(nv, k):
    """Openings the oracle makes on the CPU at other sizes (k = 0: one
    column, else a batch of k) through the deferred verifier: the entries
    satisfy A = tau B under the SRS's tau, the transcript ends where the
    prover's did; a bumped claim breaks the relation."""
    import ctypes

    A = _A()
    rng = random.Random(700 + 10 * nv + k)
    tau = rng.randrange(1, P)
    n = 1 << nv
    srs = O.toy_srs(tau, n)
    cols = [[rng.choice([0, 1, rng.getrandbits(32), rng.randrange(P)]) for _ in range(n)] for _ in range(max(k, 1))]
    u = [rng.randrange(P) for _ in range(nv)]
    cms = []
    for c in cols:
        out = O.buf(64)
        assert O.lib().oracle_commit(srs, ctypes.c_size_t(n), b"".join(O.fe(x) for x in c), nv, 4, out) == 0
        cms.append(out.raw)
    snap = O.new_snapshot()
    after = bytearray(snap)
    s = (ctypes.c_uint8 * O.SNAP).from_buffer(after)
    proof = O.buf(704)
    if k == 0:
        v = O.buf(32)
        assert O.lib().oracle_mercury_open(srs, ctypes.c_size_t(n), b"".join(O.fe(x) for x in cols[0]), nv, cms[0],
                                           b"".join(O.fe(x) for x in u), s, 4, v, proof) == 0
        del s
        got = A.mercury_verify_deferred(cms[0], u, O.fe_int(v.raw), proof.raw, bytes(snap))
        bad = A.mercury_verify_deferred(cms[0], u, (O.fe_int(v.raw) + 1) % P, proof.raw, bytes(snap))
    else:
        vs = O.buf(32 * k)
        assert O.lib().oracle_mercury_batch_open(srs, ctypes.c_size_t(n), b"".join(O.fe(x) for c in cols for x in c),
                                                 ctypes.c_size_t(k), nv, b"".join(cms), b"".join(O.fe(x) for x in u),
                                                 s, 4, vs, proof) == 0
        del s
        vals = [O.fe_int(vs.raw[32 * i:32 * i + 32]) for i in range(k)]
        got = A.mercury_batch_verify_deferred(cms, u, vals, proof.raw, bytes(snap))
        vals[-1] = (vals[-1] + 1) % P
        bad = A.mercury_batch_verify_deferred(cms, u, vals, proof.raw, bytes(snap))
    assert got[3] == bytes(after)

    def holds(entries, t):
        rc, a, b, _, _ = O.accumulator_msms(entries[0], entries[1], entries[2], [12], weights=[1])
        return rc == 0 and a == O.g1_mul(b, t)

    assert holds(got, tau) and not holds(bad, tau)
