"""The host pairing (host_pairing.hpp) and the full verifications built on
it, against what the reference holds:

* G2 arithmetic and decoding against g2_kats.txt (P + Q, 2P, kP, -P, the
  rejection classes including points outside the order-r subgroup) and the
  Fq12 tower and exact final exponent against fq12_kats.txt, compiled for the
  host here from the library's header;
* apg_pairing against every pairing_kats.txt case (the exact final exponent
  (q^12 - 1)/r of the optimal ate Miller loop), and bilinearity;
* apg_mercury_verify / apg_mercury_batch_verify on the golden proofs and the
  accumulator fixture's instances under the toy tau's verifier points
  ([1]_1, [1]_2, [tau]_2), refusing bumped values with VerificationFailed.

Host only."""
import os
import shutil
import subprocess

import pytest

import oracle_lib as O
from oracle_lib import hexb

pytestmark = pytest.mark.cpu_host
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
P = O.P_R
TOY_TAU = 0xABCDEF
G1_GEN = bytes([1] + [0] * 31 + [2] + [0] * 31)


def _A():
    import apogee_gpu as A

    try:
        A.lib()
    except ImportError as e:
        pytest.skip(str(e))
    return A


def _g2_generator():
    for line in O.golden_lines("g2_kats.txt"):
        f = line.split()
        if f[0] == "g2_generator":
            return hexb(f[1])
    raise AssertionError("no generator line")


def test_g2_arithmetic_and_decoding():
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not found")
    exe = os.path.join(os.environ.get("TMPDIR", "/tmp"), f"g2_check_{os.getpid()}")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "apogee-vm_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "g2_check.cpp"), "-o", exe], check=True,
                   capture_output=True)
    try:
        r = subprocess.run([exe, os.path.join(O.GOLDEN, "g2_kats.txt")], capture_output=True, text=True,
                           timeout=300)
    finally:
        os.unlink(exe)
    assert r.returncode == 0, r.stdout + r.stderr
    ops, rejects, gens = map(int, r.stdout.split())
    assert ops == 200 and rejects == 14 and gens == 1


def test_fq12_tower_and_final_exponent():
    """The tower's Fq12 arithmetic and the exact final exponent against
    fq12_kats.txt: 64 edge-grid and 4 random lines of a + b, a - b, ab, a^2,
    1/a, conj a, a^q, a^(q^2), a^(q^3), and 20 final exponentiations."""
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not found")
    exe = os.path.join(os.environ.get("TMPDIR", "/tmp"), f"fq12_check_{os.getpid()}")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "apogee-vm_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "fq12_check.cpp"), "-o", exe], check=True,
                   capture_output=True)
    try:
        r = subprocess.run([exe, os.path.join(O.GOLDEN, "fq12_kats.txt")], capture_output=True, text=True,
                           timeout=300)
    finally:
        os.unlink(exe)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.split() == ["68", "20"]


def test_pairing_known_answers():
    A = _A()
    n = 0
    for line in O.golden_lines("pairing_kats.txt"):
        f = line.split()
        p, q, e = (f[2], f[3], f[4]) if f[0] == "pairing_named" else (f[1], f[2], f[3])
        assert A.pairing(hexb(p), hexb(q)) == hexb(e), line[:40]
        n += 1
    assert n == 126


def test_pairing_bilinear_and_refusals():
    A = _A()
    g2 = _g2_generator()
    a, b = 0x1234567, 0x89ABCDE
    lhs_p = O.g1_mul(G1_GEN, a * b % P)
    neg = O.g1_mul(G1_GEN, P - a)
    qb = A.g2_mul(g2, b)
    # e(ab G1, G2) e(-a G1, b G2) = 1, and not with b + 1.
    assert A.pairing_check([lhs_p, neg], [g2, qb])
    assert not A.pairing_check([lhs_p, neg], [g2, A.g2_mul(g2, b + 1)])
    off = bytearray(g2)
    off[0] ^= 1
    with pytest.raises(A.ApogeeError) as e:
        A.pairing(G1_GEN, bytes(off))
    assert e.value.variant == "InvalidPoint"


def _toy_vsrs(A):
    g2 = _g2_generator()
    return G1_GEN + g2 + A.g2_mul(g2, TOY_TAU)


def test_full_verifications_under_the_toy_tau():
    import test_mercury_verify as M

    A = _A()
    vsrs = _toy_vsrs(A)
    u, v, cm, proof, probe = M._proof_kat("mercury_proof.txt")
    snap = A.mercury_verify(vsrs, cm, u, v, proof, A.transcript_init())
    s = bytearray(snap)
    assert O.transcript_op(s, 1).hex() == probe
    with pytest.raises(A.VerifyPcsError) as e:
        A.mercury_verify(vsrs, cm, u, (v + 1) % P, proof, A.transcript_init())
    assert e.value.variant == "VerificationFailed"
    u, v, cm, proof, _ = M._proof_kat("mercury_batch.txt")
    A.mercury_batch_verify(vsrs, [cm], u, [v], proof, A.transcript_init())
    single, batch = M._accumulator_kat()
    A.mercury_verify(vsrs, single["cm"], single["u"], single["v"], single["proof"], A.transcript_init())
    A.mercury_batch_verify(vsrs, batch["cms"], batch["u"], batch["vs"], batch["proof"], A.transcript_init())
    with pytest.raises(A.VerifyPcsError) as e:
        A.mercury_batch_verify(vsrs, batch["cms"][::-1], batch["u"], batch["vs"][::-1], batch["proof"],
                               A.transcript_init())
    assert e.value.variant == "VerificationFailed"
    # A verifier key with a point outside G2's subgroup is refused.
    bad = bytearray(vsrs)
    bad[64] ^= 1
    with pytest.raises(A.VerifyPcsError) as e:
        A.mercury_verify(bytes(bad), single["cm"], single["u"], single["v"], single["proof"], A.transcript_init())
    assert e.value.variant == "InvalidPoint"
