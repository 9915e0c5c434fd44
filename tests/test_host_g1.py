"""The host G1 sum the stacked opening uses for its cm* (msm_small in
host_g1.hpp: Fq Montgomery arithmetic, Jacobian formulas, 4-bit Straus),
compiled for the host here from the library's own header and checked against
the oracle's MSM on the reference corpus's input patterns (random, zero
scalars, identical scalars, every third base at infinity) and on sums that
cancel to infinity."""
import os
import shutil
import subprocess

import pytest

import oracle_lib as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not found")
    exe = tmp_path_factory.mktemp("g1") / "g1_msm_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "apogee-vm_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "g1_msm_check.cpp"), "-o", str(exe)], check=True,
                   capture_output=True)
    return str(exe)


def _run(exe, cases):
    lines = []
    for bases, scalars, n in cases:
        lines.append(str(n))
        for j in range(n):
            lines.append(bases[64 * j:64 * j + 64].hex() + " " + scalars[32 * j:32 * j + 32].hex())
    r = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    return [bytes.fromhex(h) for h in r.stdout.split()]


def test_host_msm_matches_oracle(checker):
    cases = []
    for pattern in ("random", "zeros", "identical", "infinity"):
        for n, seed in ((1, 3), (2, 5), (8, 7), (16, 11), (33, 13), (64, 17)):
            bases, scalars = O.msm_case(pattern, n, seed)
            cases.append((bases, scalars, n))
    # P and -P with equal scalars: the sum is the point at infinity.
    bases, scalars = O.msm_case("random", 1, 19)
    x, y = bases[:32], int.from_bytes(bases[32:], "little")
    neg = x + ((O.P_Q - y) % O.P_Q).to_bytes(32, "little")
    cases.append((bases + neg, scalars + scalars, 2))
    got = _run(checker, cases)
    for (bases, scalars, n), g in zip(cases, got):
        assert g == O.msm(bases, scalars, n), n
    assert got[-1] == bytes(64)
