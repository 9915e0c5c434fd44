"""The library's own transcript (the host duplex the C ABI exposes, not the
oracle's) replayed against the reference's committed vectors, through
apg_poseidon2_permute and apg_transcript_*: the 128 permutation vectors
(crates/transcript/tests/vectors/poseidon2_perm.txt), the raw and typed
transcript scripts (transcript_cases.txt) and the public I/O digests
(io_digest.txt). Marked gpu with the other calls into the library."""
import ctypes

import pytest

import oracle_lib as O
from oracle_lib import hexb

pytestmark = pytest.mark.gpu


def _lib():
    import apogee_gpu as A

    return A.lib()


def test_poseidon2_permutation_vectors():
    L = _lib()
    n = 0
    for line in O.golden_lines("poseidon2_perm.txt"):
        f = line.split()
        st = ctypes.create_string_buffer(b"".join(hexb(x) for x in f[1:4]), 96)
        assert L.apg_poseidon2_permute(st) == 0
        assert st.raw[:96].hex() == "".join(f[4:7])
        n += 1
    assert n == 128


def test_transcript_scripts():
    import apogee_gpu as A

    L = _lib()
    snap = None
    cases = 0

    def mont(hexval):
        return A.to_mont_bytes([O.fe_int(hexb(hexval))])

    def canon(b):
        return O.fe(A.from_mont_bytes(b)[0]).hex()

    for line in O.golden_lines("transcript_cases.txt"):
        f = line.split()
        if f[0] == "case":
            snap = ctypes.create_string_buffer(A.transcript_init(), 226)
        elif f[0] == "end":
            cases += 1
        elif f[0] == "observe":
            assert L.apg_transcript_observe(snap, mont(f[1])) == 0
        elif f[0] == "sample":
            out = ctypes.create_string_buffer(32)
            assert L.apg_transcript_sample(snap, out) == 0
            assert canon(out.raw) == f[1]
        elif f[0] in ("append_scalar", "append_scalars"):
            xs = [f[2]] if f[0] == "append_scalar" else f[3:3 + int(f[2])]
            data = b"".join(mont(x) for x in xs)
            assert L.apg_transcript_append_scalars(snap, ctypes.c_uint64(O.TAG_NAMES[f[1]]), data,
                                                   ctypes.c_size_t(len(xs))) == 0
        elif f[0] == "append_bytes":
            data = b"" if f[3] == "-" else hexb(f[3])
            assert len(data) == int(f[2])
            assert L.apg_transcript_append_bytes(snap, ctypes.c_uint64(O.TAG_NAMES[f[1]]), data,
                                                 ctypes.c_size_t(len(data))) == 0
        elif f[0] == "challenge":
            out = ctypes.create_string_buffer(32)
            assert L.apg_transcript_challenge(snap, ctypes.c_uint64(O.TAG_NAMES[f[1]]), out) == 0
            assert canon(out.raw) == f[2]
        else:
            raise AssertionError(line)
    assert cases > 5


def test_io_digest_vectors():
    import apogee_gpu as A

    L = _lib()
    n = 0
    for line in O.golden_lines("io_digest.txt"):
        f = line.split()
        assert f[0] == "io"
        inp = b"" if f[2] == "-" else hexb(f[2])
        outp = b"" if f[3] == "-" else hexb(f[3])
        d = ctypes.create_string_buffer(32)
        assert L.apg_io_digest(inp, ctypes.c_size_t(len(inp)), outp, ctypes.c_size_t(len(outp)), d) == 0
        assert O.fe(A.from_mont_bytes(d.raw)[0]).hex() == f[4], f[1]
        n += 1
    assert n >= 10


def test_transcript_refuses_bad_snapshots_and_values():
    import apogee_gpu as A

    L = _lib()
    snap = ctypes.create_string_buffer(A.transcript_init(), 226)
    bad = ctypes.create_string_buffer(b"\xff" * 32, 32)
    assert L.apg_transcript_observe(snap, bad) == 20  # APG_ERR_NONCANONICAL
    st = ctypes.create_string_buffer(O.fe(O.P_R) + bytes(64), 96)
    assert L.apg_poseidon2_permute(st) == 20
    broken = bytearray(A.transcript_init())
    broken[5 * 32] = 2  # input_len = 2 is never a snapshot's
    assert L.apg_transcript_sample(ctypes.create_string_buffer(bytes(broken), 226), ctypes.create_string_buffer(32)) == 21
