"""apg_msm_noalloc: the MSM entry point for callers that cannot let the
library allocate device memory (a serving loop whose HBM is already promised
to admitted requests, or a pipeline that cannot take cudaMalloc's device-wide
synchronisation). It must give exactly what apg_msm gives, call after call,
although every call reuses the same fixed scratch array; its results are also
held to the oracle and to the known-tau identity, and a call must leave the
device's free memory where it was.

Kept in a file of its own that pytest collects last, so a run that stops at
the first failure has already run every other test."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

NONCANONICAL = 20
INVALID_POINT = 9
NOALLOC_TOO_LARGE = 25
MAX_POINTS = 4096


def _lib():
    import apogee_gpu as A

    lib = A.lib()
    lib.apg_msm_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                    ctypes.c_void_p]
    return lib


def _device_bytes(torch, data: bytes):
    return torch.frombuffer(bytearray(data), dtype=torch.uint8).to("cuda:0")


def _call(torch, bases: bytes, mont_scalars: bytes, n: int):
    lib = _lib()
    d_bases = _device_bytes(torch, bases) if n else torch.zeros(64, dtype=torch.uint8, device="cuda:0")
    d_scalars = _device_bytes(torch, mont_scalars) if n else torch.zeros(32, dtype=torch.uint8, device="cuda:0")
    d_out = torch.full((64,), 0xAB, dtype=torch.uint8, device="cuda:0")
    torch.cuda.synchronize()
    rc = lib.apg_msm_noalloc(d_bases.data_ptr(), d_scalars.data_ptr(), n, d_out.data_ptr(), None)
    return rc, bytes(d_out.cpu().numpy().tobytes())


def test_noalloc_matches_msm_on_consecutive_calls():
    import torch

    import apogee_gpu as A
    import oracle_lib as O

    with A.Context(0) as ctx:
        # Two calls in a row: the full size, then a smaller one over the same
        # array (its stale contents from the first call must not leak in).
        for n, seed in ((MAX_POINTS, 11), (1000, 12)):
            bases, scalars = O.msm_case("random", n, seed)
            xs = [int.from_bytes(scalars[i:i + 32], "little") for i in range(0, len(scalars), 32)]
            mont = A.to_mont_bytes(xs)
            want = ctx.msm(bases, mont)
            rc, got = _call(torch, bases, mont, n)
            assert rc == 0
            assert got == want, f"n = {n}"
            assert got == O.msm(bases, scalars, n, threads=8), f"n = {n} against the oracle"


def test_noalloc_known_tau_and_empty():
    """Over the powers of a seeded tau the MSM is a commitment: [f(tau)]G.
    n = 0 gives the identity (64 zero bytes)."""
    import random

    import torch

    import apogee_gpu as A
    import oracle_lib as O

    tau = 0xA110C
    n = 3000
    srs = O.toy_srs(tau, n)
    rng = random.Random(7)
    coeffs = [rng.choice([0, 1, rng.getrandbits(32), rng.randrange(O.P_R)]) for _ in range(n)]
    rc, got = _call(torch, srs, A.to_mont_bytes(coeffs), n)
    assert rc == 0
    assert got == O.g1_mul(O.G1_GEN, O.poly_at(b"".join(O.fe(c) for c in coeffs), n, tau))
    rc, got = _call(torch, b"", b"", 0)
    assert rc == 0 and got == bytes(64)


def test_noalloc_error_paths():
    """A scalar >= r and a base off the curve are refused with their status;
    the next call still computes the right value."""
    import torch

    import apogee_gpu as A
    import oracle_lib as O

    n = 64
    bases, scalars = O.msm_case("random", n, 21)
    xs = [int.from_bytes(scalars[i:i + 32], "little") for i in range(0, len(scalars), 32)]
    mont = bytearray(A.to_mont_bytes(xs))
    bad_scalar = bytes(mont[:32 * 5]) + O.P_R.to_bytes(32, "little") + bytes(mont[32 * 6:])
    rc, _ = _call(torch, bases, bad_scalar, n)
    assert rc == NONCANONICAL
    off = bytearray(bases)
    off[64 * 3] ^= 1  # breaks the curve equation
    rc, _ = _call(torch, bytes(off), bytes(mont), n)
    assert rc == INVALID_POINT
    rc, got = _call(torch, bases, bytes(mont), n)
    assert rc == 0 and got == O.msm(bases, scalars, n)


def test_noalloc_allocates_nothing():
    """Around a call (after the first one on the device, which loads the
    module), the device's free memory does not move."""
    import torch

    import apogee_gpu as A
    import oracle_lib as O

    n = 2048
    bases, scalars = O.msm_case("random", n, 33)
    xs = [int.from_bytes(scalars[i:i + 32], "little") for i in range(0, len(scalars), 32)]
    lib = _lib()
    d_bases = _device_bytes(torch, bases)
    d_scalars = _device_bytes(torch, A.to_mont_bytes(xs))
    d_out = torch.zeros(64, dtype=torch.uint8, device="cuda:0")
    torch.cuda.synchronize()
    assert lib.apg_msm_noalloc(d_bases.data_ptr(), d_scalars.data_ptr(), n, d_out.data_ptr(), None) == 0
    free0, _ = torch.cuda.mem_get_info()
    assert lib.apg_msm_noalloc(d_bases.data_ptr(), d_scalars.data_ptr(), n, d_out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert bytes(d_out.cpu().numpy().tobytes()) == O.msm(bases, scalars, n)


def test_noalloc_rejects_more_than_its_maximum():
    import torch

    lib = _lib()
    d = torch.zeros(64, dtype=torch.uint8, device="cuda:0")
    rc = lib.apg_msm_noalloc(d.data_ptr(), d.data_ptr(), MAX_POINTS + 1, d.data_ptr(), None)
    assert rc == NOALLOC_TOO_LARGE
