"""apg_msm_noalloc: the MSM entry point for callers that cannot let the
library allocate device memory (a serving loop whose HBM is already promised
to admitted requests, or a pipeline that cannot take cudaMalloc's device-wide
synchronisation). It must give exactly what apg_msm gives, call after call,
although every call reuses the same fixed scratch array.

Kept in a file of its own that pytest collects last, so a run that stops at
the first failure has already run every other test."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

NOALLOC_TOO_LARGE = 25
MAX_POINTS = 4096


def _device_bytes(torch, data: bytes):
    return torch.frombuffer(bytearray(data), dtype=torch.uint8).to("cuda:0")


def test_noalloc_matches_msm_on_consecutive_calls():
    import torch

    import apogee_gpu as A
    import oracle_lib as O

    lib = A.lib()
    lib.apg_msm_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                    ctypes.c_void_p]
    with A.Context(0) as ctx:
        # Two calls in a row: the full size, then a smaller one over the same
        # array (its stale contents from the first call must not leak in).
        for n, seed in ((MAX_POINTS, 11), (1000, 12)):
            bases, scalars = O.msm_case("random", n, seed)
            xs = [int.from_bytes(scalars[i:i + 32], "little") for i in range(0, len(scalars), 32)]
            mont = A.to_mont_bytes(xs)
            want = ctx.msm(bases, mont)
            d_bases = _device_bytes(torch, bases)
            d_scalars = _device_bytes(torch, mont)
            d_out = torch.zeros(64, dtype=torch.uint8, device="cuda:0")
            torch.cuda.synchronize()
            rc = lib.apg_msm_noalloc(d_bases.data_ptr(), d_scalars.data_ptr(), n, d_out.data_ptr(), None)
            assert rc == 0
            assert bytes(d_out.cpu().numpy().tobytes()) == want, f"n = {n}"


def test_noalloc_rejects_more_than_its_maximum():
    import torch

    import apogee_gpu as A

    lib = A.lib()
    lib.apg_msm_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                    ctypes.c_void_p]
    d = torch.zeros(64, dtype=torch.uint8, device="cuda:0")
    rc = lib.apg_msm_noalloc(d.data_ptr(), d.data_ptr(), MAX_POINTS + 1, d.data_ptr(), None)
    assert rc == NOALLOC_TOO_LARGE
