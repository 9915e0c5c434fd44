"""The device generator of benchmark columns (apg_synth_column) against the
host one (synth.py), byte for byte: both read the same ChaCha20 keystream
layout, so the benchmark's device-made columns are the values its host-side
checks recompute."""
import numpy as np
import pytest

import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import apogee_gpu as A

    with A.Context(0) as c:
        yield c


@pytest.mark.parametrize("n", [0, 1, 7, 9, 255, 1000, 1 << 16, (1 << 20) + 3])
@pytest.mark.parametrize("kind", ["mixed", "uniform"])
def test_device_column_matches_host(ctx, n, kind):
    import torch

    seed = 20260903 + n
    got = synth.device_column(ctx, torch, n, seed, kind, "cuda:0").cpu().numpy().view(np.uint32).reshape(n, 8)
    want = (synth.mixed_column if kind == "mixed" else synth.uniform_column)(n, seed)
    assert np.array_equal(got, want)


def test_device_column_refusals(ctx):
    import apogee_gpu as A
    import torch

    t = torch.empty(8, dtype=torch.int32, device="cuda:0")
    with pytest.raises(A.ApogeeError):
        ctx.synth_column(1, 2, 1, t.data_ptr())  # no such kind
    with pytest.raises(A.ApogeeError):
        ctx.synth_column(1, 0, 1, 0)  # null output
