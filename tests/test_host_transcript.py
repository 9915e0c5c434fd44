"""The library's host transcript needs no GPU: the same replays of the
reference's permutation vectors, transcript scripts and I/O digests as the
GPU suite's, run in the CPU suite too (so a change to the host field
arithmetic is checked on every machine the library is built on)."""
import pytest

from test_gpu_transcript import *  # noqa: F401,F403

pytestmark = pytest.mark.cpu_host
