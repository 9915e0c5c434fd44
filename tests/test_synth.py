"""The seeded benchmark inputs (synth.py): the ChaCha20 block function against
the `cryptography` package's ChaCha20, the keystream layout restated entry by
entry from that package's keystream, and the value distribution. No GPU."""
import numpy as np
import pytest

import synth


def _keystream(seed: int, stream: int, nbytes: int) -> bytes:
    """Keystream bytes from the `cryptography` package (its 16-byte nonce is
    the 32-bit initial counter followed by the RFC 8439 nonce)."""
    alg = pytest.importorskip("cryptography.hazmat.primitives.ciphers")
    cipher = alg.Cipher(alg.algorithms.ChaCha20(synth.seed_key(seed), bytes(4) + synth.stream_nonce(stream)),
                        mode=None)
    return cipher.encryptor().update(bytes(nbytes))


@pytest.mark.parametrize("seed,stream", [(0, 0), (20260903, 0), (20260903, 3), (2**64 - 1, 7)])
def test_blocks_match_cryptography(seed, stream):
    n = 3 * synth._CHUNK // 2 + 5  # crosses a chunk boundary
    want = _keystream(seed, stream, 64 * n)
    got = synth.chacha20_blocks(synth.seed_key(seed), synth.stream_nonce(stream), np.arange(n)).tobytes()
    assert got == want
    # Blocks at scattered counters are the same blocks.
    ctr = np.array([n - 1, 0, 17, 17, 4096])
    part = synth.chacha20_blocks(synth.seed_key(seed), synth.stream_nonce(stream), ctr)
    for row, c in zip(part, ctr):
        assert row.tobytes() == want[64 * c:64 * c + 64]


def _words(b: bytes, i: int) -> int:
    return int.from_bytes(b[4 * i:4 * i + 4], "little")


def _entry(seed: int, i: int, uniform: bool) -> int:
    """One entry restated from the layout, over the package's keystream."""
    if not uniform:
        s0 = _keystream(seed, 0, 64 * (i // 8 + 1))
        value, c = _words(s0, 2 * i), _words(s0, 2 * i + 1) & 0xFFFF
        if c < 16384:
            return value & 1
        if c < 55706:
            return value
    for t in range(synth.MAX_ATTEMPTS):
        s = _keystream(seed, t + 1, 32 * (i + 1))
        v = int.from_bytes(s[32 * i:32 * i + 32], "little") & ((1 << 254) - 1)
        if 0 < v < synth.P_R:
            return v
    raise AssertionError("no canonical candidate")


@pytest.mark.parametrize("n,seed", [(1, 5), (13, 77), (100, 20260903)])
def test_layout_entry_by_entry(n, seed):
    assert synth.to_ints(synth.mixed_column(n, seed)) == [_entry(seed, i, False) for i in range(n)]
    assert synth.to_ints(synth.uniform_column(n, seed)) == [_entry(seed, i, True) for i in range(n)]


def test_distribution_and_canonicity():
    n = 1 << 16
    vals = synth.to_ints(synth.mixed_column(n, 11))
    assert all(v < synth.P_R for v in vals)
    bits = sum(v < 2 for v in vals) / n
    fr = sum(v >= 1 << 32 for v in vals) / n
    assert abs(bits - 0.25) < 0.01 and abs(fr - 0.15) < 0.01
    u = synth.to_ints(synth.uniform_column(1 << 12, 11))
    assert all(0 < v < synth.P_R for v in u)
    # All 254 bits are in play: the top quarter of [0, 2^254) is rejected,
    # so about 1/3 of accepted values are at least 2^253.
    top = sum(v >> 253 for v in u) / len(u)
    assert 0.28 < top < 0.38
    # Seeds give different columns; a seed gives the same one twice.
    assert (synth.mixed_column(64, 1) != synth.mixed_column(64, 2)).any()
    assert (synth.mixed_column(64, 1) == synth.mixed_column(64, 1)).all()
    assert synth.mixed_column(0, 1).shape == (0, 8)
