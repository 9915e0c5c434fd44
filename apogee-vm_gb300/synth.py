"""Seeded synthetic inputs for the shard-proving workloads.

Columns are drawn to look like VM trace columns, the distribution the
workloads name: 25% of entries in {0, 1}, 60% uniform 32-bit register values,
15% uniform field elements.

The source of randomness is a ChaCha20 keystream (RFC 8439 §2.3 block
function, restated below) keyed from a 64-bit seed, the generator the
reference's bench tool draws its inputs from. A uniform Fr entry follows the
reference's rule (tools/bench/src/timing.rs:56-67): 32 little-endian bytes
with the top two bits cleared, redrawn while the value is >= r or zero.

Keystream layout (the device generator, csrc/synth.cu, follows the same one,
so a column made on either side from one seed is the same bytes). The key is
the seed as 8 little-endian bytes followed by 24 zero bytes; block counters
start at 0.

* stream 0 (nonce words 0, 0, 0): entry i reads word pair (2j, 2j+1),
  j = i mod 8, of block i // 8 — a 32-bit value and, in the low 16 bits of the
  second word, a class draw c: c < 16384 gives value & 1, c < 55706 gives the
  value, anything else a uniform Fr.
* stream t + 1 (nonce words t + 1, 0, 0): attempt t of entry i's uniform Fr,
  words 8 (i mod 2) .. 8 (i mod 2) + 7 of block i // 2.

A uniform column takes every entry from the attempt streams.
"""
import struct

import numpy as np

P_R = 21888242871839275222246405745257275088548364400416034343698204186575808495617

CLASS_BITS = 16384   # 25% of 2^16
CLASS_WORD = 55706   # 85% of 2^16, rounded up
MAX_ATTEMPTS = 64    # each attempt is accepted with probability > 3/4

_SIGMA = np.array([0x61707865, 0x3320646E, 0x79622D32, 0x6B206574], dtype=np.uint32)
_R_LIMBS = np.array([(P_R >> (32 * k)) & 0xFFFFFFFF for k in range(8)], dtype=np.uint32)
_CHUNK = 1 << 15     # blocks per vectorised pass: the state stays in cache


def seed_key(seed: int) -> bytes:
    """The 32-byte ChaCha20 key of a 64-bit seed."""
    return struct.pack("<Q", seed & 0xFFFFFFFFFFFFFFFF) + bytes(24)


def stream_nonce(stream: int) -> bytes:
    return struct.pack("<III", stream, 0, 0)


def _rotl(x, r, tmp):
    np.left_shift(x, np.uint32(r), out=tmp)
    np.right_shift(x, np.uint32(32 - r), out=x)
    np.bitwise_or(x, tmp, out=x)


def _quarter(x, a, b, c, d, tmp):
    x[a] += x[b]
    x[d] ^= x[a]
    _rotl(x[d], 16, tmp)
    x[c] += x[d]
    x[b] ^= x[c]
    _rotl(x[b], 12, tmp)
    x[a] += x[b]
    x[d] ^= x[a]
    _rotl(x[d], 8, tmp)
    x[c] += x[d]
    x[b] ^= x[c]
    _rotl(x[b], 7, tmp)


def chacha20_blocks(key: bytes, nonce: bytes, counters) -> np.ndarray:
    """ChaCha20 blocks (RFC 8439 §2.3) at the given 32-bit block counters:
    a (len(counters), 16) uint32 array of little-endian keystream words."""
    counters = np.asarray(counters, dtype=np.uint32).reshape(-1)
    out = np.empty((counters.size, 16), dtype=np.uint32)
    kw = np.frombuffer(key, dtype="<u4").astype(np.uint32)
    nw = np.frombuffer(nonce, dtype="<u4").astype(np.uint32)
    for lo in range(0, counters.size, _CHUNK):
        ctr = counters[lo:lo + _CHUNK]
        b = ctr.size
        init = np.empty((16, b), dtype=np.uint32)
        init[0:4] = _SIGMA[:, None]
        init[4:12] = kw[:, None]
        init[12] = ctr
        init[13:16] = nw[:, None]
        x = init.copy()
        tmp = np.empty(b, dtype=np.uint32)
        for _ in range(10):
            _quarter(x, 0, 4, 8, 12, tmp)
            _quarter(x, 1, 5, 9, 13, tmp)
            _quarter(x, 2, 6, 10, 14, tmp)
            _quarter(x, 3, 7, 11, 15, tmp)
            _quarter(x, 0, 5, 10, 15, tmp)
            _quarter(x, 1, 6, 11, 12, tmp)
            _quarter(x, 2, 7, 8, 13, tmp)
            _quarter(x, 3, 4, 9, 14, tmp)
        x += init
        out[lo:lo + b] = x.T
    return out


def _below_r_nonzero(v: np.ndarray) -> np.ndarray:
    """Rows of an (m, 8) limb array that are canonical (< r) and nonzero."""
    lt = np.zeros(v.shape[0], dtype=bool)
    eq = np.ones(v.shape[0], dtype=bool)
    for k in range(7, -1, -1):
        lt |= eq & (v[:, k] < _R_LIMBS[k])
        eq &= v[:, k] == _R_LIMBS[k]
    return lt & v.any(axis=1)


def uniform_fr(seed: int, entries) -> np.ndarray:
    """The uniform Fr of the given entry indices, an (m, 8) uint32 array."""
    key = seed_key(seed)
    entries = np.asarray(entries, dtype=np.int64).reshape(-1)
    out = np.zeros((entries.size, 8), dtype=np.uint32)
    pending = np.arange(entries.size)
    for t in range(MAX_ATTEMPTS):
        if pending.size == 0:
            return out
        idx = entries[pending]
        blocks, inv = np.unique(idx >> 1, return_inverse=True)
        blk = chacha20_blocks(key, stream_nonce(t + 1), blocks)[inv.reshape(-1)]
        cand = np.where((idx & 1).astype(bool)[:, None], blk[:, 8:], blk[:, :8])
        cand[:, 7] &= np.uint32(0x3FFFFFFF)
        ok = _below_r_nonzero(cand)
        out[pending[ok]] = cand[ok]
        pending = pending[~ok]
    if pending.size:
        raise RuntimeError(f"{pending.size} entries found no canonical Fr in {MAX_ATTEMPTS} attempts")
    return out


def mixed_column(n: int, seed: int) -> np.ndarray:
    """n canonical Fr values as an (n, 8) uint32 array (little-endian limbs),
    drawn like a VM trace column."""
    out = np.zeros((n, 8), dtype=np.uint32)
    if n == 0:
        return out
    ks = chacha20_blocks(seed_key(seed), stream_nonce(0), np.arange((n + 7) // 8)).reshape(-1, 2)[:n]
    value, cls = ks[:, 0], ks[:, 1] & np.uint32(0xFFFF)
    bits = cls < CLASS_BITS
    word = (~bits) & (cls < CLASS_WORD)
    out[bits, 0] = value[bits] & np.uint32(1)
    out[word, 0] = value[word]
    full = np.nonzero(cls >= CLASS_WORD)[0]
    out[full] = uniform_fr(seed, full)
    return out


def uniform_column(n: int, seed: int) -> np.ndarray:
    """n uniform canonical Fr with all 254 bits in play (the MSM worst case)."""
    return uniform_fr(seed, np.arange(n))


KINDS = {"mixed": 0, "uniform": 1}


def device_column(ctx, torch, n: int, seed: int, kind: str = "mixed", device: str = "cuda:0"):
    """The same column generated on the device by the library: a flat int32
    tensor of n * 8 canonical limbs."""
    t = torch.empty(n * 8, dtype=torch.int32, device=device)
    ctx.synth_column(seed, KINDS[kind], n, t.data_ptr())
    return t


def to_ints(col: np.ndarray):
    return [int.from_bytes(col[i].tobytes(), "little") for i in range(col.shape[0])]
