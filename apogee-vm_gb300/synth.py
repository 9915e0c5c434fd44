"""Seeded synthetic inputs for the shard-proving workloads.

Columns are drawn to look like VM trace columns, the distribution the
workloads name: 25% of entries in {0, 1}, 60% uniform 32-bit register values,
15% uniform field elements. A "uniform Fr" entry is 254 random bits with the
top limb masked below p's top limb (0x30644e72), so it is always canonical;
the bias against the top sliver of Fr is irrelevant to the arithmetic cost.

Generation uses numpy's PCG64 from an explicit seed, so both measurement arms
and the tests see identical values on any machine.
"""
import numpy as np

P_R = 21888242871839275222246405745257275088548364400416034343698204186575808495617


def mixed_column(n: int, seed: int) -> np.ndarray:
    """n canonical Fr values as an (n, 8) uint32 array (little-endian limbs)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = np.zeros((n, 8), dtype=np.uint32)
    cls = rng.random(n)
    bits = cls < 0.25
    word = (~bits) & (cls < 0.85)
    full = cls >= 0.85
    out[bits, 0] = rng.integers(0, 2, size=int(bits.sum()), dtype=np.uint32)
    out[word, 0] = rng.integers(0, 1 << 32, size=int(word.sum()), dtype=np.uint64).astype(np.uint32)
    nf = int(full.sum())
    words = rng.integers(0, 1 << 32, size=(nf, 8), dtype=np.uint64).astype(np.uint32)
    words[:, 7] &= np.uint32(0x2FFFFFFF)
    out[full] = words
    return out


def uniform_column(n: int, seed: int) -> np.ndarray:
    """n canonical Fr values with all 254 bits in play (the MSM worst case)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    words = rng.integers(0, 1 << 32, size=(n, 8), dtype=np.uint64).astype(np.uint32)
    words[:, 7] &= np.uint32(0x2FFFFFFF)
    return words


def to_ints(col: np.ndarray):
    return [int.from_bytes(col[i].tobytes(), "little") for i in range(col.shape[0])]
