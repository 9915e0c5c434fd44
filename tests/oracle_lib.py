"""ctypes access to the CPU oracle (oracle/liboracle.so), plus the small
field/RNG helpers the tests share.

The oracle is test infrastructure: the tests use it to check the CUDA
library, never the other way round.
"""
import ctypes
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")

P_R = 21888242871839275222246405745257275088548364400416034343698204186575808495617
P_Q = 21888242871839275222246405745257275088696311157297823662689037894645226208583
SNAP = 226

_lib = None


def lib():
    global _lib
    if _lib is None:
        so = os.path.join(ORACLE_DIR, "liboracle.so")
        srcs = [os.path.join(ORACLE_DIR, f) for f in os.listdir(ORACLE_DIR) if f.endswith((".cpp", ".hpp"))]
        if not os.path.exists(so) or any(os.path.getmtime(s) > os.path.getmtime(so) for s in srcs):
            subprocess.check_call(["make", "-s", "-C", ORACLE_DIR])
        _lib = ctypes.CDLL(so)
        _lib.oracle_time_msm.restype = ctypes.c_double
    return _lib


def fe(x: int) -> bytes:
    return int(x).to_bytes(32, "little")


def fe_int(b: bytes) -> int:
    return int.from_bytes(b, "little")


def hexb(s: str) -> bytes:
    return bytes.fromhex(s)


class Rng:
    """splitmix64, as tools/test-support/src/lib.rs:26-66 defines it."""

    def __init__(self, seed: int):
        self.s = seed & 0xFFFFFFFFFFFFFFFF

    def next_u64(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        return z ^ (z >> 31)

    def next_le32(self) -> bytes:
        return b"".join(self.next_u64().to_bytes(8, "little") for _ in range(4))

    def next_fr(self) -> int:
        """Rejection sampling with the top two bits cleared
        (crates/curve/tests/common/mod.rs:33-41)."""
        while True:
            b = bytearray(self.next_le32())
            b[31] &= 0x3F
            v = int.from_bytes(b, "little")
            if v < P_R:
                return v


def buf(n: int):
    return ctypes.create_string_buffer(n)


def new_snapshot() -> bytearray:
    s = buf(SNAP)
    lib().oracle_transcript_new(s)
    return bytearray(s.raw)


def transcript_op(snap: bytearray, op: int, tag: int = 0, data: bytes = b"", n: int = 0) -> bytes:
    s = (ctypes.c_uint8 * SNAP).from_buffer(snap)
    out = buf(32)
    rc = lib().oracle_transcript_op(s, op, ctypes.c_uint64(tag), data, ctypes.c_size_t(n), out)
    assert rc == 0, f"oracle transcript op {op} failed: {rc}"
    return out.raw


def g1_mul(point: bytes, k: int) -> bytes:
    out = buf(64)
    assert lib().oracle_g1_op(2, point, fe(k), out) == 0
    return out.raw


G1_GEN = fe(1) + fe(2)


def msm(bases: bytes, scalars: bytes, n: int, threads: int = 4) -> bytes:
    out = buf(64)
    rc = lib().oracle_msm(bases, scalars, ctypes.c_size_t(n), ctypes.c_size_t(threads), out)
    assert rc == 0, rc
    return out.raw


def toy_srs(tau: int, count: int, threads: int = 8) -> bytes:
    out = buf(64 * count)
    assert lib().oracle_toy_srs(fe(tau), ctypes.c_size_t(count), ctypes.c_size_t(threads), out) == 0
    return out.raw


def msm_case(pattern: str, n: int, seed: int):
    """The input expansion of the MSM corpus (crates/curve/tests/msm.rs:41-69):
    n bases k*G, then n scalars; 'infinity' zeroes every third base,
    'zeros' and 'identical' rewrite the scalars after drawing them."""
    rng = Rng(seed)
    bases = []
    for i in range(n):
        k = rng.next_fr()
        bases.append(b"\x00" * 64 if (pattern == "infinity" and i % 3 == 0) else g1_mul(G1_GEN, k))
    draws = [rng.next_fr() for _ in range(n)]
    if pattern == "zeros":
        scalars = [0] * n
    elif pattern == "identical":
        scalars = [draws[0] if n else 0] * n
    else:
        scalars = draws
    return b"".join(bases), b"".join(fe(s) for s in scalars)


def golden_lines(name: str):
    with open(os.path.join(GOLDEN, name)) as f:
        for line in f:
            line = line.rstrip("\n")
            if line and not line.startswith("#"):
                yield line


TAG_NAMES = {
    "PROTOCOL_SUITE": 1, "PUBLIC_INPUTS": 2, "COMMITMENT": 3, "SUMCHECK_ROUND": 4, "SUMCHECK_CHALLENGE": 5,
    "EVALUATION_CLAIM": 6, "PCS_OPENING": 7, "WITNESS_DIGEST": 8, "SUMCHECK_FINAL_EVALS": 9,
    "MERCURY_INSTANCE": 10, "MERCURY_ALPHA": 11, "MERCURY_GAMMA": 12, "MERCURY_Z": 13, "BDFG_BATCH": 14,
    "BDFG_POINT": 15, "PAIRING_MERGE": 16, "MERCURY_BATCH": 17, "ACCUMULATOR_DIGEST": 18,
    "ACCUMULATOR_MERGE": 19, "PUBLIC_INPUT_STREAM": 20, "PUBLIC_OUTPUT_STREAM": 21, "PROGRAM_IDENTITY": 22,
    "VM_CONFIG": 23, "SHARD_COUNTS": 24, "GKR_OUTPUTS": 25, "GKR_OUTPUT_POINT": 26, "GKR_BATCH": 27,
    "GKR_LAYER_CLAIMS": 28, "GKR_CHILD": 29, "MEMORY_WINDOWS": 30, "MEMORY_BOUNDARY": 31, "PROGRAM_ENTRY": 32,
    "LOOKUP_CHALLENGE": 33, "SRS_DIGEST": 34, "SRS_VERIFIER": 35, "MEMORY_GROUP": 36, "MEMORY_CHALLENGE": 37,
    "GLOBAL_STATE_DIGEST": 38, "SHARD_SEED": 39, "SHARD_TS_WINDOW": 40, "GENERIC_TABLE": 41,
    "STACK_CHALLENGE": 42, "FOLD_STATE": 43, "FOLD_WEIGHT": 44, "FOLD_CHILD": 45,
}


def golden_artifacts():
    """The reference's committed circuit artifacts: {file name: bytes}."""
    d = os.path.join(GOLDEN, "artifacts")
    return {f: open(os.path.join(d, f), "rb").read() for f in sorted(os.listdir(d)) if f.endswith(".bin")}


# ---- the deferred-pairing accumulator --------------------------------------

INFINITY_SENTINEL = 1 << 128


def golden_accumulator():
    """accumulator.txt: the toy tau, the concatenated accumulator's words and
    their digest (crates/pcs/tests/vectors/accumulator.txt)."""
    tau, words, digest = None, {}, None
    for line in golden_lines("accumulator.txt"):
        t = line.split()
        if t[0] == "tau":
            tau = fe_int(hexb(t[1]))
        elif t[0] == "word":
            words[int(t[1])] = fe_int(hexb(t[2]))
        elif t[0] == "digest":
            digest = fe_int(hexb(t[1]))
    return tau, [words[i] for i in range(len(words))], digest


def entries_from_words(words):
    """accumulator_from_words (crates/pcs/src/accumulator.rs:90-126, limbs
    decoded as g1_from_limbs :292-318): (sides, scalars, points, checks) with
    sides as bytes, scalars as ints, points as 64-byte encodings."""
    sides, scalars, points, checks = [], [], [], []
    at = 0
    while at < len(words):
        count = words[at]
        at += 1
        assert count < 1 << 64 and count <= (len(words) - at) // 6, "malformed count word"
        for _ in range(count):
            side, scalar, limbs = words[at], words[at + 1], words[at + 2:at + 6]
            assert side in (0, 1), "malformed side tag"
            if all(x == INFINITY_SENTINEL for x in limbs):
                point = bytes(64)
            else:
                assert all(x < INFINITY_SENTINEL for x in limbs), "malformed limb"
                point = b"".join(x.to_bytes(16, "little") for x in limbs)
            sides.append(side)
            scalars.append(scalar)
            points.append(point)
            at += 6
        checks.append(count)
    return bytes(sides), scalars, points, checks


def accumulator_msms(sides: bytes, scalars, points, checks, weights=None, threads: int = 8):
    """The oracle's group side of discharge (weights None) or check_pairings:
    (status, A, B, nu, digest) with A, B as 64-byte points, nu and digest ints."""
    import ctypes as ct
    n = len(sides)
    a, b, nu, dg = buf(64), buf(64), buf(32), buf(32)
    cs = (ct.c_uint64 * max(len(checks), 1))(*checks)
    w = b"".join(fe(x) for x in weights) if weights is not None else None
    rc = lib().oracle_accumulator_msms(bytes(sides), b"".join(fe(s) for s in scalars), b"".join(points),
                                       ct.c_size_t(n), cs, ct.c_size_t(len(checks)), w, ct.c_size_t(threads),
                                       a, b, nu, dg)
    return rc, a.raw, b.raw, fe_int(nu.raw), fe_int(dg.raw)


def accumulator_words(sides: bytes, scalars, points, checks):
    import ctypes as ct
    n = len(sides)
    out = buf(32 * (len(checks) + 6 * n))
    cs = (ct.c_uint64 * max(len(checks), 1))(*checks)
    rc = lib().oracle_accumulator_words(bytes(sides), b"".join(fe(s) for s in scalars), b"".join(points),
                                        ct.c_size_t(n), cs, ct.c_size_t(len(checks)), out)
    assert rc == 0, rc
    return [fe_int(out.raw[32 * i:32 * i + 32]) for i in range(len(checks) + 6 * n)]


def mle_eval(table, point):
    """A multilinear table (variable j = bit j of the index) at `point`."""
    t = [x % P_R for x in table]
    for rj in point:
        t = [(t[2 * i] + rj * (t[2 * i + 1] - t[2 * i])) % P_R for i in range(len(t) // 2)]
    return t[0]


def batch_open_stacked(srs: bytes, srs_n: int, stacks, col_nv, cms, u, r, snap: bytearray, threads: int = 8):
    """The oracle's batch_open_stacked over canonical-int columns (stack after
    stack, column c of 2^col_nv[c] entries). Returns (rc, values, proof); rc
    is 0, or 10 + the oracle's refusal status. `snap` advances in place."""
    flat = [c for st in stacks for c in st]
    nc, ns = len(flat), len(stacks)
    nvs = (ctypes.c_size_t * max(nc, 1))(*col_nv)
    lens = (ctypes.c_size_t * max(ns, 1))(*[len(st) for st in stacks])
    s = (ctypes.c_uint8 * SNAP).from_buffer(snap)
    vs, proof = buf(32 * max(ns, 1)), buf(704)
    rc = lib().oracle_mercury_batch_open_stacked(
        srs, ctypes.c_size_t(srs_n), b"".join(fe(x) for c in flat for x in c), nvs, lens, ctypes.c_size_t(ns),
        b"".join(cms), ctypes.c_size_t(len(cms)), b"".join(fe(x) for x in u), ctypes.c_size_t(len(u)),
        b"".join(fe(x) for x in r), ctypes.c_size_t(len(r)), s, ctypes.c_size_t(threads), vs, proof)
    return rc, [fe_int(vs.raw[32 * j:32 * j + 32]) for j in range(ns)], proof.raw


def poly_at(coeffs: bytes, n: int, x: int, threads: int = 16) -> int:
    """sum_i c_i x^i over n canonical 32-byte coefficients (the oracle's
    threaded Horner): the scalar of the known-tau identity cm = [f(tau)]G."""
    out = buf(32)
    rc = lib().oracle_poly_at(coeffs, ctypes.c_size_t(n), fe(x), ctypes.c_size_t(threads), out)
    assert rc == 0, rc
    return fe_int(out.raw)
