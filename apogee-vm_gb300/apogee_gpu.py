"""Python host mirror of the reference's hot-path interface over the C ABI
(include/apogee_gpu.h, libapogee_gpu.so).

Names and error behaviour follow the reference crates: `msm`/`msm_small_u32`
(crates/curve/src/msm.rs:48,79) raise MsmError on a length mismatch; `commit`,
`open`, `batch_open` (crates/pcs/src/lib.rs:237,313,688) raise PcsError with the
reference's variant name. Field elements cross as Python ints (canonical) or as
raw in-memory bytes; points as 64-byte canonical encodings.

There is no CPU fallback: importing this module without the compiled library,
or calling it without a CUDA device, raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("APOGEE_GPU_LIB") or os.path.join(HERE, "libapogee_gpu.so")

P_R = 21888242871839275222246405745257275088548364400416034343698204186575808495617
P_Q = 21888242871839275222246405745257275088696311157297823662689037894645226208583
R_MONT = pow(2, 256, P_R)
R_MONT_INV = pow(R_MONT, -1, P_R)
TRANSCRIPT_BYTES = 226
PROOF_BYTES = 704

STATUS = {
    0: "Ok", 1: "LengthMismatch", 2: "UnsupportedNumVars", 3: "PointLengthMismatch", 4: "SrsTooSmall",
    5: "DegenerateChallenge", 6: "EmptyBatch", 7: "BatchLengthMismatch", 8: "MixedColumnSizes",
    9: "InvalidPoint", 10: "MalformedAccumulator", 11: "VerificationFailed", 20: "NonCanonical", 21: "InvalidArgument", 22: "BadCircuit", 23: "NoSrs",
    24: "Internal", 25: "NoAllocTooLarge", 26: "Pending", 27: "UnknownTicket", 28: "MissingChallenge",
    29: "OutputShape", 30: "ProofShape", 31: "LayerInconsistency", 32: "RoundCountMismatch",
    33: "FinalEvalCountMismatch", 34: "RoundSumMismatch", 35: "FinalEvalMismatch", 100: "Cuda", 101: "OutOfMemory",
    103: "NoDevice",
}
PENDING = 26
PCS_CODES = {2, 3, 4, 5, 6, 7, 8, 9, 10, 11}


class ApogeeError(RuntimeError):
    def __init__(self, status: int, message: str = ""):
        self.status = status
        self.variant = STATUS.get(status, f"status {status}")
        super().__init__(f"{self.variant}: {message}" if message else self.variant)


class MsmError(ApogeeError):
    """curve::msm::MsmError."""


class PcsError(ApogeeError):
    """pcs_verify::PcsError."""


_lib = None


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = ctypes.CDLL(LIB_PATH)
        L.apg_last_error.restype = ctypes.c_char_p
        L.apg_ctx_stream.restype = ctypes.c_void_p
        L.apg_srs_len.restype = ctypes.c_size_t
        for name in ("apg_srs_len", "apg_last_error", "apg_ctx_stream"):
            getattr(L, name).argtypes = [ctypes.c_void_p]
        _lib = L
    return _lib


# ---------------------------------------------------------------------------
# Encodings
# ---------------------------------------------------------------------------

def to_mont_bytes(xs) -> bytes:
    """Canonical ints -> Fr in-memory (Montgomery) bytes, 32 per element."""
    return b"".join(((int(x) * R_MONT) % P_R).to_bytes(32, "little") for x in xs)


def from_mont_bytes(b: bytes):
    return [(int.from_bytes(b[i:i + 32], "little") * R_MONT_INV) % P_R for i in range(0, len(b), 32)]


def fe(x: int) -> bytes:
    return int(x).to_bytes(32, "little")


def narrow_bytes(values, bits: int) -> bytes:
    """A column's stored form (PolyBacking, crates/poly/src/lib.rs:44-57):
    bits 1 a bitset in u64 limbs (entry i = bit i % 64 of limb i / 64),
    8/16/32 little-endian unsigned integers, 0 Fr in memory."""
    if bits == 0:
        return to_mont_bytes(values)
    if bits == 1:
        limbs = [0] * ((len(values) + 63) // 64)
        for i, v in enumerate(values):
            if v:
                limbs[i // 64] |= 1 << (i % 64)
        return b"".join(x.to_bytes(8, "little") for x in limbs)
    return b"".join(int(v).to_bytes(bits // 8, "little") for v in values)


def struct_u32(blob: bytes, off: int) -> int:
    return int.from_bytes(blob[off:off + 4], "little")


class GkrValues:
    """Device-resident layer values from gkr_forward (gkr::LayerValues)."""

    def __init__(self, ctx, handle):
        self.ctx = ctx
        self.handle = handle
        ctx._values.add(self)

    def read(self, layer: int, col: int):
        L = lib()
        L.apg_gkr_values_len.restype = ctypes.c_size_t
        n = L.apg_gkr_values_len(self.handle, ctypes.c_size_t(layer))
        out = ctypes.create_string_buffer(32 * n)
        st = L.apg_gkr_values_read(self.handle, ctypes.c_size_t(layer), ctypes.c_size_t(col), out)
        if st:
            raise ApogeeError(st, "apg_gkr_values_read")
        return from_mont_bytes(out.raw)

    def free(self):
        # Values live on their context's device memory: free them while the
        # context is open (Context.close frees any still alive first).
        if self.handle and self.ctx._h:
            lib().apg_gkr_values_free(self.handle)
        self.handle = None
        self.ctx._values.discard(self)

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Transcript snapshots (crates/transcript/src/lib.rs)
# ---------------------------------------------------------------------------

def transcript_init() -> bytes:
    snap = ctypes.create_string_buffer(TRANSCRIPT_BYTES)
    lib().apg_transcript_init(snap)
    return snap.raw


def transcript_append_scalars(snap: bytes, tag: int, xs) -> bytes:
    buf = ctypes.create_string_buffer(bytes(snap), TRANSCRIPT_BYTES)
    data = to_mont_bytes(xs)
    st = lib().apg_transcript_append_scalars(buf, ctypes.c_uint64(tag), data, ctypes.c_size_t(len(xs)))
    if st:
        raise ApogeeError(st, "apg_transcript_append_scalars")
    return buf.raw


def transcript_challenge(snap: bytes, tag: int):
    buf = ctypes.create_string_buffer(bytes(snap), TRANSCRIPT_BYTES)
    out = ctypes.create_string_buffer(32)
    st = lib().apg_transcript_challenge(buf, ctypes.c_uint64(tag), out)
    if st:
        raise ApogeeError(st, "apg_transcript_challenge")
    return buf.raw, from_mont_bytes(out.raw)[0]


# ---------------------------------------------------------------------------
# The GKR verifier (crates/gkr-verify/src/lib.rs:647), host only
# ---------------------------------------------------------------------------

class GkrError(ApogeeError):
    """gkr_verify::GkrError: `variant` is MissingChallenge, OutputShape,
    ProofShape or LayerInconsistency; `info` the slot or gate list."""

    def __init__(self, status: int, info: int):
        super().__init__(status, f"info {info}")
        self.info = info


def gkr_verify(circuit: bytes, outputs, proof: bytes, challenges: dict, snap: bytes):
    """gkr_verify::verify: the output tables (each a bytes of Fr in memory,
    in the circuit's output-map order), the proof as apg_gkr_prove writes it,
    the external challenges {slot: int} and the transcript bound to the base.
    Returns (base point, base claim values, the advanced transcript) with
    canonical ints; raises GkrError where the reference returns a GkrError."""
    n_out = len(outputs)
    bufs = [ctypes.create_string_buffer(bytes(o), max(len(o), 1)) for o in outputs]
    ptrs = (ctypes.c_void_p * max(n_out, 1))(*[ctypes.cast(b, ctypes.c_void_p).value for b in bufs])
    lens = (ctypes.c_size_t * max(n_out, 1))(*[len(o) // 32 for o in outputs])
    slots = sorted(challenges)
    sarr = (ctypes.c_uint32 * max(len(slots), 1))(*slots)
    vals = to_mont_bytes([challenges[k] for k in slots])
    tr = ctypes.create_string_buffer(bytes(snap), TRANSCRIPT_BYTES)
    # The APGC header: magic, version, trace_vars, n_committed (u32 LE).
    nv, ncols = (int.from_bytes(circuit[o:o + 4], "little") for o in (8, 12)) if len(circuit) >= 16 else (0, 0)
    if nv > 40 or ncols > 1 << 20:
        raise ApogeeError(22, "apg_gkr_verify: bad base shape")
    point = ctypes.create_string_buffer(32 * max(nv, 1))
    values = ctypes.create_string_buffer(32 * max(ncols, 1))
    info = ctypes.c_uint64(0)
    st = lib().apg_gkr_verify(circuit, ctypes.c_size_t(len(circuit)), ptrs, lens, ctypes.c_size_t(n_out), proof,
                              ctypes.c_size_t(len(proof)), sarr, vals, ctypes.c_size_t(len(slots)), tr, point, values,
                              ctypes.byref(info))
    if st in (28, 29, 30, 31):
        raise GkrError(st, info.value)
    if st:
        raise ApogeeError(st, "apg_gkr_verify")
    return from_mont_bytes(point.raw[:32 * nv]), from_mont_bytes(values.raw[:32 * ncols]), tr.raw


class VerifyPcsError(PcsError):
    """pcs_verify::PcsError from a verification: `info` names the refused
    point (0..7 the proof's h, q, g, s, d, pi_z, w, w'; 8 a commitment)."""

    def __init__(self, status: int, info: int):
        super().__init__(status, f"info {info}")
        self.info = info


def _deferred_result(st, info, sides, scalars, points, tr, name):
    if st in PCS_CODES:
        raise VerifyPcsError(st, info.value)
    if st:
        raise ApogeeError(st, name)
    return (bytes(sides.raw[:12]), from_mont_bytes(scalars.raw[:12 * 32]),
            [points.raw[64 * i:64 * i + 64] for i in range(12)], tr.raw)


def mercury_verify_deferred(cm: bytes, u, v: int, proof: bytes, snap: bytes):
    """pcs::verify_deferred: the commitment (64 bytes), the point u and the
    value v (canonical ints), the 704-byte proof and the transcript before
    the opening. Returns (sides, scalars, points, transcript after): the
    twelve accumulator entries, scalars as canonical ints."""
    sides, scalars, points = (ctypes.create_string_buffer(n) for n in (12, 12 * 32, 12 * 64))
    tr = ctypes.create_string_buffer(bytes(snap), TRANSCRIPT_BYTES)
    info = ctypes.c_uint64(0)
    st = lib().apg_mercury_verify_deferred(bytes(cm), to_mont_bytes(u), ctypes.c_size_t(len(u)), to_mont_bytes([v]),
                                           bytes(proof), tr, sides, scalars, points, ctypes.byref(info))
    return _deferred_result(st, info, sides, scalars, points, tr, "apg_mercury_verify_deferred")


def mercury_batch_verify_deferred(cms, u, vs, proof: bytes, snap: bytes):
    """pcs::batch_verify_deferred over k commitments (64 bytes each) claimed
    to open to vs at u. Returns what mercury_verify_deferred returns."""
    sides, scalars, points = (ctypes.create_string_buffer(n) for n in (12, 12 * 32, 12 * 64))
    tr = ctypes.create_string_buffer(bytes(snap), TRANSCRIPT_BYTES)
    info = ctypes.c_uint64(0)
    st = lib().apg_mercury_batch_verify_deferred(b"".join(cms), ctypes.c_size_t(len(cms)), to_mont_bytes(u),
                                                 ctypes.c_size_t(len(u)), to_mont_bytes(vs), ctypes.c_size_t(len(vs)),
                                                 bytes(proof), tr, sides, scalars, points, ctypes.byref(info))
    return _deferred_result(st, info, sides, scalars, points, tr, "apg_mercury_batch_verify_deferred")


def pairing(p: bytes, q: bytes) -> bytes:
    """curve::pairing::pairing of a canonical G1 (64 bytes) and G2 (128 bytes)
    point: the Fq12 value as 384 canonical bytes."""
    out = ctypes.create_string_buffer(384)
    st = lib().apg_pairing(bytes(p), bytes(q), out)
    if st:
        raise PcsError(st, "apg_pairing") if st in PCS_CODES else ApogeeError(st, "apg_pairing")
    return out.raw


def pairing_check(ps, qs) -> bool:
    """curve::pairing::pairing_check: prod_i e(ps[i], qs[i]) == 1."""
    holds = ctypes.c_int(0)
    st = lib().apg_pairing_check(b"".join(ps), b"".join(qs), ctypes.c_size_t(len(ps)), ctypes.byref(holds))
    if st:
        raise PcsError(st, "apg_pairing_check") if st in PCS_CODES else ApogeeError(st, "apg_pairing_check")
    return bool(holds.value)


def g2_mul(q: bytes, k: int) -> bytes:
    out = ctypes.create_string_buffer(128)
    st = lib().apg_g2_mul(bytes(q), int(k % (1 << 256)).to_bytes(32, "little"), out)
    if st:
        raise PcsError(st, "apg_g2_mul") if st in PCS_CODES else ApogeeError(st, "apg_g2_mul")
    return out.raw


def mercury_verify(vsrs: bytes, cm: bytes, u, v: int, proof: bytes, snap: bytes) -> bytes:
    """pcs::verify under the SrsVerifier's 320-byte wire form: returns the
    transcript after the verification, raises VerifyPcsError where the
    reference returns a PcsError (VerificationFailed included)."""
    tr = ctypes.create_string_buffer(bytes(snap), TRANSCRIPT_BYTES)
    info = ctypes.c_uint64(0)
    st = lib().apg_mercury_verify(bytes(vsrs), bytes(cm), to_mont_bytes(u), ctypes.c_size_t(len(u)),
                                  to_mont_bytes([v]), bytes(proof), tr, ctypes.byref(info))
    if st in PCS_CODES:
        raise VerifyPcsError(st, info.value)
    if st:
        raise ApogeeError(st, "apg_mercury_verify")
    return tr.raw


def mercury_batch_verify(vsrs: bytes, cms, u, vs, proof: bytes, snap: bytes) -> bytes:
    """pcs::batch_verify; as mercury_verify."""
    tr = ctypes.create_string_buffer(bytes(snap), TRANSCRIPT_BYTES)
    info = ctypes.c_uint64(0)
    st = lib().apg_mercury_batch_verify(bytes(vsrs), b"".join(cms), ctypes.c_size_t(len(cms)), to_mont_bytes(u),
                                        ctypes.c_size_t(len(u)), to_mont_bytes(vs), ctypes.c_size_t(len(vs)),
                                        bytes(proof), tr, ctypes.byref(info))
    if st in PCS_CODES:
        raise VerifyPcsError(st, info.value)
    if st:
        raise ApogeeError(st, "apg_mercury_batch_verify")
    return tr.raw


class SumcheckError(ApogeeError):
    """sumcheck::SumcheckError: `variant` is RoundCountMismatch,
    FinalEvalCountMismatch, RoundSumMismatch or FinalEvalMismatch; `info`
    the count found or the round."""

    def __init__(self, status: int, info: int):
        super().__init__(status, f"info {info}")
        self.info = info


def verify_zerocheck(terms, arity: int, num_vars: int, rounds, finals, snap: bytes):
    """sumcheck::verify_zerocheck over the gate `terms` ((coef, a, b-or-None),
    as prove_zerocheck takes them) of `arity` inputs: rounds as 4-tuples and
    finals as canonical ints. Returns (the claim's point, the advanced
    transcript); raises SumcheckError where the reference does."""
    nt = len(terms)
    coefs = to_mont_bytes([t[0] for t in terms])
    ta = (ctypes.c_uint32 * max(nt, 1))(*[t[1] for t in terms])
    tb = (ctypes.c_uint32 * max(nt, 1))(*[0xFFFFFFFF if t[2] is None else t[2] for t in terms])
    rb = to_mont_bytes([x for g in rounds for x in g])
    fb = to_mont_bytes(list(finals))
    tr = ctypes.create_string_buffer(bytes(snap), TRANSCRIPT_BYTES)
    point = ctypes.create_string_buffer(32 * max(num_vars, 1))
    info = ctypes.c_uint64(0)
    st = lib().apg_verify_zerocheck(ctypes.c_size_t(arity), coefs, ta, tb, ctypes.c_size_t(nt),
                                    ctypes.c_size_t(num_vars), rb, ctypes.c_size_t(len(rounds)), fb,
                                    ctypes.c_size_t(len(finals)), tr, point, ctypes.byref(info))
    if st in (32, 33, 34, 35):
        raise SumcheckError(st, info.value)
    if st:
        raise ApogeeError(st, "apg_verify_zerocheck")
    return from_mont_bytes(point.raw[:32 * num_vars]), tr.raw


# ---------------------------------------------------------------------------
# Context
# ---------------------------------------------------------------------------

class Context:
    """One device context: a CUDA stream, scratch memory and a resident SRS."""

    def __init__(self, device: int = 0):
        import weakref

        self._values = weakref.WeakSet()
        self._h = ctypes.c_void_p()
        st = lib().apg_ctx_create(device, ctypes.byref(self._h))
        if st != 0:
            raise ApogeeError(st, "apg_ctx_create")

    def close(self):
        if self._h:
            for v in list(self._values):
                v.free()
            lib().apg_ctx_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return lib().apg_ctx_stream(self._h) or 0

    def _check(self, st: int, cls=ApogeeError):
        if st != 0:
            msg = lib().apg_last_error(self._h).decode(errors="replace")
            if st == 1:
                raise MsmError(st, msg)
            if st in PCS_CODES:
                raise PcsError(st, msg)
            raise cls(st, msg)

    def synchronize(self):
        self._check(lib().apg_ctx_synchronize(self._h))

    # ---- SRS --------------------------------------------------------------
    def srs_upload(self, points: bytes):
        assert len(points) % 64 == 0
        self._check(lib().apg_srs_upload(self._h, points, ctypes.c_size_t(len(points) // 64)))

    def srs_generate(self, tau: int, n: int):
        self._check(lib().apg_srs_generate(self._h, fe(tau), ctypes.c_size_t(n)))

    def srs_download(self, n: int) -> bytes:
        out = ctypes.create_string_buffer(64 * n)
        self._check(lib().apg_srs_download(self._h, out, ctypes.c_size_t(n)))
        return out.raw

    def srs_len(self) -> int:
        return lib().apg_srs_len(self._h)

    def srs_prepare(self, cbits: int = 0):
        self._check(lib().apg_srs_prepare(self._h, cbits))

    def msm_autotune(self, d_sample: int, n_sample: int, min_log2n: int, max_log2n: int, cands=(8, 12, 16, 20)):
        """Time SRS commits of each size class with each candidate window
        width over a device sample (Fr in memory) and keep the fastest.
        Returns {log2n: width} (0 where the class was skipped)."""
        arr = (ctypes.c_int * len(cands))(*cands)
        out = (ctypes.c_int * (max_log2n - min_log2n + 1))()
        self._check(lib().apg_msm_autotune(self._h, ctypes.c_void_p(d_sample), ctypes.c_size_t(n_sample),
                                           min_log2n, max_log2n, arr, ctypes.c_size_t(len(cands)), out))
        return {min_log2n + i: out[i] for i in range(len(out))}

    # ---- MSM ----------------------------------------------------------------
    def msm(self, bases: bytes, scalars: bytes) -> bytes:
        """curve::msm::msm: bases 64-byte canonical points, scalars Fr in-memory bytes."""
        out = ctypes.create_string_buffer(64)
        self._check(lib().apg_msm(self._h, bases, ctypes.c_size_t(len(bases) // 64), scalars,
                                  ctypes.c_size_t(len(scalars) // 32), out))
        return out.raw

    def msm_small_u32(self, bases: bytes, scalars) -> bytes:
        arr = (ctypes.c_uint32 * len(scalars))(*scalars)
        out = ctypes.create_string_buffer(64)
        self._check(lib().apg_msm_small_u32(self._h, bases, ctypes.c_size_t(len(bases) // 64), arr,
                                            ctypes.c_size_t(len(scalars)), out))
        return out.raw

    # ---- deferred-pairing accumulator ---------------------------------------
    def _acc_args(self, sides, scalars: bytes, points: bytes, checks):
        n = len(sides)
        assert len(scalars) == 32 * n and len(points) == 64 * n
        cs = (ctypes.c_size_t * max(len(checks), 1))(*checks)
        return bytes(sides), scalars, points, ctypes.c_size_t(n), cs

    def discharge_msms(self, sides, scalars: bytes, points: bytes, checks):
        """pcs::discharge up to its pairing (crates/pcs/src/accumulator.rs:146-163):
        sides (0 G2One / 1 G2X a byte), scalars Fr in-memory bytes, points
        64-byte canonical, checks the group counts. Returns (A, B, nu) with A, B
        canonical points and nu as Fr in-memory bytes."""
        sd, sc, pt, n, cs = self._acc_args(sides, scalars, points, checks)
        a, b, nu = (ctypes.create_string_buffer(k) for k in (64, 64, 32))
        self._check(lib().apg_discharge_msms(self._h, sd, sc, pt, n, cs, ctypes.c_size_t(len(checks)), a, b, nu))
        return a.raw, b.raw, nu.raw

    def discharge(self, vsrs: bytes, sides, scalars: bytes, points: bytes, checks):
        """pcs::discharge (crates/pcs/src/accumulator.rs:146): the MSMs on the
        device, the pairing on the host, under the SrsVerifier's 320-byte wire
        form. Returns None; raises PcsError (VerificationFailed among them)."""
        sd, sc, pt, n, cs = self._acc_args(sides, scalars, points, checks)
        self._check(lib().apg_discharge(self._h, bytes(vsrs), sd, sc, pt, n, cs, ctypes.c_size_t(len(checks))))

    def pairing_msms(self, sides, scalars: bytes, points: bytes, checks, weights: bytes):
        """check_pairings' two MSMs (accumulator.rs:171-214) with one weight a
        check (Fr in-memory bytes). Returns (A, B)."""
        sd, sc, pt, n, cs = self._acc_args(sides, scalars, points, checks)
        assert len(weights) == 32 * len(checks)
        a, b = ctypes.create_string_buffer(64), ctypes.create_string_buffer(64)
        self._check(lib().apg_pairing_msms(self._h, sd, sc, pt, n, cs, weights, ctypes.c_size_t(len(checks)), a, b))
        return a.raw, b.raw

    # ---- commit -------------------------------------------------------------
    def commit(self, evals: bytes, num_vars: int) -> bytes:
        """pcs::commit over the resident SRS; evals are Fr in-memory bytes."""
        out = ctypes.create_string_buffer(64)
        self._check(lib().apg_commit(self._h, evals, ctypes.c_size_t(num_vars), out))
        return out.raw

    def commit_u32(self, evals, num_vars: int) -> bytes:
        arr = (ctypes.c_uint32 * len(evals))(*evals)
        out = ctypes.create_string_buffer(64)
        self._check(lib().apg_commit_u32(self._h, arr, ctypes.c_size_t(num_vars), out))
        return out.raw

    def commit_stack(self, cols, num_vars) -> bytes:
        """pcs::commit_stack: cols are Fr in-memory byte strings, num_vars one
        variable count per column (an int applies to every column)."""
        k = len(cols)
        nvs = [num_vars] * k if isinstance(num_vars, int) else list(num_vars)
        ptrs = (ctypes.c_char_p * k)(*cols)
        nv_arr = (ctypes.c_size_t * max(k, 1))(*nvs)
        out = ctypes.create_string_buffer(64)
        self._check(lib().apg_commit_stack(self._h, ptrs, nv_arr, ctypes.c_size_t(k), out))
        return out.raw

    def commit_stack_device(self, d_ptrs, num_vars) -> bytes:
        k = len(d_ptrs)
        nvs = [num_vars] * k if isinstance(num_vars, int) else list(num_vars)
        arr = (ctypes.c_void_p * max(k, 1))(*d_ptrs)
        nv_arr = (ctypes.c_size_t * max(k, 1))(*nvs)
        out = ctypes.create_string_buffer(64)
        self._check(lib().apg_commit_stack_device(self._h, arr, nv_arr, ctypes.c_size_t(k), out))
        return out.raw

    def commit_narrow(self, data: bytes, bits: int, num_vars: int) -> bytes:
        """pcs::commit of a narrow backing: `data` holds 2^num_vars values of
        `bits` bits (1: bit-packed u64 limbs; 8/16/32: little-endian)."""
        out = ctypes.create_string_buffer(64)
        self._check(lib().apg_commit_narrow(self._h, data, ctypes.c_int(bits), ctypes.c_size_t(num_vars), out))
        return out.raw

    def commit_batch(self, cols, num_vars: int) -> list:
        k = len(cols)
        ptrs = (ctypes.c_char_p * k)(*cols)
        out = ctypes.create_string_buffer(64 * k)
        self._check(lib().apg_commit_batch(self._h, ptrs, ctypes.c_size_t(k), ctypes.c_size_t(num_vars), out))
        return [out.raw[64 * j:64 * j + 64] for j in range(k)]

    def commit_device(self, d_ptr: int, num_vars: int) -> bytes:
        out = ctypes.create_string_buffer(64)
        self._check(lib().apg_commit_device(self._h, ctypes.c_void_p(d_ptr), ctypes.c_size_t(num_vars), out))
        return out.raw

    def commit_batch_device(self, d_ptrs, num_vars: int) -> list:
        k = len(d_ptrs)
        arr = (ctypes.c_void_p * k)(*d_ptrs)
        out = ctypes.create_string_buffer(64 * k)
        self._check(lib().apg_commit_batch_device(self._h, arr, ctypes.c_size_t(k), ctypes.c_size_t(num_vars), out))
        return [out.raw[64 * j:64 * j + 64] for j in range(k)]

    def commit_batch_host(self, host_ptrs, num_vars: int) -> list:
        """apg_commit_batch over raw host pointers (e.g. pinned tensors)."""
        k = len(host_ptrs)
        arr = (ctypes.c_void_p * k)(*host_ptrs)
        out = ctypes.create_string_buffer(64 * k)
        self._check(lib().apg_commit_batch(self._h, arr, ctypes.c_size_t(k), ctypes.c_size_t(num_vars), out))
        return [out.raw[64 * j:64 * j + 64] for j in range(k)]

    def fr_to_mont_device(self, d_ptr: int, n: int):
        self._check(lib().apg_fr_to_mont_device(self._h, ctypes.c_void_p(d_ptr), ctypes.c_size_t(n)))

    def synth_column(self, seed: int, kind: int, n: int, d_ptr: int):
        """n seeded benchmark Fr (canonical, 8 LE u32 words each) into device
        memory at d_ptr from the ChaCha20 keystream: kind 0 trace-like, kind 1
        uniform Fr (the layout synth.py restates in numpy)."""
        self._check(lib().apg_synth_column(self._h, ctypes.c_uint64(seed), ctypes.c_int(kind), ctypes.c_size_t(n),
                                           ctypes.c_void_p(d_ptr)))

    def launch_count(self) -> int:
        f = lib().apg_ctx_launch_count
        f.restype = ctypes.c_uint64
        return f(self._h)

    # ---- Mercury --------------------------------------------------------------
    def open(self, evals: bytes, num_vars: int, cm: bytes, u, transcript: bytes):
        """pcs::open. evals: Fr in-memory bytes; u: canonical ints. Returns
        (v canonical int, 704-byte proof, transcript)."""
        snap = ctypes.create_string_buffer(bytes(transcript), TRANSCRIPT_BYTES)
        v = ctypes.create_string_buffer(32)
        proof = ctypes.create_string_buffer(PROOF_BYTES)
        self._check(lib().apg_mercury_open(self._h, evals, ctypes.c_size_t(num_vars), cm, to_mont_bytes(u),
                                           ctypes.c_size_t(len(u)), snap, v, proof))
        return from_mont_bytes(v.raw)[0], proof.raw, snap.raw

    def batch_open(self, cols, num_vars: int, cms, u, transcript: bytes, on_device: bool = False):
        """pcs::batch_open. cols: Fr in-memory bytes per column (or device
        pointers with on_device); cms: 64-byte commitments. Returns (values,
        704-byte proof, transcript)."""
        k = len(cols)
        snap = ctypes.create_string_buffer(bytes(transcript), TRANSCRIPT_BYTES)
        vs = ctypes.create_string_buffer(32 * max(k, 1))
        proof = ctypes.create_string_buffer(PROOF_BYTES)
        cmb = b"".join(cms)
        if on_device:
            ptrs = (ctypes.c_void_p * max(k, 1))(*cols)
            st = lib().apg_mercury_batch_open_device(self._h, ptrs, ctypes.c_size_t(k), ctypes.c_size_t(num_vars), cmb,
                                                     to_mont_bytes(u), ctypes.c_size_t(len(u)), snap, vs, proof)
        else:
            ptrs = (ctypes.c_char_p * max(k, 1))(*cols)
            st = lib().apg_mercury_batch_open(self._h, ptrs, ctypes.c_size_t(k), ctypes.c_size_t(num_vars), cmb,
                                              to_mont_bytes(u), ctypes.c_size_t(len(u)), snap, vs, proof)
        self._check(st)
        return from_mont_bytes(vs.raw[:32 * k]), proof.raw, snap.raw

    def batch_open_stacked(self, stacks, num_vars, cms, u, r, transcript: bytes, on_device: bool = False):
        """pcs::batch_open_stacked. stacks: per stack its columns in slot
        order (Fr in-memory bytes, or device pointers with on_device);
        num_vars: one variable count per column, flattened (an int applies to
        every column); cms: 64-byte commitments; u, r: canonical ints.
        Returns (the stacks' values, 704-byte proof, transcript)."""
        flat = [c for st in stacks for c in st]
        nc, ns = len(flat), len(stacks)
        nvs = [num_vars] * nc if isinstance(num_vars, int) else list(num_vars)
        lens = (ctypes.c_size_t * max(ns, 1))(*[len(st) for st in stacks])
        nv_arr = (ctypes.c_size_t * max(nc, 1))(*nvs)
        snap = ctypes.create_string_buffer(bytes(transcript), TRANSCRIPT_BYTES)
        vs = ctypes.create_string_buffer(32 * max(ns, 1))
        proof = ctypes.create_string_buffer(PROOF_BYTES)
        args = (nv_arr, lens, ctypes.c_size_t(ns), b"".join(cms), ctypes.c_size_t(len(cms)), to_mont_bytes(u),
                ctypes.c_size_t(len(u)), to_mont_bytes(r), ctypes.c_size_t(len(r)), snap, vs, proof)
        if on_device:
            st = lib().apg_mercury_batch_open_stacked_device(self._h, (ctypes.c_void_p * max(nc, 1))(*flat), *args)
        else:
            st = lib().apg_mercury_batch_open_stacked(self._h, (ctypes.c_char_p * max(nc, 1))(*flat), *args)
        self._check(st)
        return from_mont_bytes(vs.raw[:32 * ns]), proof.raw, snap.raw

    # ---- zerocheck -----------------------------------------------------------
    def prove_zerocheck(self, terms, polys, num_vars: int, transcript: bytes, on_device: bool = False):
        """sumcheck::prove_zerocheck. terms: (coef, a, b-or-None) with coef a
        canonical int; polys: per column Fr in-memory bytes (or device pointers
        with on_device). Returns (rounds, finals, transcript) with rounds as
        lists of 4 canonical ints and finals canonical ints."""
        nt = len(terms)
        coefs = to_mont_bytes([t[0] for t in terms])
        ta = (ctypes.c_uint32 * max(nt, 1))(*[t[1] for t in terms])
        tb = (ctypes.c_uint32 * max(nt, 1))(*[0xFFFFFFFF if t[2] is None else t[2] for t in terms])
        k = len(polys)
        snap = ctypes.create_string_buffer(bytes(transcript), TRANSCRIPT_BYTES)
        rounds = ctypes.create_string_buffer(128 * max(num_vars, 1))
        finals = ctypes.create_string_buffer(32 * k)
        if on_device:
            ptrs = (ctypes.c_void_p * k)(*polys)
            st = lib().apg_prove_zerocheck_device(self._h, ctypes.c_size_t(k), coefs, ta, tb, ctypes.c_size_t(nt),
                                                  ptrs, ctypes.c_size_t(num_vars), snap, rounds, finals)
        else:
            ptrs = (ctypes.c_char_p * k)(*polys)
            st = lib().apg_prove_zerocheck(self._h, ctypes.c_size_t(k), coefs, ta, tb, ctypes.c_size_t(nt), ptrs,
                                           ctypes.c_size_t(num_vars), snap, rounds, finals)
        self._check(st)
        rs = from_mont_bytes(rounds.raw[:128 * num_vars])
        return [rs[4 * i:4 * i + 4] for i in range(num_vars)], from_mont_bytes(finals.raw), snap.raw

    def prove_zerocheck_narrow(self, terms, polys, bits, num_vars: int, transcript: bytes, on_device: bool = False):
        """prove_zerocheck over columns in their stored widths: polys[k] the
        column's bytes (a bitset in u64 limbs for bits 1, little-endian
        unsigned integers for 8/16/32, Fr in memory for 0) or device pointers
        with on_device. Returns what prove_zerocheck returns."""
        nt = len(terms)
        coefs = to_mont_bytes([t[0] for t in terms])
        ta = (ctypes.c_uint32 * max(nt, 1))(*[t[1] for t in terms])
        tb = (ctypes.c_uint32 * max(nt, 1))(*[0xFFFFFFFF if t[2] is None else t[2] for t in terms])
        k = len(polys)
        snap = ctypes.create_string_buffer(bytes(transcript), TRANSCRIPT_BYTES)
        rounds = ctypes.create_string_buffer(128 * max(num_vars, 1))
        finals = ctypes.create_string_buffer(32 * k)
        ptrs = (ctypes.c_void_p * k)(*polys) if on_device else (ctypes.c_char_p * k)(*polys)
        barr = (ctypes.c_uint8 * k)(*bits)
        self._check(lib().apg_prove_zerocheck_narrow(self._h, ctypes.c_size_t(k), coefs, ta, tb, ctypes.c_size_t(nt),
                                                     ptrs, barr, 1 if on_device else 0, ctypes.c_size_t(num_vars),
                                                     snap, rounds, finals))
        rs = from_mont_bytes(rounds.raw[:128 * num_vars])
        return [rs[4 * i:4 * i + 4] for i in range(num_vars)], from_mont_bytes(finals.raw), snap.raw

    # ---- GKR ------------------------------------------------------------------
    def gkr_forward_narrow(self, blob: bytes, base, bits, challenges: dict, on_device: bool = False):
        """gkr::forward over committed columns in their stored widths (see
        prove_zerocheck_narrow for the byte forms). Returns a GkrValues handle."""
        k = len(base)
        slots = sorted(challenges)
        sarr = (ctypes.c_uint32 * max(len(slots), 1))(*slots)
        vals = to_mont_bytes([challenges[s] for s in slots])
        h = ctypes.c_void_p()
        ptrs = (ctypes.c_void_p * k)(*base) if on_device else (ctypes.c_char_p * k)(*base)
        barr = (ctypes.c_uint8 * k)(*bits)
        self._check(lib().apg_gkr_forward_narrow(self._h, blob, ctypes.c_size_t(len(blob)), ptrs, barr,
                                                 1 if on_device else 0, sarr, vals, ctypes.c_size_t(len(slots)),
                                                 ctypes.byref(h)))
        return GkrValues(self, h)

    def gkr_forward(self, blob: bytes, base, challenges: dict, on_device: bool = False):
        """gkr::forward. base: committed columns as Fr in-memory bytes (layout
        order), or device pointers with on_device; challenges: {slot:
        canonical int}. Returns a GkrValues handle."""
        k = len(base)
        slots = sorted(challenges)
        sarr = (ctypes.c_uint32 * max(len(slots), 1))(*slots)
        vals = to_mont_bytes([challenges[s] for s in slots])
        h = ctypes.c_void_p()
        if on_device:
            ptrs = (ctypes.c_void_p * k)(*base)
            st = lib().apg_gkr_forward_device(self._h, blob, ctypes.c_size_t(len(blob)), ptrs, sarr, vals,
                                              ctypes.c_size_t(len(slots)), ctypes.byref(h))
        else:
            ptrs = (ctypes.c_char_p * k)(*base)
            st = lib().apg_gkr_forward(self._h, blob, ctypes.c_size_t(len(blob)), ptrs, sarr, vals,
                                       ctypes.c_size_t(len(slots)), ctypes.byref(h))
        self._check(st)
        return GkrValues(self, h)

    def gkr_prove(self, blob: bytes, values: "GkrValues", challenges: dict, transcript: bytes,
                  with_point: bool = False):
        """gkr::prove. Returns (proof as canonical ints in the documented
        layout, transcript) and, with with_point, the base layer's point."""
        L = lib()
        L.apg_gkr_proof_len.restype = ctypes.c_size_t
        cap = L.apg_gkr_proof_len(blob, ctypes.c_size_t(len(blob)))
        out = ctypes.create_string_buffer(max(cap, 32))
        n = ctypes.c_size_t()
        slots = sorted(challenges)
        sarr = (ctypes.c_uint32 * max(len(slots), 1))(*slots)
        vals = to_mont_bytes([challenges[s] for s in slots])
        snap = ctypes.create_string_buffer(bytes(transcript), TRANSCRIPT_BYTES)
        point = ctypes.create_string_buffer(32 * 64)
        self._check(L.apg_gkr_prove(self._h, blob, ctypes.c_size_t(len(blob)), values.handle, sarr, vals,
                                    ctypes.c_size_t(len(slots)), snap, out, ctypes.c_size_t(cap), ctypes.byref(n),
                                    point))
        proof = from_mont_bytes(out.raw[:n.value])
        if with_point:
            nv = struct_u32(blob, 8)
            return proof, snap.raw, point.raw[:32 * nv]
        return proof, snap.raw

    def gkr_prove_sumcheck(self, blob: bytes, layer: int, weights, challenges: dict, eq_point, d_lower,
                           d_upper, transcript: bytes):
        """gkr::prove_sumcheck for gate list `layer` over device tables
        (d_lower, and d_upper for a halving list: pointers to 2^len(eq_point)
        Fr each). Returns (rounds as 4-tuples, point, finals, transcript), the
        field elements as canonical ints."""
        L = lib()
        n, width = len(eq_point), len(d_lower)
        slots = sorted(challenges)
        sarr = (ctypes.c_uint32 * max(len(slots), 1))(*slots)
        vals = to_mont_bytes([challenges[s] for s in slots])
        lo = (ctypes.c_void_p * max(width, 1))(*d_lower)
        up = (ctypes.c_void_p * max(width, 1))(*(d_upper or [0] * width))
        snap = ctypes.create_string_buffer(bytes(transcript), TRANSCRIPT_BYTES)
        rounds = ctypes.create_string_buffer(128 * max(n, 1))
        point = ctypes.create_string_buffer(32 * max(n, 1))
        finals = ctypes.create_string_buffer(64 * max(width, 1))
        self._check(L.apg_gkr_prove_sumcheck(self._h, blob, ctypes.c_size_t(len(blob)), ctypes.c_size_t(layer),
                                             to_mont_bytes(weights), ctypes.c_size_t(len(weights)), sarr, vals,
                                             ctypes.c_size_t(len(slots)), to_mont_bytes(eq_point), ctypes.c_size_t(n),
                                             lo, up, ctypes.c_size_t(width), snap, rounds, point, finals))
        r = from_mont_bytes(rounds.raw[:128 * n])
        nf = width * (2 if d_upper else 1)
        return ([tuple(r[4 * i:4 * i + 4]) for i in range(n)], from_mont_bytes(point.raw[:32 * n]),
                from_mont_bytes(finals.raw[:32 * nf]), snap.raw)

    def srs_share(self, src: "Context"):
        self._check(lib().apg_srs_share(self._h, src._h))

    def witness_digest(self, cols, num_vars: int) -> int:
        k = len(cols)
        ptrs = (ctypes.c_char_p * k)(*cols)
        out = ctypes.create_string_buffer(32)
        self._check(lib().apg_witness_digest(self._h, ptrs, ctypes.c_size_t(k), ctypes.c_size_t(num_vars), out))
        return from_mont_bytes(out.raw)[0]

    (TIMER_MSM_ACCUMULATE, TIMER_MSM_TOTAL, TIMER_SUMCHECK_ROUND, TIMER_GKR_FORWARD, TIMER_MERCURY_PASS,
     TIMER_KERNELS, TIMER_HOST_ROUND) = range(7)

    def set_timing(self, on, kernels: bool = False):
        """Timers on or off; with kernels, every launch is timed too
        (TIMER_KERNELS, the device's busy time)."""
        self._check(lib().apg_ctx_set_timing(self._h, (2 if kernels else 1) if on else 0))

    def device_bytes(self) -> int:
        L = lib()
        L.apg_ctx_device_bytes.restype = ctypes.c_size_t
        L.apg_ctx_device_bytes.argtypes = [ctypes.c_void_p]
        return L.apg_ctx_device_bytes(self._h)

    def prove_shard(self, shard: "Shard") -> "ShardProof":
        """Prove one shard (apg_prove_shard): commit, shard transcript, GKR
        forward and proof, batched opening at the base point."""
        proof = ShardProof(shard)
        self._check(lib().apg_prove_shard(self._h, ctypes.byref(shard.c), ctypes.byref(proof.c)))
        return proof

    def timer(self, which: int):
        ms = ctypes.c_double()
        n = ctypes.c_uint64()
        self._check(lib().apg_ctx_timer(self._h, which, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def probe_fq_mul_rate(self, ms: float = 200.0) -> float:
        r = ctypes.c_double()
        self._check(lib().apg_probe_fq_mul_rate(self._h, ctypes.c_double(ms), ctypes.byref(r)))
        return r.value


# ---------------------------------------------------------------------------
# Shard proofs and the server
# ---------------------------------------------------------------------------

class _CShard(ctypes.Structure):
    _fields_ = [("circuit", ctypes.c_char_p), ("circuit_len", ctypes.c_size_t),
                ("cols", ctypes.POINTER(ctypes.c_void_p)), ("n_cols", ctypes.c_size_t),
                ("cols_on_device", ctypes.c_int), ("num_vars", ctypes.c_size_t),
                ("statement_digest", ctypes.c_char_p), ("family", ctypes.c_uint32), ("index", ctypes.c_uint32),
                ("ts_lo", ctypes.c_uint64), ("ts_hi", ctypes.c_uint64), ("ext_slots", ctypes.c_void_p),
                ("ext_values", ctypes.c_char_p), ("n_ext", ctypes.c_size_t), ("decoder_width", ctypes.c_uint32)]


class _CShardProof(ctypes.Structure):
    _fields_ = [("cms", ctypes.c_void_p), ("gkr_proof", ctypes.c_void_p), ("gkr_cap", ctypes.c_size_t),
                ("gkr_len", ctypes.c_size_t), ("point", ctypes.c_void_p), ("values", ctypes.c_void_p),
                ("opening", ctypes.c_uint8 * PROOF_BYTES), ("transcript", ctypes.c_uint8 * TRANSCRIPT_BYTES),
                ("phase_ms", ctypes.c_double * 4)]


class _CTimes(ctypes.Structure):
    _fields_ = [("submit_ns", ctypes.c_uint64), ("admit_ns", ctypes.c_uint64), ("start_ns", ctypes.c_uint64),
                ("done_ns", ctypes.c_uint64), ("reserved_bytes", ctypes.c_uint64), ("worker", ctypes.c_int),
                ("phase_ms", ctypes.c_double * 4)]


class _CStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("submitted", "completed", "failed", "queued", "in_flight", "workers",
                                                "peak_workers", "peak_in_flight", "held_bytes", "reserved_bytes")]
    _fields_ += [("kernel_ms", ctypes.c_double), ("host_round_ms", ctypes.c_double)]


class _CServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget", ctypes.c_size_t), ("hbm_reserve", ctypes.c_size_t), ("max_workers", ctypes.c_int),
                ("timing", ctypes.c_int)]


class Shard:
    """One shard request (apg_shard): the circuit blob, its committed columns
    (device pointers, or host bytes with on_device=False; Fr in memory) and
    the shard's identity for its transcript seed
    (verifier_core::shard_transcript)."""

    def __init__(self, circuit: bytes, cols, num_vars: int, digest: int, family: int, index: int, ts_lo: int,
                 ts_hi: int, on_device: bool = True, ext=None, decoder_width: int = 0):
        """`ext`: {slot: value} for the statement-level challenge slots the
        circuit reads (the memory challenges 1-4, a window's constant 5);
        `decoder_width`: the circuit's decoder lookup tuple width (0 if it
        has no decoder channel). The shard draws g and beta itself."""
        self.circuit = bytes(circuit)
        self.cols = list(cols)  # keeps host buffers alive
        self.num_vars = num_vars
        if on_device:
            ptrs = self.cols
        else:
            self._host = [ctypes.c_char_p(c) for c in self.cols]
            ptrs = [ctypes.cast(h, ctypes.c_void_p).value for h in self._host]
        self._ptrs = (ctypes.c_void_p * len(ptrs))(*ptrs)
        self._digest = to_mont_bytes([digest])
        ext = dict(ext or {})
        self._ext_slots = (ctypes.c_uint32 * max(len(ext), 1))(*sorted(ext))
        self._ext_values = to_mont_bytes([ext[k] for k in sorted(ext)]) if ext else b""
        self.c = _CShard(self.circuit, len(self.circuit), ctypes.cast(self._ptrs, ctypes.POINTER(ctypes.c_void_p)),
                         len(self.cols), 1 if on_device else 0, num_vars, self._digest, family, index, ts_lo, ts_hi,
                         ctypes.cast(self._ext_slots, ctypes.c_void_p), self._ext_values or None, len(ext),
                         decoder_width)


class ShardProof:
    """Where a shard proof lands (apg_shard_proof), with readers."""

    def __init__(self, shard: Shard):
        k, nv = len(shard.cols), shard.num_vars
        L = lib()
        L.apg_gkr_proof_len.restype = ctypes.c_size_t
        cap = L.apg_gkr_proof_len(shard.circuit, ctypes.c_size_t(len(shard.circuit)))
        self._cms = ctypes.create_string_buffer(64 * k)
        self._gkr = ctypes.create_string_buffer(max(cap, 32))
        self._point = ctypes.create_string_buffer(32 * max(nv, 1))
        self._values = ctypes.create_string_buffer(32 * k)
        self.k, self.nv = k, nv
        self.c = _CShardProof(ctypes.cast(self._cms, ctypes.c_void_p), ctypes.cast(self._gkr, ctypes.c_void_p), cap,
                              0, ctypes.cast(self._point, ctypes.c_void_p), ctypes.cast(self._values, ctypes.c_void_p))

    @property
    def cms(self):
        return [self._cms.raw[64 * j:64 * j + 64] for j in range(self.k)]

    @property
    def gkr(self):
        return from_mont_bytes(self._gkr.raw[:self.c.gkr_len])

    @property
    def point(self):
        return from_mont_bytes(self._point.raw[:32 * self.nv])

    @property
    def values(self):
        return from_mont_bytes(self._values.raw[:32 * self.k])

    @property
    def opening(self) -> bytes:
        return bytes(self.c.opening)

    @property
    def transcript(self) -> bytes:
        return bytes(self.c.transcript)

    @property
    def phase_ms(self):
        return list(self.c.phase_ms)


class Server:
    """The library's shard-proof server (apg_server): continuous batching with
    admission by measured free HBM. Workers share `owner`'s SRS and tables."""

    def __init__(self, owner: Context, hbm_budget: int = 0, hbm_reserve: int = 0, max_workers: int = 0,
                 timing: bool = False):
        self.owner = owner
        self._h = ctypes.c_void_p()
        cfg = _CServerConfig(hbm_budget, hbm_reserve, max_workers, 1 if timing else 0)
        st = lib().apg_server_create(owner.handle, ctypes.byref(cfg), ctypes.byref(self._h))
        if st:
            raise ApogeeError(st, "apg_server_create")
        self._live = {}

    def submit(self, shard: Shard) -> int:
        proof = ShardProof(shard)
        t = ctypes.c_uint64()
        st = lib().apg_submit(self._h, ctypes.byref(shard.c), ctypes.byref(proof.c), ctypes.byref(t))
        if st:
            raise ApogeeError(st, "apg_submit")
        self._live[t.value] = (shard, proof)
        return t.value

    def _result(self, st, ticket, tm):
        if st == PENDING:
            return None
        if st:
            raise ApogeeError(st, f"shard request {ticket}")
        _, proof = self._live[ticket]
        times = {"submit_ns": tm.submit_ns, "admit_ns": tm.admit_ns, "start_ns": tm.start_ns,
                 "done_ns": tm.done_ns, "reserved_bytes": tm.reserved_bytes, "worker": tm.worker,
                 "phase_ms": list(tm.phase_ms)}
        return proof, times

    def poll(self, ticket: int):
        """None while pending, else (ShardProof, times)."""
        tm = _CTimes()
        return self._result(lib().apg_poll(self._h, ctypes.c_uint64(ticket), ctypes.byref(tm)), ticket, tm)

    def wait(self, ticket: int):
        tm = _CTimes()
        return self._result(lib().apg_wait(self._h, ctypes.c_uint64(ticket), ctypes.byref(tm)), ticket, tm)

    def stats(self) -> dict:
        s = _CStats()
        st = lib().apg_server_query(self._h, ctypes.byref(s))
        if st:
            raise ApogeeError(st, "apg_server_query")
        return {n: getattr(s, n) for n, _ in _CStats._fields_}

    def close(self):
        if self._h:
            lib().apg_server_destroy(self._h)
            self._h = ctypes.c_void_p()
            self._live.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
