"""Parity at the benchmark sizes, on the GPU.

* The headline configuration itself: 16 mixed 2^22-point columns committed by
  one commit_batch_device call (the library splits them into four groups of
  four over its two lanes, the call the benchmark times), with the window
  tables the autotuner picks at 2^22 (18 bits) and the opening width (20
  bits); and 2^18- and 2^20-point columns at 12- and 16-bit tables. Every commitment is
  held to the known-tau identity cm = [f(tau)]G, f(tau) by the oracle's Horner.
* Config 1 at its full size: a 2^16 commit, the witness digest and the
  16-round Product zerocheck against the oracle.
* Config 2's circuit at its full size: 8 columns of 2^20 rows, the 12 gate
  lists (sumchecks of 20, 20, 20, 20, 19, ... 18 variables), forward values
  and proof against the oracle.
* Config 3's opening at 16 columns of 2^20: the batched Mercury opening
  against the oracle, byte for byte.

Columns are drawn like VM traces (synth.mixed_column): 25% {0,1}, 60% u32,
15% uniform Fr."""
import ctypes

import pytest

import oracle_lib as O

pytestmark = pytest.mark.gpu
P = O.P_R


@pytest.fixture(scope="module")
def ctx():
    import apogee_gpu as A

    with A.Context(0) as c:
        yield c


def device_mixed(ctx, n, seeds):
    """Mixed columns: (canonical numpy arrays, device Montgomery tensors)."""
    import numpy as np
    import torch

    import synth

    host, dev = [], []
    for s in seeds:
        col = synth.mixed_column(n, s)
        t = torch.from_numpy(col.view(np.int32).reshape(-1)).to("cuda:0")
        ctx.fr_to_mont_device(t.data_ptr(), n)
        host.append(col)
        dev.append(t)
    torch.cuda.synchronize()
    return host, dev


def known_tau(col, tau):
    return O.g1_mul(O.G1_GEN, O.poly_at(col.tobytes(), col.shape[0], tau))


@pytest.mark.parametrize("cbits", [18, 20])
def test_headline_commit_known_tau(ctx, cbits):
    tau = (0x7A0 + cbits) * 0x9E3779B97F4A7C15 % P
    log2n = 22
    n = 1 << log2n
    ctx.srs_generate(tau, n)
    host, dev = device_mixed(ctx, n, [4242 + 31 * cbits + j for j in range(16)])
    chosen = ctx.msm_autotune(dev[0].data_ptr(), n, log2n, log2n, cands=(cbits,))
    assert chosen == {log2n: cbits}
    cms = ctx.commit_batch_device([t.data_ptr() for t in dev], log2n)
    assert len(cms) == 16
    for j, (col, cm) in enumerate(zip(host, cms)):
        assert cm == known_tau(col, tau), f"column {j} at {cbits}-bit tables"
    # The same columns from pinned host buffers (the end-to-end leg).
    import torch

    pinned = [torch.empty_like(t, device="cpu").pin_memory() for t in dev[:4]]
    for h, t in zip(pinned, dev[:4]):
        h.copy_(t)
    assert ctx.commit_batch_host([h.data_ptr() for h in pinned], log2n) == cms[:4]
    del dev
    torch.cuda.empty_cache()


@pytest.mark.parametrize("cbits", [12, 16])
def test_mid_sizes_commit_known_tau(ctx, cbits):
    tau = (0x1D0 + cbits) * 0x9E3779B97F4A7C15 % P
    ctx.srs_generate(tau, 1 << 20)
    host, dev = device_mixed(ctx, 1 << 20, [77 + cbits])
    chosen = ctx.msm_autotune(dev[0].data_ptr(), 1 << 20, 17, 20, cands=(cbits,))
    assert chosen == {k: cbits for k in range(17, 21)}
    for log2n in (18, 20):  # commits take even variable counts (Mercury)
        n = 1 << log2n
        cols, devs = device_mixed(ctx, n, [1000 * log2n + cbits + j for j in range(5)])
        cms = ctx.commit_batch_device([t.data_ptr() for t in devs], log2n)
        for j, (col, cm) in enumerate(zip(cols, cms)):
            assert cm == known_tau(col, tau), f"2^{log2n} column {j} at {cbits}-bit tables"


def test_config1_full_size(ctx):
    """Config 1: commit a (2^16), absorb the witness digest of (a, b), prove
    the Product zerocheck a*b over 16 rounds; every byte against the oracle."""
    import random

    import apogee_gpu as A
    from test_gpu_zerocheck import run_case

    nv = 16
    n = 1 << nv
    rng = random.Random(0xC0F1)
    tau = rng.randrange(P)
    ctx.srs_generate(tau, n)
    cols = [[rng.randrange(P) for _ in range(n)] for _ in range(2)]
    cm = ctx.commit(A.to_mont_bytes(cols[0]), nv)
    want = O.buf(64)
    assert O.lib().oracle_commit(ctx.srs_download(n), ctypes.c_size_t(n), b"".join(O.fe(v) for v in cols[0]), nv,
                                 16, want) == 0
    assert cm == want.raw
    run_case(ctx, [(1, 0, 1)], cols, nv, 1)


def test_config2_circuit_full_size(ctx):
    """Config 2's circuit over 2^20 rows and 8 committed columns: the top
    layer, the 12 layer sumchecks and the claims, and the transcript after,
    equal the oracle's."""
    import numpy as np
    import torch

    import circuits as C
    import synth

    nv, width = 20, 8
    n = 1 << nv
    circ = C.shard_circuit(nv, width)
    blob = circ.to_blob()
    host, dev = device_mixed(ctx, n, [2020 + j for j in range(width)])
    ch = {0: 0x5EED5EED}
    import apogee_gpu as A

    snap = A.transcript_append_scalars(A.transcript_init(), 39, [2020])
    values = ctx.gkr_forward(blob, [t.data_ptr() for t in dev], ch, on_device=True)
    try:
        top = circ.depth()
        got_top = [values.read(top, j) for j in range(circ.width(top))]
        proof, after = ctx.gkr_prove(blob, values, ch, snap)
    finally:
        values.free()
    del dev
    torch.cuda.empty_cache()
    sarr = (ctypes.c_uint32 * 1)(0)
    osnap = bytearray(snap)
    s = (ctypes.c_uint8 * O.SNAP).from_buffer(osnap)
    n_proof = circ.proof_elems()
    top_n = 1 << circ.vars(top)
    oproof, otop = O.buf(32 * n_proof), O.buf(32 * circ.width(top) * top_n)
    base = np.concatenate(host).tobytes()
    assert O.lib().oracle_gkr_prove(blob, ctypes.c_size_t(len(blob)), base, sarr, O.fe(ch[0]), ctypes.c_size_t(1),
                                    s, oproof, otop) == 0
    want_top = [O.fe_int(otop.raw[32 * i:32 * i + 32]) for i in range(circ.width(top) * top_n)]
    assert [x for col in got_top for x in col] == want_top
    assert proof == [O.fe_int(oproof.raw[32 * i:32 * i + 32]) for i in range(n_proof)]
    assert after == bytes(osnap)
    assert synth  # the columns' distribution


def test_config3_opening_16x2p20(ctx):
    """Config 3's batched opening at 16 columns of 2^20: values, the 704-byte
    proof and the transcript after, against the oracle."""
    import random

    import numpy as np
    import torch

    import apogee_gpu as A

    nv, k = 20, 16
    n = 1 << nv
    rng = random.Random(0xC0F3)
    tau = rng.randrange(P)
    ctx.srs_generate(tau, n)
    srs = ctx.srs_download(n)
    host, dev = device_mixed(ctx, n, [3030 + j for j in range(k)])
    cms = ctx.commit_batch_device([t.data_ptr() for t in dev], nv)
    for col, cm in zip(host[:2], cms[:2]):
        assert cm == known_tau(col, tau)
    u = [rng.randrange(P) for _ in range(nv)]
    snap = A.transcript_append_scalars(A.transcript_init(), 39, [3030])
    vs, proof, after = ctx.batch_open([t.data_ptr() for t in dev], nv, cms, u, snap, on_device=True)
    del dev
    torch.cuda.empty_cache()
    osnap = bytearray(snap)
    s = (ctypes.c_uint8 * O.SNAP).from_buffer(osnap)
    ovs, oproof = O.buf(32 * k), O.buf(704)
    rc = O.lib().oracle_mercury_batch_open(srs, ctypes.c_size_t(n), np.concatenate(host).tobytes(),
                                            ctypes.c_size_t(k), nv, b"".join(cms), b"".join(O.fe(x) for x in u), s,
                                            16, ovs, oproof)
    assert rc == 0
    assert vs == [O.fe_int(ovs.raw[32 * i:32 * i + 32]) for i in range(k)]
    assert proof == oproof.raw
    assert after == bytes(osnap)
