"""The reference's committed circuit artifacts (crates/constraints/tests/
vectors/*.bin, copied by tests/golden/make_golden.py) decode from their wire
form into APGC blobs the library accepts. CPU only: no device work."""
import ctypes

import pytest

import oracle_lib as O

ARTS = O.golden_artifacts()


def test_every_committed_artifact_is_present():
    assert len(ARTS) == 16
    assert {"add_sub.bin", "mul_div.bin", "shift_bitwise.bin", "toy_cached.bin"} <= set(ARTS)


@pytest.mark.parametrize("name", sorted(ARTS))
def test_decode_and_resolve(name):
    import artifact

    art = artifact.decode(ARTS[name])
    n_committed = len(art["memory"]) + len(art["witness"]) + len(art["setup"])
    for tv in sorted({art["trace_vars"], min(6, art["trace_vars"])}):
        circuit = artifact.to_circuit(art, tv)
        assert circuit.trace_vars == tv and circuit.n_committed == n_committed
        assert circuit.vars(circuit.depth()) >= 0
        assert len(circuit.outputs) == len(art["outputs"])
        blob = circuit.to_blob()
        # The library parses the blob and agrees on the proof's size.
        import apogee_gpu as A

        L = A.lib()
        L.apg_gkr_proof_len.restype = ctypes.c_size_t
        assert L.apg_gkr_proof_len(blob, ctypes.c_size_t(len(blob))) == 32 * circuit.proof_elems()


def test_malformed_artifacts_are_refused():
    import artifact

    data = ARTS["toy_cached.bin"]
    with pytest.raises(artifact.ArtifactError):
        artifact.decode(data[:-1])
    with pytest.raises(artifact.ArtifactError):
        artifact.decode(data + b"\x00")
    with pytest.raises(artifact.ArtifactError):
        artifact.decode(b"\x02" + data[1:])  # another format version
    art = artifact.decode(data)
    with pytest.raises(artifact.ArtifactError):
        artifact.to_circuit(art, art["trace_vars"] + 1)
