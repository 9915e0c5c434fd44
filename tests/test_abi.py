"""CPU checks of the C ABI: the library builds, loads without a GPU, and
exports every symbol the public header declares."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            text = open(os.path.join(ROOT, "include", f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"\b(apg_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def built_lib():
    import build_lib

    path = build_lib.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("apg_ctx_create", "apg_msm", "apg_msm_small_u32", "apg_commit", "apg_srs_upload"):
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    missing = [n for n in declared_symbols() if not hasattr(built_lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_host_module_refuses_without_library(tmp_path, monkeypatch):
    import apogee_gpu

    monkeypatch.setattr(apogee_gpu, "_lib", None)
    monkeypatch.setattr(apogee_gpu, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(ImportError):
        apogee_gpu.lib()


def test_montgomery_encoding_round_trip():
    import apogee_gpu as A

    xs = [0, 1, 2, A.P_R - 1, 12345678901234567890]
    assert A.from_mont_bytes(A.to_mont_bytes(xs)) == xs
    # R itself is the in-memory form of one (crates/field/src/lib.rs:197).
    assert A.to_mont_bytes([1]) == A.R_MONT.to_bytes(32, "little")


def test_binding_struct_layouts_match_the_header(built_lib):
    """The ctypes mirrors of the header's structs have the C sizes (a field
    added on one side only would shift every later field)."""
    import apogee_gpu as A

    built_lib.apg_abi_sizes.restype = ctypes.c_size_t
    out = (ctypes.c_size_t * 5)()
    assert built_lib.apg_abi_sizes(out, ctypes.c_size_t(5)) == 5
    mirrors = [A._CShard, A._CShardProof, A._CTimes, A._CStats, A._CServerConfig]
    assert list(out) == [ctypes.sizeof(m) for m in mirrors]
