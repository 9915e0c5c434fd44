"""The device field inversion (Bernstein-Yang divsteps in batches of 30,
`inverse_divsteps` in field.cuh) is plain C++ marked __host__ __device__, so
the very code the kernels run is compiled for the host here and checked on
40,000 inputs of both fields; the GPU suite exercises it again inside every
MSM (the pair rounds invert a product per block, every result is normalised
to affine)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_divsteps_inverse_on_host(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = tmp_path / "inverse_check"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-x", "cu", "-I", os.path.join(ROOT, "apogee-vm_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "inverse_check.cu"), "-o", str(exe)], check=True,
                   capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 bad" in r.stdout
