"""Device kernels compiled as host C++ (tests/host_kernels/shim.h) and run
once per thread index on the CPU, against the reference's own semantics:
the image file packing against its PNG and TGA writers, and the batched
hit test against the sequential is_point_in_path.  The GPU tests run the
same kernels on the device (tests/test_encode.py, tests/test_points_in_path.py)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..")
HERE = os.path.join(ROOT, "tests", "host_kernels")


def _cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    return inc if os.path.exists(os.path.join(inc, "cuda_runtime.h")) else None


def _run(tmp_path, sources):
    inc = _cuda_include()
    if not shutil.which("g++") or inc is None:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path / "check")
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-w", "-I", os.path.join(ROOT, "include"), "-I", inc,
           *sources, "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return subprocess.run([exe], check=True, capture_output=True, text=True).stdout.strip()


def test_pack_kernels_match_reference_writers(tmp_path):
    out = _run(tmp_path, [os.path.join(HERE, "pack_check.cpp")])
    assert out.endswith("mismatching 0"), out
    assert not out.startswith("cases 0"), out


def test_hit_kernel_matches_sequential_is_point_in_path(tmp_path):
    out = _run(tmp_path, [os.path.join(HERE, "hit_check.cpp"),
                          os.path.join(ROOT, "canvas_ity_gb300", "csrc", "canvas.cpp")])
    assert out.endswith("differing 0"), out
    assert not out.startswith("queries 0"), out
