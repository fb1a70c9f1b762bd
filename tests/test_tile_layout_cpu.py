"""The in-CTA transform's shared-memory index arithmetic (csrc/ntt.cuh),
checked on the host for every tile shape: the split form of a swizzled tile
address equals the full form for the rows each super-stage touches, and the
stage-ordered twiddle table holds each super-stage's exponents
(tests/cpp/tile_layout.cu, compiled by nvcc as host code; no GPU)."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="nvcc not found")
def test_tile_addresses_and_twiddle_table(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = str(tmp_path / "tile_layout")
    cmd = [nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-I", os.path.join(REPO, "plonky3-gpu_gb300", "csrc"),
           "-I", os.path.join(REPO, "include"), os.path.join(REPO, "tests", "cpp", "tile_layout.cu"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([out], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "mismatches 0" in r.stdout, r.stdout + r.stderr
