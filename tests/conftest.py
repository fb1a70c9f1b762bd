import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("", "oracle", "plonky3-gpu_gb300"):
    p = os.path.join(REPO, sub) if sub else REPO
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def golden():
    import json
    with open(os.path.join(REPO, "tests", "golden", "golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def gpu_ctx():
    """One library context on cuda:0 with the seeded Poseidon2 constants."""
    import p3g_gb300 as P
    ctx = P.Context(0)
    ctx.set_default_poseidon2()
    yield ctx
    ctx.close()


def compile_cpp(src: str, out: str, extra=()):
    """g++ -std=c++17 of a test program against include/ and the built library;
    returns (returncode, compiler output)."""
    import subprocess
    import p3g_gb300 as P
    libdir = os.path.dirname(P.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(REPO, "include"), *extra,
           os.path.join(REPO, "tests", "cpp", src), "-L", libdir, "-lp3g_gb300", f"-Wl,-rpath,{libdir}", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.returncode, r.stdout + r.stderr
