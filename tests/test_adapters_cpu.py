"""The C++ adapters (include/p3g_adapters.hpp) compile and link without a GPU:
against stand-ins of the reference's types, and -- where the reference's
headers are present -- inside the reference's own TwoAdicFriPcs,
MerkleTreeMmcs and TwoAdicFriFolding in place of the CPU classes."""
import os

import pytest

from conftest import compile_cpp

# the reference's src/include directory; the tests that need it are skipped
# when the variable is unset
REF_INCLUDE = os.environ.get("P3G_REFERENCE_INCLUDE", "")


def test_standin_program_compiles_and_links(tmp_path):
    rc, log = compile_cpp("adapters_standin.cpp", str(tmp_path / "standin"))
    assert rc == 0, log
    assert "warning" not in log, log


@pytest.mark.skipif(not (REF_INCLUDE and os.path.isdir(REF_INCLUDE)),
                    reason="P3G_REFERENCE_INCLUDE does not name the reference headers")
def test_adapters_drop_into_reference_types(tmp_path):
    rc, log = compile_cpp("adapters_reference.cpp", str(tmp_path / "ref"), ["-I", REF_INCLUDE])
    assert rc == 0, log
    assert os.path.exists(tmp_path / "ref")


@pytest.mark.skipif(not (REF_INCLUDE and os.path.isdir(REF_INCLUDE)),
                    reason="P3G_REFERENCE_INCLUDE does not name the reference headers")
def test_proof_wire_format_round_trips_through_reference_verifier(tmp_path):
    """include/p3g_proof.hpp: a TwoAdicFriPcs proof and its opened values made by
    the reference's own prover survive encode/decode byte for byte, the
    reference's verifier accepts the decoded objects and rejects a changed
    opened value, and malformed input is refused (tests/cpp/proof_wire.cpp;
    host code only, so it runs here)."""
    import subprocess
    out = str(tmp_path / "wire")
    rc, log = compile_cpp("proof_wire.cpp", out, ["-I", REF_INCLUDE])
    assert rc == 0, log
    assert "warning" not in log, log
    r = subprocess.run([out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL OK" in r.stdout
