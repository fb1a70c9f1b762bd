"""The C++ adapters (include/p3g_adapters.hpp) compile and link without a GPU:
against stand-ins of the reference's types, and -- where the reference's
headers are present -- inside the reference's own TwoAdicFriPcs,
MerkleTreeMmcs and TwoAdicFriFolding in place of the CPU classes."""
import os

import pytest

from conftest import compile_cpp

REF_INCLUDE = os.environ.get("P3G_REFERENCE_INCLUDE", "/root/reference/src/include")


def test_standin_program_compiles_and_links(tmp_path):
    rc, log = compile_cpp("adapters_standin.cpp", str(tmp_path / "standin"))
    assert rc == 0, log
    assert "warning" not in log, log


@pytest.mark.skipif(not os.path.isdir(REF_INCLUDE), reason="reference headers not present")
def test_adapters_drop_into_reference_types(tmp_path):
    rc, log = compile_cpp("adapters_reference.cpp", str(tmp_path / "ref"), ["-I", REF_INCLUDE])
    assert rc == 0, log
    assert os.path.exists(tmp_path / "ref")
