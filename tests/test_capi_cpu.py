"""C-ABI checks that need no GPU: the library loads, exports every function
include/p3g.h declares, and reports errors through status codes."""
import ctypes as C
import os
import re

import pytest

import p3g_gb300 as P

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(REPO, "include", "p3g.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(p3g_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_expected_entry_points():
    assert set(P.EXPORTS) <= set(_declared())


def test_library_exports_every_declared_symbol():
    L = P.load()
    missing = [n for n in _declared() if not hasattr(L, n)]
    assert not missing, missing


def test_version_and_status_strings():
    L = P.load()
    assert L.p3g_version() == 1
    assert L.p3g_status_string(0) == b"ok"
    assert L.p3g_status_string(1) == b"invalid argument"


def test_null_arguments_rejected_without_gpu_work():
    L = P.load()
    # a null context is rejected before any CUDA call
    rc = L.p3g_coset_lde(None, 0, None, 4, 4, 1, 31, 1, None, None)
    assert rc == 1
    buf = C.create_string_buffer(256)
    L.p3g_last_error(buf, 256)
    assert b"null" in buf.value
    assert L.p3g_ctx_create(0, None) == 1
    assert L.p3g_dft(None, 0, P.DFT, None, 4, 4, 0, 0, None, None) == 1
    assert L.p3g_bb4_axpy(None, None, None, 4, None, None) == 1
    assert L.p3g_pcs_open_values(None, None, 4, 4, 0, 31, None, 1, None, None) == 1


def test_seeded_constants_match_oracle():
    import oracle as O
    ini, ter, inr = P.seeded_constants_bb16(13)
    oi, ot, on = O.example_constants_bb16()
    assert ini.tolist() == oi.reshape(-1).tolist()
    assert ter.tolist() == ot.reshape(-1).tolist()
    assert inr.tolist() == on.tolist()
    ini, ter, inr = P.seeded_constants_gl8(22)
    oi, ot, on = O.example_constants_gl8()
    assert [int(x) for x in ini] == [int(x) for x in oi.reshape(-1)]
    assert [int(x) for x in inr] == [int(x) for x in on]
