"""The C-ABI library loads and exports every symbol of include/gbxtb.h
(no device calls: this runs without a GPU)."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def lib():
    from dxtb_gb300 import _lib, build

    build.build()
    return _lib.load()


def declared():
    text = (ROOT / "include" / "gbxtb.h").read_text()
    return sorted(set(re.findall(r"\b(gbxtb_\w+)\s*\(", text)))


def test_header_matches_binding():
    from dxtb_gb300 import _lib

    assert sorted(_lib.EXPORTED) == declared()


def test_exports(lib):
    for name in declared():
        assert hasattr(lib, name), name


def test_version_and_errors(lib):
    from dxtb_gb300 import _lib

    assert lib.gbxtb_version() == 1
    # argument errors are reported without touching a device
    assert lib.gbxtb_ctx_create(None, None) == _lib.GBXTB_OK - 1
    assert b"null" in lib.gbxtb_last_error()
    h = C.c_void_p()
    ws = C.c_size_t()
    assert lib.gbxtb_plan_create(None, 0, None, None, None, None, C.byref(h), C.byref(ws)) == -1
    assert lib.gbxtb_get_status(None, None, None) == -1
