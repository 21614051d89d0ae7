"""The C-ABI library loads on a machine without a GPU and exports every entry
point include/mcx.h declares; calls that need a device fail with a status
code instead of crashing."""
import ctypes
import re
from pathlib import Path

import pytest

from mocassin_xray_gb300 import abi

HEADER = Path(__file__).resolve().parents[1] / "include" / "mcx.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mcx_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = abi.lib()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the ctypes signature table covers the same set
    assert sorted(n for n, _, _ in abi.SIGNATURES) == names


def test_version_string():
    assert b"sm_103a" in abi.lib().mcx_version()


def test_context_without_device_fails_cleanly():
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = abi.lib().mcx_ctx_create(0, ctypes.byref(h))
    assert rc == 3 and not h.value   # MCX_ERR_CUDA


def test_null_arguments_are_rejected():
    lib = abi.lib()
    assert lib.mcx_setup_from_input(None, None, None, None) == 1
    assert lib.mcx_transport(None, None, None) == 1
    assert lib.mcx_opacity(None, None, None) == 1
