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


STRUCTS = [("mcx_setup_opts", "SetupOpts"), ("mcx_setup_info", "SetupInfo"), ("mcx_phase_opts", "PhaseOpts"),
           ("mcx_phase_stats", "PhaseStats"), ("mcx_balance_opts", "BalanceOpts"),
           ("mcx_balance_stats", "BalanceStats"), ("mcx_transport_opts", "TransportOpts"),
           ("mcx_transport_stats", "TransportStats"), ("mcx_iterate_opts", "IterateOpts"),
           ("mcx_iterate_stats", "IterateStats"), ("mcx_lines", "Lines"),
           ("mcx_noalloc_transport_args", "NoallocTransportArgs")]


def test_struct_layouts_match_the_header(tmp_path):
    """Every ABI struct has the same size and field offsets in include/mcx.h (compiled by the C
    compiler) as in the ctypes mirror the Python host uses."""
    import ctypes
    import shutil
    import subprocess
    from pathlib import Path
    from mocassin_xray_gb300 import abi
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    inc = Path(__file__).resolve().parents[1] / "include"
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "mcx.h"', "int main(void) {"]
    for cname, pyname in STRUCTS:
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in getattr(abi, pyname)._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", str(inc), str(src), "-o", str(exe)], check=True)
    got = {}
    for row in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        name, field, val = row.split()
        got[(name, field)] = int(val)
    for cname, pyname in STRUCTS:
        cls = getattr(abi, pyname)
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for field, _ in cls._fields_:
            assert got[(cname, field)] == getattr(cls, field).offset, f"{cname}.{field}"
