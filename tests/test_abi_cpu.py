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


def _fortran_types(text: str) -> dict:
    """The `type, bind(c)` blocks of INTEGRATION.md's Fortran module: name ->
    [(field, bytes)] in order, arrays expanded to their element count."""
    import re
    kinds = {"c_int32_t": 4, "c_int": 4, "c_int64_t": 8, "c_double": 8, "c_float": 4, "c_size_t": 8}
    out = {}
    for m in re.finditer(r"type, bind\(c\) :: (\w+)\n(.*?)\n\s*end type", text, re.S):
        fields = []
        for line in m.group(2).splitlines():
            line = line.split("!")[0].strip()
            if not line:
                continue
            decl, names = line.split("::")
            size = 8 if "c_ptr" in decl else kinds[re.search(r"\((c_\w+)\)", decl).group(1)]
            for nm in names.split(","):
                nm = nm.strip()
                a = re.match(r"(\w+)\((\d+)\)", nm)
                fields.append((a.group(1), size * int(a.group(2))) if a else (nm, size))
        out[m.group(1)] = fields
    return out


def _c_struct(text: str, name: str) -> list:
    import re
    sizes = {"int32_t": 4, "int64_t": 8, "uint64_t": 8, "double": 8, "float": 4}
    body = re.search(r"typedef struct " + name + r" \{(.*?)\} " + name + ";", text, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = re.sub(r"^const\s+", "", decl.strip())
        if not decl:
            continue
        m = re.match(r"(\w+)\s*(\*?)\s*(.*)", decl)
        base, ptr, rest = m.groups()
        for nm in rest.split(","):
            nm = nm.strip()
            a = re.match(r"(\w+)\[(\d+)\]", nm)
            size = 8 if ptr or nm.startswith("*") else sizes[base]
            nm = nm.lstrip("*")
            fields.append((a.group(1), size * int(a.group(2))) if a else (nm, size))
    return fields


def test_fortran_binding_matches_header():
    """INTEGRATION.md's ISO_C_BINDING types have the header's fields, in order and of the same sizes."""
    root = Path(__file__).resolve().parents[1]
    ftypes = _fortran_types((root / "INTEGRATION.md").read_text())
    header = (root / "include" / "mcx.h").read_text()
    assert {"mcx_balance_opts", "mcx_transport_opts", "mcx_lines", "mcx_line_ref", "mcx_sens_opts",
            "mcx_adjoint_out"} <= set(ftypes)
    for name, ffields in ftypes.items():
        assert ffields == _c_struct(header, name), name
