"""C-ABI checks that need no GPU: the library loads, exports every function the headers
declare, and the ctypes mirrors have the C layouts (and, where the reference tree is
present, the reference headers' layouts)."""
import re
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT

HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ \*]*?\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", text,
                             flags=re.M):
            if not m.group(0).lstrip().startswith("typedef"):
                names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert "LANCZOS_SYM" in names and "dg_ground_state" in names and "EXACT_V_M_Q3" in names
    out = subprocess.run(["nm", "-D", "--defined-only", str(ROOT / "dmrg_c_gb300" / "libdmrg_gb300.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = sorted(names - exported)
    assert not missing, f"declared but not exported: {missing}"
    for n in names:
        getattr(lib, n)


def test_python_signatures_cover_headers():
    from dmrg_c_gb300 import lib as L
    assert declared_functions() == set(L.SIGNATURES)


STRUCTS = ["CRS1", "BOX_CG", "BOX_II", "BOX_LAN", "DMRG_PARAMETER", "DMRG_TIME", "DMRG_BASIS", "DMRG_STATUS",
           "DMRG_BOX_LAN", "DMRG_BOX_CG", "DMRG_BOX_II", "EXACT_PARAMETER", "EXACT_TIME", "EXACT_HAM_INFO",
           "EXACT_BASIS_INFO", "EXACT_WHOLE_BASIS_Q1", "EXACT_WHOLE_BASIS_Q2", "EXACT_WHOLE_BASIS_Q3",
           "DMRG_WHOLE_BASIS_Q1", "DMRG_WHOLE_BASIS_Q2", "DMRG_WHOLE_BASIS_Q3", "DMRG_WHOLE_BASIS_Q4", "CCS1",
           "DMRG_SYSTEM_INFO"]


def c_layout(tmp_path: Path, include_dirs, header):
    """sizeof and field offsets of every struct, from the C compiler."""
    from dmrg_c_gb300 import abi
    lines = [f'#include "{header}"', "#include <stdio.h>", "#include <stddef.h>", "int main(void) {"]
    for s in STRUCTS:
        cls = getattr(abi, s)
        lines.append(f'printf("{s} %zu\\n", sizeof({s}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{s}.{f} %zu\\n", offsetof({s}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", *[f"-I{d}" for d in include_dirs], str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    return dict(line.split() for line in out.splitlines())


def ctypes_layout():
    import ctypes as C

    from dmrg_c_gb300 import abi
    out = {}
    for s in STRUCTS:
        cls = getattr(abi, s)
        out[s] = str(C.sizeof(cls))
        for f, _ in cls._fields_:
            out[f"{s}.{f}"] = str(getattr(cls, f).offset)
    return out


def test_struct_layouts_match_our_header(tmp_path):
    assert c_layout(tmp_path, [ROOT / "include"], "dmrg_gb300.h") == ctypes_layout()


def test_struct_layouts_match_reference_headers(tmp_path):
    ref = Path("/root/reference/include")
    if not (ref / "SML.h").exists():
        pytest.skip("reference headers not present")
    (tmp_path / "both.h").write_text('#include "dmrg.h"\n#include "exact.h"\n')
    assert c_layout(tmp_path, [ref, tmp_path], "both.h") == ctypes_layout()


def test_headers_compile_after_reference_headers(tmp_path):
    """A reference translation unit can include our header after its own."""
    ref = Path("/root/reference/include")
    if not (ref / "SML.h").exists():
        pytest.skip("reference headers not present")
    src = tmp_path / "tu.c"
    src.write_text('#include "SML.h"\n#include "dmrg.h"\n#include "exact.h"\n#include "dmrg_gb300.h"\nint main(void){return 0;}\n')
    subprocess.run(["gcc", f"-I{ref}", f"-I{ROOT / 'include'}", "-c", str(src), "-o", str(tmp_path / "tu.o")], check=True)


def test_native_api_without_device_reports_nodevice(lib):
    """With no CUDA device the native API returns DG_ERR_NODEVICE (never a CPU result)."""
    from dmrg_c_gb300 import lib as L
    if L.device_count() > 0:
        pytest.skip("a device is present")
    import numpy as np
    from dmrg_c_gb300 import abi
    crs = abi.Crs(np.array([0, 1]), np.array([0], np.int32), np.array([1.0]))
    with pytest.raises(L.DgError) as e:
        L.DeviceMatrix(crs)
    assert e.value.code == 6
