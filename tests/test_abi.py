"""C-ABI checks that need no GPU: the library loads, exports every function the headers
declare, and the ctypes mirrors have the C layouts (and, where the reference tree is
present, the reference headers' layouts)."""
import os
import re
import subprocess
import sys
from pathlib import Path

import pytest

from conftest import ROOT

# the reference source tree, where it exists (its headers are compared with ours)
REF = Path(os.environ.get("DMRG_REF", "/root/reference"))

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


# the library's own structs (include/dmrg_gb300*.h)
OWN_STRUCTS = ["dg_solver_params", "dg_solve_info", "dg_tune_result", "dg_sb_term", "dg_sb_model", "dg_sb_expect_term",
               "dg_sb_basis_spec", "dg_engine_config", "dg_job_result", "dg_ed_term", "dg_ed_model"]


def c_layout(tmp_path: Path, include_dirs, header, structs=None):
    """sizeof and field offsets of every struct, from the C compiler."""
    from dmrg_c_gb300 import abi
    lines = [f'#include "{header}"', "#include <stdio.h>", "#include <stddef.h>", "int main(void) {"]
    for s in structs or STRUCTS:
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


def ctypes_layout(structs=None):
    import ctypes as C

    from dmrg_c_gb300 import abi
    out = {}
    for s in structs or STRUCTS:
        cls = getattr(abi, s)
        out[s] = str(C.sizeof(cls))
        for f, _ in cls._fields_:
            out[f"{s}.{f}"] = str(getattr(cls, f).offset)
    return out


def test_struct_layouts_match_our_header(tmp_path):
    assert c_layout(tmp_path, [ROOT / "include"], "dmrg_gb300.h") == ctypes_layout()


def test_own_struct_layouts_match_our_headers(tmp_path):
    """The ctypes mirrors of the library's own structs (solver parameters, engine configuration,
    ED and superblock models) have the C layouts."""
    hdr = tmp_path / "own.h"
    hdr.write_text("".join(f'#include "{h.name}"\n' for h in HEADERS))
    assert c_layout(tmp_path, [ROOT / "include", tmp_path], "own.h", OWN_STRUCTS) == ctypes_layout(OWN_STRUCTS)


def test_struct_layouts_match_reference_headers(tmp_path):
    ref = REF / "include"
    if not (ref / "SML.h").exists():
        pytest.skip("reference headers not present")
    (tmp_path / "both.h").write_text('#include "dmrg.h"\n#include "exact.h"\n')
    assert c_layout(tmp_path, [ref, tmp_path], "both.h") == ctypes_layout()


def test_headers_compile_after_reference_headers(tmp_path):
    """A reference translation unit can include our header after its own."""
    ref = REF / "include"
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


def _link_trace(tmp_path, objs, symbols, out_name):
    """Link objs against libdmrg_gb300.so ahead of the reference's archives (oracle/_ref) the way a
    reference program is linked (LFLAGS = -ldmrg -lonsite_op -lsml, main/dmrg/xxz_vf/makefile:17,22);
    returns {symbol: [file defining it]} from the linker's -y trace."""
    openblas = subprocess.run([sys.executable, "-c", "import scipy, os, glob; d = os.path.join(os.path.dirname(scipy.__file__), "
                               "os.pardir, 'scipy.libs'); print(os.path.abspath(sorted(glob.glob(os.path.join(d, "
                               "'libscipy_openblas*.so')))[0]))"], capture_output=True, text=True, check=True).stdout.strip()
    refdir = ROOT / "oracle" / "_ref"
    cmd = ["gcc", "-fopenmp", "-o", str(tmp_path / out_name), *map(str, objs), str(refdir / "obj" / "lapack_shim.o"),
           f"-L{ROOT / 'dmrg_c_gb300'}", "-ldmrg_gb300", f"-L{refdir}", "-ldmrg", "-lonsite_op", "-lsml", openblas, "-lm"]
    cmd += [f"-Wl,-y,{s}" for s in symbols]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    defs = {}
    for line in (r.stdout + r.stderr).splitlines():
        m = re.match(r".*?([^\s:]+): definition of (\w+)", line)
        if m:
            defs.setdefault(m.group(2), []).append(Path(m.group(1)).name)
    return defs


def _ref_build(ref):
    subprocess.run(["make", "-s", "-j8", "-C", str(ROOT / "oracle"), "archives", f"REF={ref.REF_SRC}"], check=True)


def test_reference_dmrg_program_links_the_gpu_library(ref, lib, tmp_path):
    """The reference's own Hubbard DMRG program (every object of main/dmrg/hubbard_vf, its main.c
    included, compiled unchanged) links with libdmrg_gb300 ahead of the reference archives: the
    superblock solve it calls (GET_GROUND_STATE.c:18) and the solvers resolve to the GPU library."""
    _ref_build(ref)
    objs = sorted((ROOT / "oracle" / "_ref" / "obj" / "main" / "dmrg" / "hubbard_vf").rglob("*.o"))
    assert any(o.name == "main.o" for o in objs)
    syms = ["DMRG_DIAGONALIZE_SUPERBLOCK_SYM", "LANCZOS_SYM", "INVERSE_ITERATION_SYM", "CONJUGATE_GRADIENT_SYM",
            "DMRG_GET_SYSTEM_INFO_Q2", "CRS_CRS_CCS_PRODUCT"]
    defs = _link_trace(tmp_path, objs, syms, "hubbard_vf_on_gb300")
    assert defs["DMRG_DIAGONALIZE_SUPERBLOCK_SYM"] == ["libdmrg_gb300.so"], defs
    for s in syms:
        assert defs.get(s) == ["libdmrg_gb300.so"], (s, defs.get(s))


def test_reference_solver_wrapper_links_the_gpu_solvers(ref, lib, tmp_path):
    """A reference translation unit that calls the solvers -- dmrg/DMRG_DIAGONALIZE_SUPERBLOCK_SYM.c
    itself, forced in as an object -- gets LANCZOS_SYM, LANCZOS_SLOW_SYM and INVERSE_ITERATION_SYM
    from the GPU library, not from the reference's libsml.a."""
    _ref_build(ref)
    main = tmp_path / "main.c"
    main.write_text('#include "dmrg.h"\nint main(void) { DMRG_DIAGONALIZE_SUPERBLOCK_SYM(0, 0, 0, 0, 1); return 0; }\n')
    subprocess.run(["gcc", f"-I{ref.REF_SRC / 'include'}", "-c", str(main), "-o", str(tmp_path / "main.o")], check=True)
    wrapper = ROOT / "oracle" / "_ref" / "obj" / "dmrg" / "DMRG_DIAGONALIZE_SUPERBLOCK_SYM.o"
    syms = ["LANCZOS_SYM", "LANCZOS_SLOW_SYM", "INVERSE_ITERATION_SYM"]
    defs = _link_trace(tmp_path, [tmp_path / "main.o", wrapper], syms, "wrapper_on_gb300")
    for s in syms:
        assert defs.get(s) == ["libdmrg_gb300.so"], (s, defs.get(s))
