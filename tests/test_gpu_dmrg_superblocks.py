"""Superblocks of the reference's own DMRG runs (tests/golden/dmrg_<model>_sweep<k>.npz: the
largest superblock of every finite sweep of main/dmrg/{xxz_vf,klm_vf,hubbard_vf} at the
benchmark configurations), built and solved on the GPU.

* the device build from the recorded term list is bitwise the reference's GET_HAM_LLLRRRRL CRS
  (dg64 checksums of Row, Col and Val);
* the FP64 solve and both mixed-precision forms reach the reference's gs_val
  (DMRG_DIAGONALIZE_SUPERBLOCK_SYM, e.g. main/dmrg/hubbard_vf/src/allocations/GET_GROUND_STATE.c:18)
  within |dE|/|E| <= 1e-10, with |<psi|psi_ref>| >= 1 - 1e-9;
* the drop-in DMRG_DIAGONALIZE_SUPERBLOCK_SYM, called through the C-ABI with the host CRS, fills
  DMRG_STATUS / DMRG_TIME as the reference does.
"""
import ctypes as C
import functools

import numpy as np
import pytest

from conftest import GOLDEN
from dmrg_c_gb300 import abi, sb_models, status_files

TOL_E = 1e-10
TOL_OV = 1e-9
FIXTURES = sorted(GOLDEN.glob("dmrg_*_sweep*.npz"))
IDS = [p.stem.replace("dmrg_", "") for p in FIXTURES]


def _params(gpu, sb, mixed=0):
    """The driver's solver settings (main/dmrg/<model>/src/main/main.c): cg_acc 1e-6 and 1000 steps
    for xxz_vf, 1e-7 and 2000 for klm_vf / hubbard_vf; Lanczos_Slow for xxz_vf."""
    xxz = sb.name.startswith("xxz")
    return gpu.default_params(mixed=mixed, seed=7, lanczos_acc=1e-14, cg_acc=1e-6 if xxz else 1e-7,
                              cg_max_step=1000 if xxz else 2000, lanczos_slow=int(xxz))


@pytest.fixture(scope="module")
def loaded():
    return functools.lru_cache(maxsize=4)(sb_models.load_dmrg_superblock)


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=IDS)
def test_dmrg_superblock_build_is_the_references(gpu, oracle, loaded, path):
    sb = loaded(path)
    s = gpu.SuperblockCRS(sb.model)
    row, col, val = s.download()
    assert row[-1] == sb.nnz
    assert (oracle.dg64(row), oracle.dg64(col), oracle.dg64(val)) == sb.crs_dg64


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [0, 1, 2], ids=["fp64", "mixed1", "mixed2"])
@pytest.mark.parametrize("path", FIXTURES, ids=IDS)
def test_dmrg_superblock_ground_state(gpu, loaded, path, mixed):
    sb = loaded(path)
    s = gpu.SuperblockCRS(sb.model)
    m = s.matrix(gpu.DG_VALUES_BOTH if mixed else gpu.DG_VALUES_F64)
    v, info = gpu.ground_state(m, _params(gpu, sb, mixed))
    assert info.converged
    dE = abs(info.eig_val - sb.gs_val) / abs(sb.gs_val)
    assert dE <= TOL_E, (sb.name, mixed, info.eig_val, sb.gs_val, dE)
    ov = abs(v @ sb.gs_vec) / (np.linalg.norm(v) * np.linalg.norm(sb.gs_vec))
    assert ov >= 1 - TOL_OV, (sb.name, mixed, ov)


@pytest.mark.gpu
@pytest.mark.parametrize("model", ["xxz_vf", "klm_vf", "hubbard_vf"])
def test_dmrg_dropin_on_final_superblock(gpu, oracle, loaded, in_tmp, model):
    """The drop-in through the C-ABI on the last recorded sweep's superblock, from host arrays, with
    the driver's parameters; gs_val, gs_error, GS_Vec and the DMRG_TIME fields."""
    paths = sorted(GOLDEN.glob(f"dmrg_{model}_sweep*.npz"))
    if not paths:
        pytest.skip(f"no {model} fixture")
    sb = loaded(paths[-1])
    row, col, val = gpu.SuperblockCRS(sb.model).download()
    low = abi.Crs(row, col, val, n=sb.model.n)
    lib = gpu.load()
    par = abi.DMRG_PARAMETER()
    par.Diag_Method = b"Lanczos_Slow" if model == "xxz_vf" else b"Lanczos"
    par.Lan_Con, par.II_Type, par.Initial_Guess = b"Normal", b"CG", b"No"
    par.diag_acc, par.diag_min_step, par.diag_max_step = 1e-14, 1, 800
    par.cg_acc, par.cg_max_step = (1e-6, 1000) if model == "xxz_vf" else (1e-7, 2000)
    par.inv_iter_acc, par.inv_iter_diag_add, par.inv_iter_max_step = 1e-9, 1e-11, 3
    gs = np.zeros(low.n)
    st = abi.DMRG_STATUS()
    st.GS_Vec = abi.ptr(gs, C.c_double)
    tm = abi.DMRG_TIME()
    lib.DMRG_DIAGONALIZE_SUPERBLOCK_SYM(low.ref, C.byref(tm), C.byref(par), C.byref(st), 8)
    assert abs(st.gs_val - sb.gs_val) <= TOL_E * abs(sb.gs_val)
    assert st.gs_error < 1e-9 and tm.diag > 0 and tm.inv_iter > 0
    assert abs(gs @ sb.gs_vec) / (np.linalg.norm(gs) * np.linalg.norm(sb.gs_vec)) >= 1 - TOL_OV
    # the step's line of result/SystemInfo/Energy_<sweep>.txt from what the drop-in filled, against
    # the reference run's line: sizes and step counter identical, E and E/N within the tolerance
    z = np.load(GOLDEN / f"dmrg_{model}_steps.npz")
    i = int(np.flatnonzero((z["sweep"] == sb.sweep) & (z["LL_site"] == sb.LL_site) & (z["RR_site"] == sb.RR_site))[0])
    ref_lines = [str(e).split("\t", 1)[1] for e in z["energy_sweep_txt"] if str(e).startswith(f"{sb.sweep}\t")]
    ref_lines = [ln for ln in ref_lines if ln and not ln.startswith("###")]
    k = i - int(np.flatnonzero(z["sweep"] == sb.sweep)[0])
    mine = status_files.energy_sweep_line(sb.LL_site, sb.RR_site, i + 1, st.gs_val, st.gs_error).split()
    ref = ref_lines[k].split()
    assert mine[:3] == ref[:3]
    assert abs(float(mine[3]) - float(ref[3])) <= TOL_E * abs(float(ref[3])) + 1e-15
    assert abs(float(mine[4]) - float(ref[4])) <= TOL_E * abs(float(ref[4])) + 1e-15
