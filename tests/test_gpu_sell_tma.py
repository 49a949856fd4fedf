"""The streamed sliced-ELL product (variant 4: one warp per slice, the slice brought into shared
memory by bulk copies several stages ahead) against the register-staged one-warp-per-slice form
with 8-element groups (variant 1): the same elements in the same order, so the products and the
solves built on them are bitwise the same, FP64 and mixed precision, on matrices with long rows,
empty rows, a dense row and ragged slice widths; and no stage wait ever gives up."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import GOLDEN
from dmrg_c_gb300 import abi, ed_models, sb_models, workloads

pytestmark = pytest.mark.gpu

V_U8, V_TMA = 1, 4


def _cases(oracle, rng):
    """(name, CRS, lower-triangle storage?)"""
    cases = []
    A = sp.random(5000, 5000, density=0.002, random_state=3, format="csr").tolil()
    A[17, :4000] = rng.standard_normal(4000)          # one dense row: 4000 elements in one slice
    A = A.tocsr()
    A.eliminate_zeros()
    cases.append(("dense_row", abi.Crs.from_scipy(A), False))
    B = sp.random(3001, 3001, density=0.001, random_state=4, format="csr")   # many empty rows
    cases.append(("empty_rows", abi.Crs.from_scipy(B), False))
    basis, row, col, val = oracle.ed_build(ed_models.hubbard_chain(8, U=4.0))
    cases.append(("hubbard8", abi.Crs(row, col, val), False))
    cases.append(("xxz_superblock_m64", workloads.xxz_superblock_m64(0).explicit_lower(), True))
    return cases


def _matrix(gpu, crs, lower):
    return gpu.DeviceMatrix(crs, gpu.DG_STORE_LOWER_DIAG_LAST if lower else gpu.DG_STORE_FULL, gpu.DG_VALUES_BOTH)


@pytest.mark.parametrize("grid", [1, 7, 600])
def test_streamed_product_is_bitwise_the_register_form(gpu, oracle, rng, grid):
    for name, crs, lower in _cases(oracle, rng):
        m = _matrix(gpu, crs, lower)
        x = rng.standard_normal(crs.n)
        x32 = x.astype(np.float32)
        out = {}
        for var in (V_U8, V_TMA):
            m.set_sell_shape(1, grid)
            m.set_sell_variant(var)
            out[var] = (m.spmv(x), m.spmv(x, sigma=-0.75), m.spmv_mixed(x32))
        for a, b in zip(out[V_U8], out[V_TMA]):
            assert np.array_equal(a, b), name
        assert m.sell_error() == 0


@pytest.mark.parametrize("mixed", [0, 2], ids=["fp64", "mixed2"])
def test_streamed_solve_is_bitwise_the_register_form(gpu, mixed):
    """Lanczos + inverse iteration / refinement on the Hubbard m=512 superblock (L=64, U=4, 4th sweep) of the reference's own
    Hubbard run (n = 238,462, 236 elements a row): the same energy bit for bit."""
    path = GOLDEN / "dmrg_hubbard_vf_sweep4.npz"
    if not path.exists():
        pytest.skip("no Hubbard m=512 superblock fixture")
    sb = sb_models.load_dmrg_superblock(path)
    s = gpu.SuperblockCRS(sb.model)
    res = {}
    for var in (V_U8, V_TMA):
        m = s.matrix(gpu.DG_VALUES_BOTH)
        m.set_sell_shape(1, 1216)
        m.set_sell_variant(var)
        p = gpu.default_params(mixed=mixed, seed=7, lanczos_acc=1e-14, cg_acc=1e-7, cg_max_step=2000)
        v, info = gpu.ground_state(m, p)
        res[var] = (info.eig_val, info.lanczos_steps, info.cg_steps, v)
        assert m.sell_error() == 0
    assert res[V_U8][:3] == res[V_TMA][:3]
    assert np.array_equal(res[V_U8][3], res[V_TMA][3])
    assert abs(res[V_TMA][0] - sb.gs_val) <= 1e-10 * abs(sb.gs_val)
