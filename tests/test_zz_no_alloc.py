"""The allocation-free CG entry point (dg_cg_noalloc), for callers that cannot let a library
allocate device memory (an application whose own memory pool owns the device, or a solve path
that must not allocate).

It must give the same solution as the allocating entry point (dg_linear_solve) on the same
system, on consecutive calls that share its static scratch array, match the reference's own
CONJUGATE_GRADIENT_SYM solution (golden cg_x), reject systems larger than the array holds and
reject a malformed CRS before any product runs.  Kept in its own file, collected last."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import golden
from dmrg_c_gb300 import abi

pytestmark = pytest.mark.gpu

TOL = 1e-9    # relative difference of the two solutions (CG to ||r||^2 < 1e-20 on both sides)


def _device_system(torch, crs, b, x0):
    dev = "cuda"
    return dict(row=torch.tensor(crs.row, device=dev), col=torch.tensor(crs.col[:crs.nnz], device=dev),
                val=torch.tensor(crs.val[:crs.nnz], device=dev), b=torch.tensor(b, device=dev),
                x=torch.tensor(x0, device=dev))


def _noalloc(gpu, torch, crs, b, x0, sigma, acc=1e-20, max_step=2000):
    t = _device_system(torch, crs, b, x0)
    it = C.c_int()
    rc = gpu.load().dg_cg_noalloc(crs.n, C.c_void_p(t["row"].data_ptr()), C.c_void_p(t["col"].data_ptr()),
                                  C.c_void_p(t["val"].data_ptr()), sigma, C.c_void_p(t["b"].data_ptr()),
                                  C.c_void_p(t["x"].data_ptr()), acc, max_step, C.byref(it))
    torch.cuda.synchronize()
    return rc, it.value, t["x"].cpu().numpy()


def _reference_solution(gpu, crs, b, x0, sigma, acc=1e-20, max_step=2000):
    m = gpu.DeviceMatrix(crs)
    x = x0.copy()
    rc, it = gpu.linear_solve(m, b, x, sigma=sigma, acc=acc, max_step=max_step)
    return rc, it, x


def _systems():
    g = golden("sml_random1500.npz")
    low = abi.Crs(g["B_row"], g["B_col"], g["B_val"])
    A = abi.full_from_lower(low)                               # SPD (shifted random matrix)
    first = (abi.Crs.from_scipy(A), g["b"], g["x0"], 0.0)
    rng = np.random.default_rng(8)
    n = 20000
    B = sp.random(n, n, density=4e-4, random_state=9, data_rvs=rng.standard_normal)
    B = (B + B.T).tocsr()
    B.setdiag(0.0)
    sigma = float(abs(B).sum(axis=1).max()) + 1.0              # diagonally dominant once shifted
    second = (abi.Crs.from_scipy(B), rng.standard_normal(n), rng.standard_normal(n), sigma)
    return [first, second]


def test_noalloc_cg_matches_allocating_entry_point_twice(gpu):
    torch = pytest.importorskip("torch")
    for crs, b, x0, sigma in _systems():          # two calls in a row sharing the scratch array
        rc, it, x = _noalloc(gpu, torch, crs, b, x0, sigma)
        rc_ref, it_ref, x_ref = _reference_solution(gpu, crs, b, x0, sigma)
        assert rc == 0 and rc_ref == 0
        assert abs(it - it_ref) <= 2
        assert np.abs(x - x_ref).max() <= TOL * np.abs(x_ref).max()


def test_noalloc_cg_matches_reference_golden(gpu):
    """The first system is the golden fixture's B x = b from x0, solved by the reference's
    CONJUGATE_GRADIENT_SYM to ||r||^2 < 1e-10 (sml/CONJUGATE_GRADIENT_SYM.c)."""
    torch = pytest.importorskip("torch")
    g = golden("sml_random1500.npz")
    crs, b, x0, sigma = _systems()[0]
    rc, it, x = _noalloc(gpu, torch, crs, b, x0, sigma, acc=1e-10, max_step=1000)
    assert rc == 0
    np.testing.assert_allclose(x, g["cg_x"], rtol=0, atol=1e-8)
    assert abs(it - int(g["cg_iters"])) <= 2


def test_noalloc_cg_rejects_malformed_crs(gpu):
    """A column outside [0, n) and decreasing row offsets are refused (DG_ERR_MATRIX) by the
    device-side check, before any product gathers through them; the next good call still works."""
    torch = pytest.importorskip("torch")
    crs, b, x0, sigma = _systems()[0]
    for how in ("column", "offsets"):
        row, col = crs.row.copy(), crs.col[:crs.nnz].copy()
        if how == "column":
            col[17] = crs.n + 100
        else:
            row[40] = row[42] + 1
        bad = abi.Crs(row, col, crs.val[:crs.nnz].copy(), n=crs.n)
        rc, it, x = _noalloc(gpu, torch, bad, b, x0, sigma)
        assert rc == 7, (how, rc)
        assert b"row" in gpu.load().dg_last_error()
    rc, it, x = _noalloc(gpu, torch, crs, b, x0, sigma)
    assert rc == 0


def test_noalloc_cg_rejects_oversized_system(gpu):
    torch = pytest.importorskip("torch")
    one = torch.zeros(4, dtype=torch.float64, device="cuda")
    rows = torch.zeros(4, dtype=torch.int64, device="cuda")
    cols = torch.zeros(4, dtype=torch.int32, device="cuda")
    it = C.c_int()
    rc = gpu.load().dg_cg_noalloc((1 << 20) + 1, C.c_void_p(rows.data_ptr()), C.c_void_p(cols.data_ptr()),
                                  C.c_void_p(one.data_ptr()), 0.0, C.c_void_p(one.data_ptr()), C.c_void_p(one.data_ptr()),
                                  1e-10, 10, C.byref(it))
    assert rc == 1
    assert b"allocation-free limit" in gpu.load().dg_last_error()
