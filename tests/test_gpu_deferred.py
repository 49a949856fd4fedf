"""Reductions finished by the consuming kernel against the last-block form.

The Lanczos step can leave <y,v> and <w,w> to the kernels that consume them (every consumer
block sums the producer's block partials in the same fixed order); DG_DEFER_REDUCTIONS=0 / =1
forces either form at the same launch grid.  In the FP64 form both sum the same double partials
in the same order, so energies, vectors and step counts must match bit for bit.  The mixed form's
consumer sums compensated FP32 pairs (the last-block form converts each block's pair to double
first), so there the step counts must match and the energies agree to rounding.  CG and the
refinement always use the consumer form; their parity against the reference is covered by the
golden tests.
"""
import numpy as np
import pytest

from conftest import golden
from dmrg_c_gb300 import abi

pytestmark = pytest.mark.gpu


def _solve(gpu, crs, mixed, guess, monkeypatch, mode):
    monkeypatch.setenv("DG_DEFER_REDUCTIONS", mode)
    m = gpu.DeviceMatrix(crs, gpu.DG_STORE_LOWER_DIAG_LAST, gpu.DG_VALUES_BOTH)
    v, info = gpu.ground_state(m, gpu.default_params(mixed=mixed), guess=guess)
    return info.eig_val, np.array(v), info.lanczos_steps, info.cg_steps


@pytest.mark.parametrize("mixed", [0, 2])
def test_deferred_lanczos_bitwise(gpu, monkeypatch, mixed):
    g = golden("sml_random1500.npz")
    low = abi.Crs(g["low_row"], g["low_col"], g["low_val"])
    e0, v0, l0, c0 = _solve(gpu, low, mixed, g["guess"], monkeypatch, "0")
    e1, v1, l1, c1 = _solve(gpu, low, mixed, g["guess"], monkeypatch, "1")
    assert (l0, c0) == (l1, c1)
    if mixed == 0:
        assert e0 == e1
        assert np.array_equal(v0, v1)
    else:
        assert abs(e0 - e1) <= 1e-13 * abs(e0)
        assert abs(v0 @ v1) >= 1 - 1e-12


def test_deferred_superblock_bitwise(gpu, monkeypatch):
    """The same on a superblock Hamiltonian (the benchmark's kind of matrix, several cycles of
    partials per consumer block)."""
    from dmrg_c_gb300 import workloads
    low = workloads.xxz_superblock_m64(0).explicit_lower()
    e0, v0, l0, c0 = _solve(gpu, low, 0, None, monkeypatch, "0")
    e1, v1, l1, c1 = _solve(gpu, low, 0, None, monkeypatch, "1")
    assert (l0, c0) == (l1, c1) and e0 == e1 and np.array_equal(v0, v1)


@pytest.mark.parametrize("n", [1, 2, 5, 33, 257, 2100])
@pytest.mark.parametrize("ws", [1, 4])
def test_deferred_small_systems(gpu, monkeypatch, n, ws):
    """Edge sizes for the consumer form: fewer partials than threads, one slice, the 1 x 1
    operator, several warps per slice; energies against numpy."""
    import scipy.sparse as sp
    rng = np.random.default_rng(n)
    A = sp.random(n, n, density=min(1.0, 6.0 / n), random_state=n)
    A = (A + A.T).tocsr()
    A.setdiag(rng.standard_normal(n) - 3.0)
    A.sort_indices()
    low = abi.lower_diag_last(A)
    exact = np.linalg.eigvalsh(A.toarray())[0]
    out = []
    for mode in ("0", "1"):
        monkeypatch.setenv("DG_DEFER_REDUCTIONS", mode)
        m = gpu.DeviceMatrix(low, gpu.DG_STORE_LOWER_DIAG_LAST)
        m.set_sell_shape(ws, 3)
        v, info = gpu.ground_state(m, gpu.default_params())
        out.append((info.eig_val, np.array(v), info.lanczos_steps, info.cg_steps))
    assert out[0][0] == out[1][0] and np.array_equal(out[0][1], out[1][1]) and out[0][2:] == out[1][2:]
    assert abs(out[0][0] - exact) <= 1e-10 * max(1.0, abs(exact))
