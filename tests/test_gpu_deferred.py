"""Reductions finished by the consuming kernel give bitwise the values of the last-block form.

The Lanczos step can leave <y,v> and <w,w> to the kernels that consume them (every consumer
block sums the producer's block partials in the same fixed order); DG_DEFER_REDUCTIONS=0 / =1
forces either form at the same launch grid, so energies, vectors and step counts must match
bit for bit.  CG and the refinement always use the consumer form; their parity against the
reference is covered by the golden tests.
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
    assert e0 == e1
    assert np.array_equal(v0, v1)


def test_deferred_superblock_bitwise(gpu, monkeypatch):
    """The same on a superblock Hamiltonian (the benchmark's kind of matrix, several cycles of
    partials per consumer block)."""
    from dmrg_c_gb300 import workloads
    low = workloads.xxz_superblock_m64(0).explicit_lower()
    e0, v0, l0, c0 = _solve(gpu, low, 0, None, monkeypatch, "0")
    e1, v1, l1, c1 = _solve(gpu, low, 0, None, monkeypatch, "1")
    assert (l0, c0) == (l1, c1) and e0 == e1 and np.array_equal(v0, v1)
