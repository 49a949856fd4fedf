"""Superblock Hamiltonian CRS built on the device (dg_sb_*): bit-exact against the reference's
element builders (golden fixture) and the oracle, at small and at m=512 size."""
import numpy as np
import pytest

from conftest import golden
from dmrg_c_gb300 import sb_models, workloads


def _same(a, b):
    for x, y in zip(a, b):
        if x.dtype == np.float64:
            assert np.array_equal(x.view(np.int64), y.view(np.int64))
        else:
            assert np.array_equal(x, y)


@pytest.mark.gpu
@pytest.mark.parametrize("tag", ["obc", "pbc"])
def test_sb_build_bit_exact_vs_reference_golden(gpu, tag):
    g = golden("sb_hubbard.npz")
    s = gpu.SuperblockCRS(sb_models.small_hubbard_model(tag == "pbc"))
    _same(s.download(), (g[f"{tag}_row"], g[f"{tag}_col"], g[f"{tag}_val"]))


@pytest.mark.gpu
def test_sb_build_m512_bit_exact_vs_oracle(gpu, oracle):
    m = workloads.hubbard_sb_model_m512(0)
    s = gpu.SuperblockCRS(m)
    assert s.n == 227652
    _same(s.download(), oracle.sb_build(m))


@pytest.mark.gpu
def test_sb_matrix_ground_state_matches_oracle(gpu, oracle):
    """The device-built superblock feeds the solvers directly (lower -> full on the device)."""
    from dmrg_c_gb300 import abi
    m = sb_models.small_hubbard_model(True)
    s = gpu.SuperblockCRS(m)
    mat = s.matrix()
    v, info = gpu.ground_state(mat, gpu.default_params(seed=4))
    row, col, val = oracle.sb_build(m)
    rc, out, vr = oracle.lanczos(abi.Crs(row, col, val, n=m.n), True, seed=4)
    assert abs(info.eig_val - out.eig_val) <= 1e-12 * abs(out.eig_val)


@pytest.mark.gpu
def test_sb_build_rejects_malformed_models(gpu):
    """Bad positions, operator indices, signs without electron tables and out-of-range basis
    states are refused on the host, before any kernel runs."""
    from dmrg_c_gb300.sb_models import SBModel

    def variant(**change):
        m = sb_models.small_hubbard_model(False)
        terms = [list(t) for t in m.terms]
        ele = list(m.ele)
        LLv = m.LL.copy()
        if "pos" in change:
            terms[4][0] = change["pos"]
        if "op" in change:
            terms[4][2] = change["op"]
        if "noele" in change:
            ele[0] = None
        if "state" in change:
            LLv[3] = change["state"]
        return SBModel(m.n, m.dim_LL, m.dim_RR, m.d, LLv, m.LR, m.RR, m.RL, m.inv, m.ops, [tuple(t) for t in terms], ele)

    for bad in (dict(pos=7), dict(op=999), dict(noele=True), dict(state=40)):
        with pytest.raises(gpu.DgError):
            gpu.SuperblockCRS(variant(**bad))
