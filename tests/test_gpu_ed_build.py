"""ED basis enumeration and Hamiltonian assembly on the device (dg_ed_*), bit-exact against
the reference's FIND_DIM / GET_BASIS / GET_HAM (golden fixture) and the oracle restatement."""
import numpy as np
import pytest

from conftest import golden, klm_model_from_golden
from dmrg_c_gb300 import ed_models


def _models():
    return [
        ed_models.xxz_chain(10, Jz=1.0),
        ed_models.xxz_chain(12, Jz=0.37, hz=0.61, twoSz=2),
        ed_models.xxz_chain(11, Jz=1.3, Jxy=0.8, hz=0.2, twoSz=-1, bc="PBC"),
        ed_models.hubbard_chain(6, t=-1.0, U=4.0, hz=0.3),
        ed_models.hubbard_chain(7, t=-1.0, U=2.5, hz=0.17, mu=0.4, n_ele=5, twoSz=1, bc="PBC"),
        ed_models.hubbard_chain(8, t=-1.0, U=7.9, hz=0.49),
    ]


def _same(a, b):
    basis, row, col, val = a
    b2, r2, c2, v2 = b
    assert np.array_equal(basis, b2)
    assert np.array_equal(row, r2)
    assert np.array_equal(col, c2)
    assert np.array_equal(val.view(np.int64), v2.view(np.int64))


def test_ed_dim_host_matches_oracle(lib, oracle):
    """dg_ed_dim counts the sector on the host (no device needed)."""
    from dmrg_c_gb300 import lib as L
    for m in _models() + [ed_models.xxz_chain(22), ed_models.hubbard_chain(12)]:
        assert L.ed_dim(m) == oracle.load().or_ed_dim(__import__("ctypes").byref(m.struct), 4), m.name


def test_ed_dim_rejects_bad_models(lib):
    from dmrg_c_gb300 import lib as L
    with pytest.raises(L.DgError):
        L.ed_dim(ed_models.xxz_chain(70))                     # 2^70 codes do not fit int64
    bad = ed_models.xxz_chain(6)
    bad.struct.terms[0].op1 = 99                              # operator index out of range
    with pytest.raises(L.DgError):
        L.ed_dim(bad)


@pytest.mark.gpu
@pytest.mark.parametrize("tag", ["obc", "pbc"])
def test_ed_build_bit_exact_vs_reference_golden(gpu, tag):
    g = golden("klm_ed.npz")
    ed = gpu.EDSystem(klm_model_from_golden(g, tag))
    _same(ed.download(), (g[f"{tag}_basis"], g[f"{tag}_row"], g[f"{tag}_col"], g[f"{tag}_val"]))


@pytest.mark.gpu
def test_ed_build_bit_exact_vs_oracle(gpu, oracle):
    for m in _models():
        ed = gpu.EDSystem(m)
        _same(ed.download(), oracle.ed_build(m))


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["xxz22", "hubbard12"])
def test_ed_build_full_size_bit_exact(gpu, oracle, which):
    """The largest batched-XXZ chain (n = 705,432) and served-Hubbard chain (n = 853,776)."""
    m = ed_models.xxz_chain(22, Jz=1.37, hz=0.42) if which == "xxz22" else ed_models.hubbard_chain(12, U=5.3, hz=0.21)
    ed = gpu.EDSystem(m)
    assert ed.dim == (705432 if which == "xxz22" else 853776)
    _same(ed.download(), oracle.ed_build(m))


@pytest.mark.gpu
def test_ed_empty_sector_is_an_error(gpu):
    with pytest.raises(gpu.DgError):
        gpu.EDSystem(ed_models.xxz_chain(6, twoSz=1))         # odd 2Sz on an even chain


@pytest.mark.gpu
def test_ed_device_matrix_solves_free_fermions(gpu):
    """U = 0 Hubbard on the device-built operator: the ground state is the filled Fermi sea."""
    L = 10
    ed = gpu.EDSystem(ed_models.hubbard_chain(L, t=-1.0, U=0.0))
    m = ed.matrix()
    v, info = gpu.ground_state(m, gpu.default_params(seed=3))
    E0 = ed_models.free_fermion_energy(L, L // 2, L // 2)
    assert abs(info.eig_val - E0) <= 1e-10 * abs(E0)
