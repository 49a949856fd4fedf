"""Mixed-precision form: FP32 operator values and Krylov vectors with compensated FP32
accumulation, FP64 recurrence / reorthogonalisation / refinement.  Energies against the FP64
oracle at |dE|/|E| <= 1e-10 and overlaps >= 1 - 1e-9; the pre-refinement Ritz value is stated."""
import numpy as np
import pytest
import scipy.sparse as sp

from dmrg_c_gb300 import abi, ed_models, superblock, workloads

TOL_E = 1e-10
TOL_OV = 1e-9


def _mixed_params(gpu, mixed=1, **kw):
    return gpu.default_params(mixed=mixed, seed=5, **kw)


@pytest.mark.gpu
def test_mixed_spmv_is_compensated(gpu):
    """The FP32-value product equals H32 x32 evaluated in FP64 to ~1e-13 (a plain FP32 sum
    of ~65 terms would be off by ~1e-6)."""
    sb = workloads.klm_superblock_m128(0)
    low = sb.explicit_lower()
    m = gpu.DeviceMatrix(low, gpu.DG_STORE_LOWER_DIAG_LAST, gpu.DG_VALUES_BOTH)
    row, col, val = m.download()
    H32 = sp.csr_matrix((val.astype(np.float32).astype(np.float64), col, row), shape=(m.n, m.n))
    x = np.random.default_rng(3).standard_normal(m.n).astype(np.float32)
    ref = H32 @ x.astype(np.float64)
    y = m.spmv_mixed(x)
    err = np.max(np.abs(y - ref)) / np.max(np.abs(ref))
    assert err < 1e-13, err


def _check_solve(gpu, oracle, crs, storage, E_ref=None, mixed=1, **kw):
    m = gpu.DeviceMatrix(crs, storage, gpu.DG_VALUES_BOTH)
    v, info = gpu.ground_state(m, _mixed_params(gpu, mixed, **kw))
    assert info.converged
    if E_ref is None:
        rc, out, v_ref = oracle.lanczos(crs, storage == gpu.DG_STORE_LOWER_DIAG_LAST, seed=5)
        rc2, oi, v_ref = oracle.inverse_iteration(crs, storage == gpu.DG_STORE_LOWER_DIAG_LAST, out.eig_val, v_ref)
        E_ref = out.eig_val
    else:
        v_ref = None
    dE = abs(info.eig_val - E_ref) / abs(E_ref)
    assert dE <= TOL_E, (info.eig_val, E_ref, dE)
    assert abs(info.eig_lanczos - E_ref) / abs(E_ref) < 1e-5      # FP32-level before refinement
    if v_ref is not None:
        assert abs(v @ v_ref) >= 1 - TOL_OV
    return info


@pytest.mark.gpu
def test_mixed_superblock_matches_fp64_oracle(gpu, oracle):
    low = workloads.xxz_superblock_m64(0).explicit_lower()
    _check_solve(gpu, oracle, low, gpu.DG_STORE_LOWER_DIAG_LAST)


@pytest.mark.gpu
def test_mixed_klm_superblock_matches_fp64_oracle(gpu, oracle):
    low = workloads.klm_superblock_m128(0).explicit_lower()
    _check_solve(gpu, oracle, low, gpu.DG_STORE_LOWER_DIAG_LAST)


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [1, 2])
def test_mixed_ed_free_fermions(gpu, mixed):
    L = 10
    ed = gpu.EDSystem(ed_models.hubbard_chain(L, t=-1.0, U=0.0))
    b, row, col, val = ed.download()
    crs = abi.Crs(row, col, val, n=ed.dim)
    _check_solve(gpu, None, crs, gpu.DG_STORE_FULL, E_ref=ed_models.free_fermion_energy(L, L // 2, L // 2), mixed=mixed)


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [1, 2])
def test_mixed_ed_matches_fp64_oracle(gpu, oracle, mixed):
    """Interacting Hubbard and XXZ chains: the mixed forms against the FP64 oracle."""
    for model in (ed_models.hubbard_chain(8, U=4.7, hz=0.13), ed_models.xxz_chain(16, Jz=1.3, hz=0.4)):
        basis, row, col, val = oracle.ed_build(model)
        _check_solve(gpu, oracle, abi.Crs(row, col, val, n=len(basis)), gpu.DG_STORE_FULL, mixed=mixed)


@pytest.mark.gpu
def test_mixed_needs_fp32_values(gpu):
    low = workloads.xxz_superblock_m64(0).explicit_lower()
    m = gpu.DeviceMatrix(low, gpu.DG_STORE_LOWER_DIAG_LAST)          # FP64 values only
    with pytest.raises(gpu.DgError):
        gpu.ground_state(m, _mixed_params(gpu))


@pytest.mark.gpu
def test_mixed_below_dense_threshold(gpu):
    """Below dense_below (1000 states) the FP64 form takes the reference's dense route; the mixed
    form runs its own Lanczos and FP64 refinement from 64 states up and still reaches the FP64
    energy; below 64 states it takes the dense route as well."""
    from dmrg_c_gb300 import ed_models
    for L, dense_mixed in ((12, 0), (6, 1)):
        ed = gpu.EDSystem(ed_models.xxz_chain(L, Jxy=1.0, Jz=0.8, hz=0.2))
        m = ed.matrix(gpu.DG_VALUES_BOTH)
        v0, i0 = gpu.ground_state(m, gpu.default_params(seed=4))
        v2, i2 = gpu.ground_state(m, gpu.default_params(seed=4, mixed=2))
        assert i0.dense == 1 and i2.dense == dense_mixed, (m.n, i0.dense, i2.dense)
        assert abs(i2.eig_val - i0.eig_val) <= 1e-10 * abs(i0.eig_val), (m.n, i2.eig_val, i0.eig_val)
        assert abs(v0 @ v2) >= 1 - 1e-9
