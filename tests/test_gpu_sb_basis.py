"""GPU superblock basis (dg_sb_basis: GET_BASIS_SUPERBLOCK with DMRG_QUICK_SORT_BASIS_Q1/_Q2 order)
against the reference-made fixture and the oracle, and the superblock CRS built from it."""
import numpy as np
import pytest

from conftest import golden
from dmrg_c_gb300 import superblock, workloads

pytestmark = pytest.mark.gpu


def _same(a, b):
    for x, y in zip(a, b):
        x, y = np.asarray(x), np.asarray(y)
        assert x.shape == y.shape
        assert np.array_equal(x.view(np.int64) if x.dtype == np.float64 else x, y.view(np.int64) if y.dtype == np.float64 else y)


def test_sb_basis_q1_vs_reference_golden(gpu):
    g = golden("sb_basis.npz")
    b = gpu.SuperblockBasis(40, 36, 2, g["q1_LL"], g["q1_RR"], g["q1_site"], int(g["q1_target"]))
    LL, LR, RR, RL, inv = b.download()
    assert np.array_equal(np.stack([LL, LR, RR, RL]), g["q1_states"])
    assert np.array_equal(inv, g["q1_inv"])


def test_sb_basis_q2_vs_reference_golden(gpu):
    g = golden("sb_basis.npz")
    t = g["q2_targets"]
    b = gpu.SuperblockBasis(48, 44, 4, g["q2_ne_LL"], g["q2_ne_RR"], g["q2_ne_site"], int(t[0]), g["q2_sz_LL"],
                            g["q2_sz_RR"], g["q2_sz_site"], int(t[1]))
    LL, LR, RR, RL, inv = b.download()
    assert np.array_equal(np.stack([LL, LR, RR, RL]), g["q2_states"])
    assert np.array_equal(inv, g["q2_inv"])


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_sb_basis_random_vs_oracle(gpu, oracle, seed):
    rng = np.random.default_rng(seed)
    dLL, dRR, d = int(rng.integers(1, 90)), int(rng.integers(1, 90)), int(rng.choice([2, 3, 4, 8]))
    q1 = (rng.integers(-4, 5, dLL), rng.integers(-4, 5, dRR), rng.integers(-1, 2, d))
    q2 = (rng.integers(0, 6, dLL), rng.integers(0, 6, dRR), rng.integers(0, 3, d))
    want = oracle.sb_basis(dLL, dRR, d, q1, q2, (0, 5))
    if len(want[0]) == 0:
        pytest.skip("empty sector for this draw")
    b = gpu.SuperblockBasis(dLL, dRR, d, *q1, 0, *q2, 5)
    _same(b.download(), want)


def test_sb_basis_m512_and_crs_from_it(gpu):
    """The Hubbard m=512 superblock (packed (N_e, 2Sz) quantum numbers): the device basis equals the
    host restatement's, and the CRS built on it equals the CRS built from host arrays."""
    qb = workloads._block_labels(512, 31, 31.0, 1.25, 0.9, 0)
    site = workloads.hubbard_site_labels()
    b = gpu.SuperblockBasis(512, 512, 4, qb, qb, site, 64 * workloads.QN_SCALE)
    model = workloads.hubbard_sb_model_m512(0)
    assert b.n == model.n == 227652
    _same(b.download(), (model.LL, model.LR, model.RR, model.RL, model.inv))
    _same(gpu.SuperblockCRS(model, basis=b).download(), gpu.SuperblockCRS(model).download())


def test_sb_basis_rejects_bad_specs(gpu):
    with pytest.raises(gpu.DgError):            # empty sector
        gpu.SuperblockBasis(4, 4, 2, [0, 0, 0, 0], [0, 0, 0, 0], [1, -1], 99)
    with pytest.raises(gpu.DgError):            # dimension beyond a short
        gpu.SuperblockBasis(40000, 2, 2, np.zeros(40000), [0, 0], [1, -1], 0)
    b = gpu.SuperblockBasis(4, 4, 2, [0, 0, 2, 2], [0, 0, -2, -2], [1, -1], 0)
    model = workloads.hubbard_sb_model_m512(0)
    with pytest.raises(gpu.DgError):            # model dimensions differ from the basis'
        gpu.SuperblockCRS(model, basis=b)
