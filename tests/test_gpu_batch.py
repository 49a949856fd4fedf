"""The batched form: dg_batch_ground_state (the Lanczos phases of many ED instances in lock-step,
one launch of each kernel per step over all of them) against the one-at-a-time dg_ground_state on
the same matrices, FP64 and mixed (mixed = 2), with instances of uneven size, one below the dense
threshold (in FP64 solved by the single path's dense route; the mixed form batches it too), and the
FP64 energies against the oracle."""
import numpy as np
import pytest

from dmrg_c_gb300 import abi, ed_models

pytestmark = pytest.mark.gpu


def _instances(gpu):
    specs = [(12, 0.7, 0.1), (14, 1.3, 0.4), (14, 0.2, 0.9), (16, 1.0, 0.0), (18, 1.9, 0.3), (20, 0.5, 0.6), (16, 1.4, 0.8)]
    out = []
    for L, Jz, hz in specs:
        model = ed_models.xxz_chain(L, Jxy=1.0, Jz=Jz, hz=hz)
        ed = gpu.EDSystem(model)
        out.append((model, ed, ed.matrix(gpu.DG_VALUES_BOTH)))
    return out


@pytest.mark.parametrize("mixed", [0, 2], ids=["fp64", "mixed2"])
def test_batch_matches_single_solves(gpu, mixed):
    inst = _instances(gpu)
    mats = [m for _, _, m in inst]
    p = gpu.default_params(seed=7, mixed=mixed)
    vecs, infos = gpu.batch_ground_state(mats, p)
    for (model, ed, m), v, info in zip(inst, vecs, infos):
        assert info.converged
        v1, i1 = gpu.ground_state(m, gpu.default_params(seed=7, mixed=0))
        tol = 1e-12 if mixed == 0 else 1e-10
        assert abs(info.eig_val - i1.eig_val) <= tol * abs(i1.eig_val), (m.n, info.eig_val, i1.eig_val)
        assert abs(v @ v1) >= 1 - 1e-9, (m.n, abs(v @ v1))
        assert abs(np.linalg.norm(v) - 1) < 1e-12


def test_batch_fp64_energies_match_oracle(gpu, oracle):
    inst = _instances(gpu)[:4]
    vecs, infos = gpu.batch_ground_state([m for _, _, m in inst], gpu.default_params(seed=3))
    for (model, ed, m), info in zip(inst, infos):
        basis, row, col, val = ed.download()
        rc, out, v = oracle.lanczos(abi.Crs(row, col, val), False, seed=3)
        assert abs(info.eig_val - out.eig_val) <= 1e-12 * abs(out.eig_val)


def test_batch_repeated_and_empty(gpu):
    """Two batches in a row on the same matrices give the same energies; an empty batch is a no-op."""
    inst = _instances(gpu)[0:4]        # the first is below the dense threshold (batched in the mixed form)
    mats = [m for _, _, m in inst]
    _, a = gpu.batch_ground_state(mats, gpu.default_params(seed=5, mixed=2), want_vectors=False)
    _, b = gpu.batch_ground_state(mats, gpu.default_params(seed=5, mixed=2), want_vectors=False)
    assert [x.eig_val for x in a] == [x.eig_val for x in b]
    assert gpu.batch_ground_state([], gpu.default_params()) == ([], [])
