"""The recorded superblocks of the reference's DMRG runs (tests/golden/dmrg_<model>_sweep<k>.npz)
checked on the CPU: the term list rebuilt by the oracle (and, where the reference tree is present,
by the reference's own DMRG_MAKE_ELEM_*_LLLRRRRL builders) gives the reference's GET_HAM_LLLRRRRL
CRS bit for bit (dg64 checksums), and the oracle's solve reaches the reference's gs_val on the small
superblocks.  Also the per-step energy log of each run."""
import numpy as np
import pytest

from conftest import GOLDEN
from dmrg_c_gb300 import abi, sb_models

FIXTURES = sorted(GOLDEN.glob("dmrg_*_sweep*.npz"))
IDS = [p.stem.replace("dmrg_", "") for p in FIXTURES]


def test_fixtures_cover_every_configuration():
    names = {p.stem for p in FIXTURES}
    for model, sweeps in (("xxz_vf", range(1, 5)), ("klm_vf", range(1, 5)), ("hubbard_vf", (4,))):
        for k in sweeps:
            assert f"dmrg_{model}_sweep{k}" in names


@pytest.mark.parametrize("path", FIXTURES, ids=IDS)
def test_oracle_build_is_the_references(oracle, path):
    sb = sb_models.load_dmrg_superblock(path)
    row, col, val = oracle.sb_build(sb.model)
    assert row[-1] == sb.nnz
    assert (oracle.dg64(row), oracle.dg64(col), oracle.dg64(val)) == sb.crs_dg64


@pytest.mark.parametrize("path", [p for p in FIXTURES if "hubbard" not in p.name],
                         ids=[i for i in IDS if "hubbard" not in i])
def test_reference_builders_on_the_recorded_terms(ref, path):
    """The reference's own element builders, driven over the recorded term list, reproduce the
    reference run's CRS: the term list is the model's MAKE_ELEMENT_HAM_LLLRRRRL."""
    sb = sb_models.load_dmrg_superblock(path)
    row, col, val = ref.ref_sb_build(sb.model, cap=sb.nnz + 1)
    assert (ref.dg64(row), ref.dg64(col), ref.dg64(val)) == sb.crs_dg64


@pytest.mark.parametrize("path", [p for p in FIXTURES if "xxz" in p.name], ids=[i for i in IDS if "xxz" in i])
def test_oracle_solve_reaches_reference_energy(oracle, path):
    sb = sb_models.load_dmrg_superblock(path)
    row, col, val = oracle.sb_build(sb.model)
    H = abi.Crs(row, col, val, n=sb.model.n)
    rc, out, v = oracle.lanczos(H, True, seed=3, threads=1)
    rc, oi, v = oracle.inverse_iteration(H, True, out.eig_val, v, cg_acc=1e-6, threads=1)
    assert abs(out.eig_val - sb.gs_val) <= 1e-12 * abs(sb.gs_val)
    assert abs(v @ sb.gs_vec) / (np.linalg.norm(v) * np.linalg.norm(sb.gs_vec)) >= 1 - 1e-9


def test_step_logs():
    """Every superblock solve of the runs: the final energies of the configurations."""
    final = {}
    for model, L in (("xxz_vf", 32), ("klm_vf", 24), ("hubbard_vf", 64)):
        p = GOLDEN / f"dmrg_{model}_steps.npz"
        z = np.load(p)
        assert np.all(np.diff(z["sweep"]) >= 0)
        final[model] = float(z["gs_val"][-1]) / L
        # the recorded sweeps are the largest superblock of their sweep
        for f in sorted(GOLDEN.glob(f"dmrg_{model}_sweep*.npz")):
            s = np.load(f)
            k = int(s["sweep"])
            assert int(s["n"]) == int(z["n"][z["sweep"] == k].max())
    assert final["xxz_vf"] * 32 == pytest.approx(-13.997315618003377, abs=1e-9)
    assert final["klm_vf"] == pytest.approx(-0.983041859235136, abs=1e-9)
    assert final["hubbard_vf"] == pytest.approx(-0.567997385721411, abs=1e-9)
