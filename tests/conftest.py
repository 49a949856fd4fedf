import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the CUDA library")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.load()
    return pyoracle


@pytest.fixture(scope="session")
def ref(oracle):
    """The reference build (oracle/_ref); skipped where the reference tree is absent."""
    if not oracle.ref_available():
        pytest.skip("reference sources not present")
    oracle.load_ref()
    return oracle


@pytest.fixture(scope="session")
def lib():
    from dmrg_c_gb300 import build, lib as L
    build.build()
    return L.load()


@pytest.fixture(scope="session")
def gpu(lib):
    """The CUDA library on a visible device.  On a GPU run this must not skip: a missing
    device or library is an error."""
    from dmrg_c_gb300 import lib as L
    n = L.device_count()
    assert n > 0, "gpu test collected but no CUDA device is visible"
    return L


@pytest.fixture
def in_tmp(tmp_path, monkeypatch):
    """Run in a scratch directory (the drop-in entry points append to ./SML_out/)."""
    monkeypatch.chdir(tmp_path)
    return tmp_path


def golden(name):
    return np.load(GOLDEN / name)


def renorm_operands_from_golden(g):
    """(M1, M2, M3) of the renormalisation fixture: T^dagger (CRS), O (CRS), T (CCS)."""
    from dmrg_c_gb300 import abi
    r1, r2, r3, c3 = (int(x) for x in g["dims"])
    M1 = abi.Crs(g["m1_row"], g["m1_col"], g["m1_val"], n=r1, ncol=r2)
    M2 = abi.Crs(g["m2_row"], g["m2_col"], g["m2_val"], n=r2, ncol=r3)
    M3 = abi.Ccs(g["m3_col"], g["m3_row"], g["m3_val"], r3, c3)
    return M1, M2, M3


@pytest.fixture
def rng():
    return np.random.default_rng(1234)


def pytest_collection_modifyitems(config, items):
    os.environ.setdefault("OMP_NUM_THREADS", str(min(8, os.cpu_count() or 1)))


def klm_model_from_golden(g, tag):
    """The KLM chain of a klm_ed.npz fixture as a dg_ed_model (site operators from the
    reference's own onsite_op builders, stored in the fixture)."""
    from dmrg_c_gb300 import ed_models
    L, ne, sz, t, I_z, I_xy = g[f"{tag}_params"]
    tabs = [(g[f"{tag}_op{k}_row"], g[f"{tag}_op{k}_col"], g[f"{tag}_op{k}_val"]) for k in range(9)]
    return ed_models.klm_chain_from_tables(int(L), tabs, int(ne), int(sz), t=float(t), I_z=float(I_z), I_xy=float(I_xy),
                                           bc="PBC" if tag == "pbc" else "OBC")


def klm_driver_model(g, tag):
    """The MODEL_1DKLM_VF of a klm_ed.npz fixture (the reference driver's model struct)."""
    from dmrg_c_gb300 import abi
    L, ne, sz, t, J, D_z, I_xy, I_z, h_z, mu, pbc = g[f"{tag}_model"]
    m = abi.MODEL_1DKLM_VF()
    m.BC = b"PBC" if pbc else b"OBC"
    m.p_threads = 1
    m.spin_loc = 1
    m.tot_site, m.tot_ele, m.tot_sz = int(L), int(ne), int(sz)
    m.dim_charge, m.dim_lspin, m.dim_onsite = 4, 2, 8
    m.t, m.J, m.D_z, m.I_xy, m.I_z, m.h_z, m.mu = t, J, D_z, I_xy, I_z, h_z, mu
    return m


def vm_whole_sectors():
    """The whole bases of vm_q13.npz (as tests/golden/make_golden.py builds them): spin-1/2 L=8 codes
    by number of up spins (Q1 index k), Hubbard L=4 codes (local states empty, up, down, up+down)
    by (N_up, N_down, 0) (Q3)."""
    codes = np.arange(2 ** 8, dtype=np.int64)
    ups = sum((codes >> s) & 1 for s in range(8))
    q1 = {(k,): codes[ups == k] for k in range(9)}
    codes = np.arange(4 ** 4, dtype=np.int64)
    digits = [(codes // 4 ** s) % 4 for s in range(4)]
    nu = sum((dg == 1) | (dg == 3) for dg in digits)
    nd = sum((dg == 2) | (dg == 3) for dg in digits)
    q3 = {(a, b, 0): codes[(nu == a) & (nd == b)] for a in range(5) for b in range(5)}
    return q1, (9,), q3, (5, 5, 1)
