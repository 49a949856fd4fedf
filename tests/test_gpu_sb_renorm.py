"""Operator renormalisation on the GPU (CRS_CRS_CCS_PRODUCT, Out = T^dagger (O T)) against the
reference-made fixture and the oracle: the intermediate CCS and the result CRS bit for bit, the work
vector left zero, and the reference's capacity error."""
import subprocess
import sys
import textwrap

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import ROOT, golden, renorm_operands_from_golden
from dmrg_c_gb300 import abi

pytestmark = pytest.mark.gpu

NAMES = ("w_col", "w_row", "w_val", "o_row", "o_col", "o_val")


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype == np.float64 or b.dtype == np.float64:
        return a.shape == b.shape and np.array_equal(a.astype(np.float64).view(np.int64), b.astype(np.float64).view(np.int64))
    return a.shape == b.shape and np.array_equal(a.astype(np.int64), b.astype(np.int64))


def test_renorm_dropin_vs_reference_golden(gpu, oracle):
    g = golden("renorm.npz")
    M1, M2, M3 = renorm_operands_from_golden(g)
    r = oracle.call_crs_crs_ccs(gpu.load(), M1, M2, M3, 60 * 24, 24 * 24)
    for a, name in zip(r[:6], NAMES):
        assert _same(a, g[name]), name
    assert not np.isnan(r[6]).any() and not r[6].any()          # work vector cleared, as the reference leaves it
    assert tuple(r[7]) == tuple(g["shape"])


def _truncation_like(seed, r3, c3, per_row, nblk):
    rng = np.random.default_rng(seed)
    blocks = np.sort(rng.integers(0, nblk, r3))
    T = np.zeros((r3, c3))
    for j in range(c3):
        rows = np.flatnonzero(blocks == j % nblk)
        T[rows, j] = rng.standard_normal(len(rows))
    # an operator that conserves the blocks, as the renormalised block operators do
    O = np.zeros((r3, r3))
    for b in range(nblk):
        idx = np.flatnonzero(blocks == b)
        k = min(per_row, len(idx))
        for i in idx:
            O[i, rng.choice(idx, size=k, replace=False)] = rng.standard_normal(k)
    return (abi.Crs.from_scipy(sp.csr_matrix(T.T)), abi.Crs.from_scipy(sp.csr_matrix(O)), abi.Ccs.from_scipy(sp.csc_matrix(T)))


@pytest.mark.parametrize("seed,r3,c3", [(1, 512, 128), (2, 1000, 257)])
def test_renorm_dropin_vs_oracle(gpu, oracle, seed, r3, c3):
    M1, M2, M3 = _truncation_like(seed, r3, c3, 12, 9)
    want = oracle.crs_crs_ccs(M1, M2, M3)
    got = oracle.call_crs_crs_ccs(gpu.load(), M1, M2, M3, r3 * c3, c3 * c3)
    for a, b, name in zip(got[:6], want, NAMES):
        assert _same(a, b), name


def test_renorm_capacity_error_matches_reference(gpu, tmp_path):
    """An Out too small for the result: the reference's message and exit status 1."""
    code = textwrap.dedent(f"""
        import sys
        sys.path.insert(0, {str(ROOT)!r}); sys.path.insert(0, {str(ROOT / 'oracle')!r}); sys.path.insert(0, {str(ROOT / 'tests')!r})
        import pyoracle
        from conftest import golden, renorm_operands_from_golden
        from dmrg_c_gb300 import lib
        M1, M2, M3 = renorm_operands_from_golden(golden("renorm.npz"))
        pyoracle.call_crs_crs_ccs(lib.load(), M1, M2, M3, 60 * 24, 10)
        print("returned")
    """)
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=tmp_path, timeout=300)
    assert p.returncode == 1, p.stdout + p.stderr
    assert "error in CRS_CRS_CCS_PRODUCT" in p.stdout and "Need more Out->max_val = 10" in p.stdout
    assert "returned" not in p.stdout
