"""Edge cases of the observable, density-matrix and renormalisation entry points on the GPU: empty
sectors, zero-state pairs, minimal site counts, zero operators."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import golden
from dmrg_c_gb300 import abi, sb_models

pytestmark = pytest.mark.gpu


def _problem():
    g = golden("sb_obs.npz")
    return sb_models.ObservableProblem.from_arrays(g), g


def _free():
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    return libc.free


def test_vm_whole_basis_empty_output_sector(gpu, oracle):
    """An output sector of dimension 0: nothing is read or written (the reference's loop is empty)."""
    p, g = _problem()
    sectors = dict(((q,), st) for q, st in ((int(np.searchsorted(p.labels, t)), s) for t, s in p.sectors.items()))
    empty = len(p.labels)                                    # an index past every label: Dim = 0
    wb = abi.WholeBasis(sectors, (len(p.labels) + 1,), p.inv, p.dim_RR, p.d)
    out = oracle.call_vm_whole(gpu.load(), wb, (empty,), p.ops["CdRR"][0], 2, g["v"], ele=p.ele, sign=True)
    assert out.shape == (0,)


def test_expectation_onsite_minimal_sites(gpu, oracle):
    """LL_site = RR_site = 0: one block operator on each side plus the two site terms."""
    p, g = _problem()
    st, inv0 = p.sectors[p.target], p.inv_sector(p.target)
    v = g["v"]
    out, temp = oracle.call_expectation_onsite(gpu.load(), st, inv0, p.dim_LL, p.dim_RR, p.d, p.ops["LL"][:1], p.ops["On"],
                                               p.ops["RR"][:1], v)
    want = [v @ oracle.sb_vm(st, inv0, p.dim_RR, p.d, op, pos, v)
            for op, pos in ((p.ops["LL"][0], 0), (p.ops["On"], 1), (p.ops["On"], 3), (p.ops["RR"][0], 2))]
    assert np.allclose(out, want, rtol=0, atol=1e-12 * float(v @ v) * 10)
    assert np.array_equal(temp, oracle.sb_vm(st, inv0, p.dim_RR, p.d, p.ops["RR"][0], 2, v))


def test_density_matrix_zero_state_pairs(gpu, oracle):
    """LLLR pairs whose label has no complement in the sector: zero blocks, as the reference gives."""
    p, g = _problem()
    st, inv0 = p.sectors[p.target], p.inv_sector(p.target)
    lllr = oracle.lllr_list(p.q_LL, p.q_site, st)
    starts = np.concatenate([[0], np.cumsum(lllr[4])])
    zero_blocks = [b for b in range(len(lllr[4])) if lllr[2][starts[b]] == 0]
    assert zero_blocks, "the fixture has no zero-state block"
    blocks = oracle.call_density_matrix(gpu.load(), st, inv0, p.dim_LL, p.dim_RR, p.d, g["v"], lllr, _free())
    for b in zero_blocks:
        assert not blocks[b].any()


def test_renorm_zero_operator_and_single_column(gpu, oracle):
    """A zero operator keeps nothing; a one-column T keeps what the oracle keeps."""
    rng = np.random.default_rng(2)
    r3, c3 = 30, 1
    T = sp.csc_matrix(rng.standard_normal((r3, c3)))
    M1, M3 = abi.Crs.from_scipy(sp.csr_matrix(T.T)), abi.Ccs.from_scipy(T)
    zero = abi.Crs(np.zeros(r3 + 1, np.int64), np.zeros(0, np.int32), np.zeros(0), n=r3, ncol=r3)
    r = oracle.call_crs_crs_ccs(gpu.load(), M1, zero, M3, r3 * c3, c3 * c3)
    assert int(r[0][-1]) == 0 and int(r[3][-1]) == 0
    O = abi.Crs.from_scipy(sp.csr_matrix(rng.standard_normal((r3, r3))))
    r = oracle.call_crs_crs_ccs(gpu.load(), M1, O, M3, r3 * c3, c3 * c3)
    want = oracle.crs_crs_ccs(M1, O, M3)
    for x, y in zip(r[:6], want):
        assert np.array_equal(np.asarray(x, np.float64), np.asarray(y, np.float64))
