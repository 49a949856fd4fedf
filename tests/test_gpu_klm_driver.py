"""Drop-ins for the KLM ED driver (FIND_DIM / GET_BASIS / GET_HAM): the driver's own outputs,
bit for bit, from the model struct alone (site operators restated, basis and CRS built on the
device), against the reference's outputs stored in klm_ed.npz."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden, klm_driver_model
from dmrg_c_gb300 import abi


@pytest.mark.parametrize("tag", ["obc", "pbc"])
def test_find_dim_matches_reference(lib, tag):
    """FIND_DIM counts the sector on the host: no device needed."""
    g = golden("klm_ed.npz")
    tm = abi.EXACT_TIME()
    dim = lib.FIND_DIM(C.byref(klm_driver_model(g, tag)), C.byref(tm))
    assert dim == len(g[f"{tag}_basis"])
    assert tm.find_dim >= 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("tag", ["obc", "pbc"])
def test_get_basis_and_get_ham_bit_exact(gpu, tag):
    g = golden("klm_ed.npz")
    L = gpu.load()
    model = klm_driver_model(g, tag)
    tm = abi.EXACT_TIME()
    dim = L.FIND_DIM(C.byref(model), C.byref(tm))
    bp = L.GET_BASIS(C.byref(model), C.byref(tm), dim)
    basis = np.ctypeslib.as_array(bp, shape=(dim,)).copy()
    assert np.array_equal(basis, g[f"{tag}_basis"])
    info = abi.EXACT_BASIS_INFO()
    info.dim = dim
    info.Basis = bp
    par = abi.EXACT_PARAMETER()
    par.est_max_row_elem_num = 1000
    H = L.GET_HAM(C.byref(model), C.byref(info), C.byref(par), C.byref(tm)).contents
    nnz = H.Row[dim]
    row = np.ctypeslib.as_array(H.Row, shape=(dim + 1,)).copy()
    col = np.ctypeslib.as_array(H.Col, shape=(nnz,)).copy()
    val = np.ctypeslib.as_array(H.Val, shape=(nnz,)).copy()
    assert H.row_dim == dim and H.col_dim == dim
    assert np.array_equal(row, g[f"{tag}_row"])
    assert np.array_equal(col, g[f"{tag}_col"])
    assert np.array_equal(val.view(np.int64), g[f"{tag}_val"].view(np.int64))
    assert tm.make_basis > 0 and tm.make_ham > 0
