"""EXACT_V_M_Q1 and EXACT_V_M_Q3 through the C-ABI, bitwise against the reference's own functions
(golden vm_q13.npz; exact/EXACT_V_M_Q1.c:8-38, exact/EXACT_V_M_Q3.c:10-60): a spin-1/2 chain whose
whole basis is split by the number of up spins (Q1) and a Hubbard chain split by (N_up, N_down, 0)
(Q3, with and without the fermion sign string)."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden, vm_whole_sectors
from dmrg_c_gb300 import abi

pytestmark = pytest.mark.gpu


def test_exact_v_m_q1_golden(gpu):
    lib = gpu.load()
    g = golden("vm_q13.npz")
    q1, s1, _, _ = vm_whole_sectors()
    W = abi.ExactWholeBasis(q1, s1)
    raise_op = abi.Crs(np.array([0, 0, 1]), np.array([0], np.int32), np.array([1.5]), n=2)
    diag_op = abi.Crs(np.array([0, 1, 2]), np.array([0, 1], np.int32), np.array([-0.5, 0.75]), n=2)
    for site in (0, 3, 7):
        for op, qin, v, key in ((raise_op, 3, g["q1_v3"], "raise"), (diag_op, 4, g["q1_v4"], "diag")):
            vec = np.ascontiguousarray(v)
            out = np.full(len(q1[(4,)]), np.nan)
            lib.EXACT_V_M_Q1(op.ref, 4, abi.ptr(vec, C.c_double), qin, abi.ptr(out, C.c_double), 2, site, 1, W.ref)
            np.testing.assert_array_equal(out, g[f"q1_{key}_site{site}"])


def test_exact_v_m_q3_golden(gpu):
    lib = gpu.load()
    g = golden("vm_q13.npz")
    _, _, q3, s3 = vm_whole_sectors()
    W = abi.ExactWholeBasis(q3, s3)
    op = abi.Crs(g["q3_op_row"], g["q3_op_col"], g["q3_op_val"], n=4)
    vec = np.ascontiguousarray(g["q3_v"])
    n_ele = np.array([0, 1, 1, 2], np.int32)
    for site in (0, 2, 3):
        for sign in (0, 1):
            out = np.full(len(q3[(2, 1, 0)]), np.nan)
            lib.EXACT_V_M_Q3(op.ref, 2, 1, 0, abi.ptr(vec, C.c_double), 1, 1, 0, abi.ptr(out, C.c_double),
                             b"Yes" if sign else b"No", abi.ptr(n_ele, C.c_int), 4, site, 1, W.ref)
            np.testing.assert_array_equal(out, g[f"q3_site{site}_sign{sign}"])
