"""GPU parity of the matrix-free OBC superblock path and the ED operator application
(reference names through the C-ABI) against the reference's golden outputs and the oracle."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden
from dmrg_c_gb300 import abi, ed_models, superblock

pytestmark = pytest.mark.gpu


def obc_case(seed=42, with_sign=True, dim=40):
    qb = superblock.spin_block_labels(dim, 9, seed=41)
    return superblock.synthetic_superblock(dim, 2, qb, [1, -1], 0, nnz_lllr=6, nnz_lrrl=2, seed=seed, with_sign=with_sign)


def test_obc_spmv_golden(gpu):
    lib = gpu.load()
    g = golden("obc_synthetic.npz")
    sb = obc_case()
    x = g["x"].copy()
    y = np.zeros(sb.n)
    lib.DMRG_MATRIX_VECTOR_PRODUCT_OBC(sb.M_LLLR.ref, sb.M_LRRL.ref, sb.M_LRRL_Sign.ref, sb.M_RRRL.ref,
                                       abi.ptr(x, C.c_double), abi.ptr(y, C.c_double), abi.ptr(sb.ele_rr, C.c_int), 4,
                                       C.byref(sb.basis))
    assert np.abs(y - g["y"]).max() <= 1e-13 * np.abs(g["y"]).max()


def test_obc_lanczos_and_ii_vs_oracle(gpu, oracle, in_tmp):
    lib = gpu.load()
    sb = obc_case(seed=7, dim=60)
    guess = np.random.default_rng(3).standard_normal(sb.n)
    vec, val = guess.copy(), np.zeros(1)
    box = abi.DMRG_BOX_LAN(Eig_Vec=abi.ptr(vec, C.c_double), eig_val=abi.ptr(val, C.c_double), acc=1e-14, min_step=1,
                           max_step=800, p_threads=4, Guess=b"Yes", Type=b"Normal", M_LLLR=sb.M_LLLR.ref,
                           M_LRRL=sb.M_LRRL.ref, M_LRRL_Sign=sb.M_LRRL_Sign.ref, M_RRRL=sb.M_RRRL.ref,
                           Ele_RR=abi.ptr(sb.ele_rr, C.c_int), Dmrg_Basis=C.pointer(sb.basis))
    lib.DMRG_LANCZOS_SLOW_OBC(C.byref(box))
    rc, out, vo = oracle.obc_lanczos_slow(sb, guess=guess)
    assert out.converged
    assert abs(val[0] - out.eig_val) < 1e-12 * abs(out.eig_val)
    assert abs(abs(vec @ vo) - 1) < 1e-9
    w = np.linalg.eigvalsh(sb.explicit().toarray())[0]
    assert abs(val[0] - w) < 1e-10 * abs(w)
    ii = abi.DMRG_BOX_II(ii_acc=1e-9, ii_diag_add=1e-11, ii_max_step=3, cg_acc=1e-7, cg_max_step=1000,
                         Eig_Vec=abi.ptr(vec, C.c_double), eig_val=abi.ptr(val, C.c_double), p_threads=4,
                         M_LLLR=sb.M_LLLR.ref, M_LRRL=sb.M_LRRL.ref, M_LRRL_Sign=sb.M_LRRL_Sign.ref,
                         M_RRRL=sb.M_RRRL.ref, Ele_RR=abi.ptr(sb.ele_rr, C.c_int), Dmrg_Basis=C.pointer(sb.basis))
    lib.DMRG_INVERSE_ITERATION_OBC(C.byref(ii))
    rc, oi, vi = oracle.obc_inverse_iteration(sb, out.eig_val, vo)
    assert ii.error < 1e-9 and oi.error < 1e-9
    assert abs(abs(vec @ vi) - 1) < 1e-12
    tmp = np.zeros(sb.n)
    r = lib.DMRG_CONVERGE_CHECK_OBC(val[0], sb.M_LLLR.ref, sb.M_LRRL.ref, sb.M_LRRL_Sign.ref, sb.M_RRRL.ref,
                                    abi.ptr(vec, C.c_double), abi.ptr(tmp, C.c_double), abi.ptr(sb.ele_rr, C.c_int), 4,
                                    C.byref(sb.basis))
    assert r < 1e-8
    np.testing.assert_allclose(tmp, sb.explicit() @ vec, rtol=0, atol=1e-12)


def test_obc_cg_vs_oracle(gpu, oracle, in_tmp):
    lib = gpu.load()
    sb = obc_case(seed=9)
    rng = np.random.default_rng(4)
    b = rng.standard_normal(sb.n)
    x0 = rng.standard_normal(sb.n)
    shift = 40.0     # makes H + shift positive definite
    x = x0.copy()
    box = abi.DMRG_BOX_CG(acc=1e-12, diag_val=shift, Vec=abi.ptr(b, C.c_double), Out_Vec=abi.ptr(x, C.c_double),
                          max_step=1000, p_threads=4, M_LLLR=sb.M_LLLR.ref, M_LRRL=sb.M_LRRL.ref,
                          M_LRRL_Sign=sb.M_LRRL_Sign.ref, M_RRRL=sb.M_RRRL.ref, Ele_RR=abi.ptr(sb.ele_rr, C.c_int),
                          Dmrg_Basis=C.pointer(sb.basis))
    lib.DMRG_CONJUGATE_GRADIENT_OBC(C.byref(box))
    A = sb.explicit()
    assert np.linalg.norm(A @ x + shift * x - b) < 1e-5


def test_obc_matches_explicit_sym_path(gpu):
    """The matrix-free and the explicit lower-triangle forms of one superblock agree."""
    sb = obc_case(seed=11, dim=80)
    m = gpu.DeviceMatrix(sb.explicit_lower(), gpu.DG_STORE_LOWER_DIAG_LAST)
    v, info = gpu.ground_state(m, gpu.default_params(dense_below=0), guess=np.ones(sb.n))
    w = np.linalg.eigvalsh(sb.explicit().toarray())[0]
    assert abs(info.eig_val - w) < 1e-10 * abs(w)


def test_exact_v_m_q0_golden(gpu):
    lib = gpu.load()
    g = golden("vm_hubbard6.npz")
    op = abi.Crs(g["op_row"], g["op_col"], g["op_val"], n=4)
    basis = g["basis"].copy()
    info = abi.EXACT_BASIS_INFO(dim=len(basis), Basis=abi.ptr(basis, C.c_long))
    vec = g["vec"].copy()
    for site in (0, 2, 5):
        out = np.zeros(len(basis))
        lib.EXACT_V_M_Q0(op.ref, abi.ptr(vec, C.c_double), abi.ptr(out, C.c_double), 4, site, 1, C.byref(info))
        np.testing.assert_array_equal(out, g[f"out_site{site}"])


def _q2_apply(lib, op, b_out, b_in, vec, n_ele, d, site):
    dims = np.zeros((1, 2), np.int32)
    dims[0, 0], dims[0, 1] = len(b_out), len(b_in)
    row_dims = (C.POINTER(C.c_int) * 1)(abi.ptr(dims[0], C.c_int))
    bases = (C.POINTER(C.c_long) * 2)(abi.ptr(b_out, C.c_long), abi.ptr(b_in, C.c_long))
    row_bases = (C.POINTER(C.POINTER(C.c_long)) * 1)(C.cast(bases, C.POINTER(C.POINTER(C.c_long))))
    W = abi.EXACT_WHOLE_BASIS_Q2(Dim=C.cast(row_dims, C.POINTER(C.POINTER(C.c_int))),
                                 Basis=C.cast(row_bases, C.POINTER(C.POINTER(C.POINTER(C.c_long)))), max_dim=0)
    out = np.zeros(len(b_out))
    lib.EXACT_V_M_Q2(op.ref, 0, 0, abi.ptr(vec, C.c_double), 0, 1, abi.ptr(out, C.c_double), b"Yes",
                     abi.ptr(n_ele, C.c_int), d, site, 1, C.byref(W))
    return out


def test_exact_v_m_q2_three_state_sites_vs_oracle(gpu, oracle):
    """A local dimension that is not a power of two (the kernel's division path), with the sign
    string: a raising operator between the digit-sum 5 and 6 sectors of six 3-state sites."""
    lib = gpu.load()
    L_, d = 6, 3
    codes = np.arange(d ** L_, dtype=np.int64)
    digit_sum = sum((codes // d ** s) % d for s in range(L_))
    b_in = np.ascontiguousarray(codes[digit_sum == 5])
    b_out = np.ascontiguousarray(codes[digit_sum == 6])
    op = abi.Crs(np.array([0, 0, 1, 2]), np.array([0, 1], np.int32), np.array([1.0, np.sqrt(2.0)]), n=3)
    n_ele = np.array([0, 1, 2], np.int32)
    vec = np.random.default_rng(7).standard_normal(len(b_in))
    for site in (0, 2, 5):
        ref = oracle.site_apply(op, b_out, b_in, d, site, vec, n_ele=n_ele)
        np.testing.assert_array_equal(_q2_apply(lib, op, b_out, b_in, vec, n_ele, d, site), ref)


def test_exact_v_m_q2_sign_vs_oracle(gpu, oracle):
    """Q2 with the Jordan-Wigner sign, between two different (N_e, 2Sz) sectors."""
    lib = gpu.load()
    m_in = ed_models.hubbard_chain(5, n_ele=4, twoSz=0)
    m_out = ed_models.hubbard_chain(5, n_ele=5, twoSz=1)
    b_in = oracle.ed_build(m_in)[0]
    b_out = oracle.ed_build(m_out)[0]
    op = m_in.ops[1]                       # c^dagger_up
    n_ele = np.array([0, 1, 1, 2], np.int32)
    vec = np.random.default_rng(5).standard_normal(len(b_in))
    for site in (0, 3):
        ref = oracle.site_apply(op, b_out, b_in, 4, site, vec, n_ele=n_ele)
        dims = np.zeros((1, 2), np.int32)
        dims[0, 0], dims[0, 1] = len(b_out), len(b_in)
        row_dims = (C.POINTER(C.c_int) * 1)(abi.ptr(dims[0], C.c_int))
        bases = (C.POINTER(C.c_long) * 2)(abi.ptr(b_out, C.c_long), abi.ptr(b_in, C.c_long))
        row_bases = (C.POINTER(C.POINTER(C.c_long)) * 1)(C.cast(bases, C.POINTER(C.POINTER(C.c_long))))
        W = abi.EXACT_WHOLE_BASIS_Q2(Dim=C.cast(row_dims, C.POINTER(C.POINTER(C.c_int))),
                                     Basis=C.cast(row_bases, C.POINTER(C.POINTER(C.POINTER(C.c_long)))), max_dim=0)
        out = np.zeros(len(b_out))
        lib.EXACT_V_M_Q2(op.ref, 0, 0, abi.ptr(vec, C.c_double), 0, 1, abi.ptr(out, C.c_double), b"Yes",
                         abi.ptr(n_ele, C.c_int), 4, site, 1, C.byref(W))
        np.testing.assert_array_equal(out, ref)
