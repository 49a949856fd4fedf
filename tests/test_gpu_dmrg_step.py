"""One DMRG step through the library, end to end, against the oracle's chain: the superblock basis
built on the device, the ground state, the site expectation values, the truncation of the LL+LR
block (DMRG_GET_SYSTEM_INFO_Q2) and the renormalisation of a block operator with the kept
states (CRS_CRS_CCS_PRODUCT).  Every stage consumes the previous stage's GPU output."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from dmrg_c_gb300 import abi, sb_models, superblock, workloads

pytestmark = pytest.mark.gpu


def _free():
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    return libc.free


def test_dmrg_step_chain(gpu, oracle):
    rng = np.random.default_rng(3)
    dim, d = 48, 4
    qb = workloads._block_labels(dim, 9, 9.0, 1.0, 0.9, 7)
    qs = workloads.hubbard_site_labels()
    target = 20 * workloads.QN_SCALE
    sb = superblock.synthetic_superblock(dim, d, qb, qs, target, nnz_lllr=6, nnz_lrrl=2, seed=8)
    states = (sb.LL, sb.LR, sb.RR, sb.RL)
    # 1. basis on the device, in the reference's order
    b = gpu.SuperblockBasis(dim, dim, d, qb, qb, qs, target)
    LL, LR, RR, RL, inv = b.download()
    assert np.array_equal(np.stack([LL, LR, RR, RL]), np.stack(states).astype(np.int16))
    assert np.array_equal(inv, sb.inv)
    # 2. ground state (FP64 Lanczos + inverse iteration) against the oracle's
    H = sb.explicit()
    m = gpu.DeviceMatrix(abi.Crs.from_scipy(H))
    psi, info = gpu.ground_state(m, gpu.default_params())
    e_ref = float(np.linalg.eigvalsh(H.toarray())[0])
    assert abs(info.eig_val - e_ref) <= 1e-10 * abs(e_ref)
    psi = psi / np.linalg.norm(psi)
    # 3. site expectation values on the ground state (density-matrix form) against product-then-dot
    ops_LL = [sb_models._crs(sb_models._random_sym_op(qb, 5, rng)) for _ in range(3)]
    host_ops = ops_LL + [sb_models._crs(sp.csr_matrix(np.diag([0.0, 1.0, 1.0, 2.0])))]
    ops = gpu.BlockOperators(host_ops, [dim] * 3 + [d])
    terms = [(0, k, 0, 0) for k in range(3)] + [(1, 3, 0, 0), (3, 3, 0, 0)]
    got = gpu.sb_expect(b, b, ops, terms, psi, psi)
    for k, (pos, op, _, _) in enumerate(terms):
        y = oracle.sb_vm(states, sb.inv, dim, d, host_ops[op], pos, psi)
        assert abs(got[k] - psi @ y) <= 1e-12 * float(np.abs(psi) @ np.abs(y)), k
    # 4. truncation of the LL+LR block to 40 states on the GPU ground state
    lllr = oracle.lllr_list(qb, qs, states)
    lab = lllr[3]
    N = np.rint(lab / workloads.QN_SCALE).astype(np.int32)
    qns = [N, (lab - N * workloads.QN_SCALE).astype(np.int32)]
    trunc = oracle.call_system_info(gpu.load(), qns, states, sb.inv, dim, dim, d, psi, lllr, 40, _free())
    assert oracle.same_truncation(trunc, oracle.system_info(qns, states, sb.inv, d, dim, psi, lllr, 40)) == []
    # 5. renormalise a block operator (O on LL, as DMRG_MAKE_LL_OP_LLLR lays it out) with the kept states
    nr, L = trunc["dim_renorm"], len(lllr[0])
    T = sp.csc_matrix((trunc["vals"], trunc["rows"], trunc["col_ptr"]), shape=(L, nr))
    O_ll = ops_LL[0]
    pair = {(int(a), int(c)): i for i, (a, c) in enumerate(zip(lllr[0], lllr[1]))}
    Od = sp.csr_matrix((O_ll.val[:O_ll.nnz], O_ll.col[:O_ll.nnz], O_ll.row), shape=(dim, dim)).toarray()
    O_lllr = np.zeros((L, L))
    for (a, lr), i in pair.items():
        for c in range(dim):
            if Od[a, c] != 0.0 and (c, lr) in pair:
                O_lllr[i, pair[(c, lr)]] = Od[a, c]
    M1, M2, M3 = abi.Crs.from_scipy(sp.csr_matrix(T.T)), abi.Crs.from_scipy(sp.csr_matrix(O_lllr)), abi.Ccs.from_scipy(T)
    r = oracle.call_crs_crs_ccs(gpu.load(), M1, M2, M3, L * nr, nr * nr)
    want = oracle.crs_crs_ccs(M1, M2, M3)
    for x, y in zip(r[:6], want):
        x, y = np.asarray(x), np.asarray(y)
        assert np.array_equal(x.astype(np.float64).view(np.int64) if x.dtype == np.float64 else x.astype(np.int64),
                              y.astype(np.float64).view(np.int64) if y.dtype == np.float64 else y.astype(np.int64))
    # the renormalised operator is T^T O T
    Out = sp.csr_matrix((r[5], r[4], r[3]), shape=(nr, nr)).toarray()
    assert np.allclose(Out, T.T @ O_lllr @ T, rtol=0, atol=1e-12)
