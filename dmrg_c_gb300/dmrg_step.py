"""The steps after the superblock solve, on the GPU: site expectation values, the truncation of the
LL+LR block and the renormalisation of a block operator with the kept states -- the work of a
model driver's EXPECTATION_VALUES, RENORMALIZE (DMRG_GET_SYSTEM_INFO_Q2) and TRANSFORM_MATRIX
(CRS_CRS_CCS_PRODUCT) -- on a superblock whose states are in the reference's order.

`post_solve` times each of them on a solved ground state; the reference-facing calls take host
arrays, as the drivers hold them."""
from __future__ import annotations

import ctypes as C
import time

import numpy as np
import scipy.sparse as sp

from . import abi
from . import lib as L
from .workloads import QN_SCALE


def lllr_list(q_LL, q_site, states):
    """The DMRG_BASIS LLLR list in the reference's order: every (LL, LR) pair by (label of LL+LR,
    LL, LR); the number of superblock states of each pair; the pair labels."""
    q_LL, q_site = np.asarray(q_LL, np.int64), np.asarray(q_site, np.int64)
    d = len(q_site)
    LL, LR = (x.ravel() for x in np.meshgrid(np.arange(len(q_LL)), np.arange(d), indexing="ij"))
    lab = q_LL[LL] + q_site[LR]
    order = np.lexsort((LR, LL, lab))
    LL, LR, lab = LL[order], LR[order], lab[order]
    cnt = np.zeros(len(q_LL) * d, np.int64)
    np.add.at(cnt, np.asarray(states[0], np.int64) * d + np.asarray(states[1], np.int64), 1)
    return LL.astype(np.int16), LR.astype(np.int16), np.ascontiguousarray(cnt[LL * d + LR], np.int32), lab


def _block_ops(q, n_ops, per_row, rng):
    """Seeded symmetric block operators conserving the labels q (stand-ins for site observables)."""
    out = []
    for _ in range(n_ops):
        rows, cols, vals = [], [], []
        for r in range(len(q)):
            cand = np.flatnonzero(q == q[r])
            k = min(len(cand), per_row)
            c = rng.choice(cand, size=k, replace=False)
            rows += [r] * k
            cols += c.tolist()
            vals += rng.standard_normal(k).tolist()
        A = sp.csr_matrix((vals, (rows, cols)), shape=(len(q), len(q)))
        A = ((A + A.T) * 0.5).tocsr()
        A.sort_indices()
        out.append(abi.Crs(A.indptr, A.indices, A.data, n=len(q)))
    return out


def post_solve(sb, q_LL, q_site, v, max_dim, n_sites, repeats=3, seed=0):
    """Time, on the solved vector v of superblock sb (block labels q_LL on both sides, site labels
    q_site): the <v|O|v> of n_sites block operators on each side and of a site operator on LR and RL
    (dg_sb_expect, vector resident); DMRG_GET_SYSTEM_INFO_Q2 keeping max_dim states; and
    CRS_CRS_CCS_PRODUCT renormalising one LL operator with the kept states.  Milliseconds per call."""
    rng = np.random.default_rng(seed)
    lib = L.load()
    d, dim = sb.d, sb.dim_LL
    states = (sb.LL, sb.LR, sb.RR, sb.RL)
    v = np.ascontiguousarray(v, np.float64) / np.linalg.norm(v)
    res = {}
    # site expectation values
    b = L.superblock_states(states, dim, sb.dim_RR, d, inv=sb.inv)
    ops_l = _block_ops(np.asarray(q_LL), n_sites, 8, rng)
    ops_r = _block_ops(np.asarray(q_LL), n_sites, 8, rng)
    site = abi.Crs(np.arange(d + 1), np.arange(d, dtype=np.int32), rng.standard_normal(d), n=d)
    ops = L.BlockOperators(ops_l + ops_r + [site], [dim] * (2 * n_sites) + [d])
    terms = ([(0, k, 0, 0) for k in range(n_sites)] + [(1, 2 * n_sites, 0, 0), (3, 2 * n_sites, 0, 0)]
             + [(2, n_sites + k, 0, 0) for k in range(n_sites)])
    import torch
    vd = torch.from_numpy(v).cuda()
    L.sb_expect(b, b, ops, terms, vd, vd)
    t0 = time.perf_counter()
    for _ in range(repeats):
        vals = L.sb_expect(b, b, ops, terms, vd, vd)
    res["expectation_ms"] = (time.perf_counter() - t0) / repeats * 1e3
    res["expectation_terms"] = len(terms)
    res["sum_of_site_values"] = float(np.sum(vals))
    # truncation (host arrays, as RENORMALIZE holds them)
    LLl, LRl, sums, lab = lllr_list(q_LL, q_site, states)
    N = np.ascontiguousarray(np.rint(lab / QN_SCALE), np.int32)
    sz = np.ascontiguousarray(lab - N * QN_SCALE, np.int32)
    st = [np.ascontiguousarray(a, np.int16) for a in states]
    inv = np.ascontiguousarray(sb.inv, np.int32)
    B = abi.DMRG_BASIS(LL_LLLRRRRL=abi.ptr(st[0], C.c_short), LR_LLLRRRRL=abi.ptr(st[1], C.c_short),
                       RR_LLLRRRRL=abi.ptr(st[2], C.c_short), RL_LLLRRRRL=abi.ptr(st[3], C.c_short),
                       Inv_LLLRRRRL=abi.ptr(inv, C.c_int), dim_LLLRRRRL=len(st[0]), dim_LL=dim, dim_RR=sb.dim_RR, dim_onsite=d,
                       LL_LLLR=abi.ptr(LLl, C.c_short), LR_LLLR=abi.ptr(LRl, C.c_short), dim_LLLR=len(LLl),
                       Sum_LLLR=abi.ptr(sums, C.c_int))
    T_time = abi.DMRG_TIME()
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]

    def truncate():
        S = lib.DMRG_GET_SYSTEM_INFO_Q2(abi.ptr(N, C.c_int), abi.ptr(sz, C.c_int), C.byref(B), abi.ptr(v, C.c_double), max_dim, 1,
                                        C.byref(T_time)).contents
        nr, TM = S.dim_renorm, S.Trans_Matrix.contents
        nnz = TM.Col[nr]
        T = sp.csc_matrix((np.array(TM.Val[:nnz]), np.array(TM.Row[:nnz]), np.array(TM.Col[:nr + 1])), shape=(len(LLl), nr))
        tr = S.tr_error
        for m in (TM, S.Trans_Matrix_Dagger.contents):
            for a in (m.Val, m.Row, m.Col):
                libc.free(C.cast(a, C.c_void_p))
        for a in (S.Trans_Matrix, S.Trans_Matrix_Dagger, S.Val_DM_Dist, S.Q_Number1, S.Q_Number2, S.Q_Number3):
            libc.free(C.cast(a, C.c_void_p))
        libc.free(C.cast(C.pointer(S), C.c_void_p))
        return T, tr

    truncate()
    t0 = time.perf_counter()
    for _ in range(repeats):
        T, tr = truncate()
    res["truncation_ms"] = (time.perf_counter() - t0) / repeats * 1e3
    res["kept"] = T.shape[1]
    res["truncation_error"] = tr
    # renormalisation of one LL operator, laid out on the LLLR basis as DMRG_MAKE_LL_OP_LLLR lays it out
    pair = -np.ones((dim, d), np.int64)
    pair[LLl.astype(np.int64), LRl.astype(np.int64)] = np.arange(len(LLl))
    O = sp.csr_matrix((ops_l[0].val[:ops_l[0].nnz], ops_l[0].col[:ops_l[0].nnz], ops_l[0].row), shape=(dim, dim)).tocoo()
    rows, cols, vals_o = [], [], []
    for lr in range(d):
        r, c = pair[O.row, lr], pair[O.col, lr]
        ok = (r >= 0) & (c >= 0)
        rows.append(r[ok])
        cols.append(c[ok])
        vals_o.append(O.data[ok])
    O_lllr = sp.csr_matrix((np.concatenate(vals_o), (np.concatenate(rows), np.concatenate(cols))), shape=(len(LLl), len(LLl)))
    O_lllr.sort_indices()
    nr, nl = T.shape[1], len(LLl)
    M1, M2, M3 = abi.Crs.from_scipy(T.T.tocsr()), abi.Crs.from_scipy(O_lllr), abi.Ccs.from_scipy(T)
    work = abi.Ccs.empty(nr, nl * nr)
    out = abi.Crs(np.zeros(nr + 1, np.int64), np.zeros(nr * nr, np.int32), np.zeros(nr * nr), n=nr)
    wv = np.zeros(nl)
    args = (M1.ref, M2.ref, M3.ref, out.ref, work.ref, abi.ptr(wv, C.c_double))
    lib.CRS_CRS_CCS_PRODUCT(*args)
    t0 = time.perf_counter()
    for _ in range(repeats):
        lib.CRS_CRS_CCS_PRODUCT(*args)
    res["renormalisation_ms"] = (time.perf_counter() - t0) / repeats * 1e3
    res["renormalised_nnz"] = int(out.row[nr])
    return res
