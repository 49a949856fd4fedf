"""Superblock operators in the reference's layout, for the matrix-free OBC path and for
the explicit *_SYM path.

A superblock state is (LL, LR, RR, RL): left block state, left site, right block state,
right site.  The reference keeps the states of one symmetry sector ordered by
(quantum number of LL+LR, LL, LR, RR, RL) (dmrg/DMRG_QUICK_SORT_BASIS_Q1.c:28-41,
main/dmrg/xxz_vf/src/allocations/GET_BASIS_SUPERBLOCK.c:231-259), maps every
(LL, LR, RR, RL) to its position through the dense table Inv_LLLRRRRL (-1 outside the
sector, :267-281), and numbers the distinct (LL, LR), (LR, RL) and (RR, RL) pairs in order
of first appearance (:283-301, dmrg/DMRG_GET_BASIS_LRRL.c, DMRG_GET_BASIS_RRRL.c).  The
Hamiltonian is H_LLLR + H_LRRL + (-1)^Ele_RR H_LRRL_Sign + H_RRRL, each acting on its pair
space (dmrg/DMRG_MATRIX_VECTOR_PRODUCT_OBC.c).

``synthetic_superblock`` builds such an operator from seeded random symmetric block
operators that conserve the quantum number, with the sizes of a chosen DMRG step; it stands
in for the block operators a DMRG sweep would produce (no reference run is involved).
``explicit`` assembles the same operator as a CRS: the full matrix, or the
lower-triangle-diagonal-last layout that GET_HAM_LLLRRRRL produces
(main/dmrg/xxz_vf/src/allocations/GET_HAM_LLLRRRRL.c:51,92,111).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp

from .abi import DMRG_BASIS, Crs, ptr


def _int2d(a: np.ndarray):
    """int** view of a 2-D int32 array (rows kept alive by the returned tuple)."""
    a = np.ascontiguousarray(a, np.int32)
    rows = (C.POINTER(C.c_int) * a.shape[0])(*[ptr(a[i], C.c_int) for i in range(a.shape[0])])
    return a, rows


def _random_sym_block(qn: np.ndarray, nnz_per_row: float, rng, scale=1.0) -> sp.csr_matrix:
    """Random symmetric matrix on a pair space conserving qn (entries only between equal qn)."""
    n = len(qn)
    rows, cols, vals = [], [], []
    order = np.argsort(qn, kind="stable")
    q_sorted = qn[order]
    bounds = np.flatnonzero(np.diff(q_sorted)) + 1
    for grp in np.split(order, bounds):
        g = len(grp)
        k = max(1, min(g, int(round(nnz_per_row))))
        # each row connects to ~k random partners of its sector (symmetrised below)
        for i in grp:
            partners = rng.choice(grp, size=k, replace=False) if g > 1 else grp
            rows.extend([i] * len(partners))
            cols.extend(partners.tolist())
            vals.extend((rng.standard_normal(len(partners)) * scale).tolist())
    A = sp.coo_matrix((vals, (rows, cols)), shape=(n, n)).tocsr()
    A = (A + A.T) * 0.5
    A.sum_duplicates()
    A.eliminate_zeros()
    A.sort_indices()
    return A.tocsr()


@dataclass
class Superblock:
    n: int
    dim_LL: int
    dim_RR: int
    d: int
    LL: np.ndarray
    LR: np.ndarray
    RR: np.ndarray
    RL: np.ndarray
    inv: np.ndarray
    lllr: np.ndarray      # (dim_LLLR, 2) pairs (LL, LR)
    lrrl: np.ndarray
    rrrl: np.ndarray
    inv_lllr: np.ndarray  # (dim_LL, d)
    inv_lrrl: np.ndarray  # (d, d)
    inv_rrrl: np.ndarray  # (dim_RR, d)
    H_LLLR: sp.csr_matrix
    H_LRRL: sp.csr_matrix
    H_LRRL_Sign: sp.csr_matrix
    H_RRRL: sp.csr_matrix
    ele_rr: np.ndarray
    _keep: list = field(default_factory=list, repr=False)

    def __post_init__(self):
        self.M_LLLR = Crs.from_scipy(self.H_LLLR)
        self.M_LRRL = Crs.from_scipy(self.H_LRRL)
        self.M_LRRL_Sign = Crs.from_scipy(self.H_LRRL_Sign)
        self.M_RRRL = Crs.from_scipy(self.H_RRRL)
        self.ele_rr = np.ascontiguousarray(self.ele_rr, np.int32)
        sh = lambda a: np.ascontiguousarray(a, np.int16)  # noqa: E731
        self._arr = dict(LL=sh(self.LL), LR=sh(self.LR), RR=sh(self.RR), RL=sh(self.RL),
                         inv=np.ascontiguousarray(self.inv, np.int32),
                         ll_lllr=sh(self.lllr[:, 0]), lr_lllr=sh(self.lllr[:, 1]), lr_lrrl=sh(self.lrrl[:, 0]),
                         rl_lrrl=sh(self.lrrl[:, 1]), rr_rrrl=sh(self.rrrl[:, 0]), rl_rrrl=sh(self.rrrl[:, 1]))
        i1, p1 = _int2d(self.inv_lllr)
        i2, p2 = _int2d(self.inv_lrrl)
        i3, p3 = _int2d(self.inv_rrrl)
        self._keep = [i1, p1, i2, p2, i3, p3]
        a = self._arr
        s = lambda k: ptr(a[k], C.c_short)  # noqa: E731
        self.basis = DMRG_BASIS(
            LL_LLLRRRRL=s("LL"), LR_LLLRRRRL=s("LR"), RL_LLLRRRRL=s("RL"), RR_LLLRRRRL=s("RR"),
            Inv_LLLRRRRL=ptr(a["inv"], C.c_int), dim_LLLRRRRL=self.n, dim_LL=self.dim_LL, dim_RR=self.dim_RR,
            dim_onsite=self.d, LL_LLLR=s("ll_lllr"), LR_LLLR=s("lr_lllr"), Inv_LLLR=C.cast(p1, C.POINTER(C.POINTER(C.c_int))),
            dim_LLLR=len(self.lllr), LR_LRRL=s("lr_lrrl"), RL_LRRL=s("rl_lrrl"),
            Inv_LRRL=C.cast(p2, C.POINTER(C.POINTER(C.c_int))), dim_LRRL=len(self.lrrl), RR_RRRL=s("rr_rrrl"),
            RL_RRRL=s("rl_rrrl"), Inv_RRRL=C.cast(p3, C.POINTER(C.POINTER(C.c_int))), dim_RRRL=len(self.rrrl))

    def _sup(self, ll, lr, rr, rl):
        d, R = self.d, self.dim_RR
        return ((ll.astype(np.int64) * d + lr) * R + rr) * d + rl

    def explicit(self) -> sp.csr_matrix:
        """The same operator as an explicit full CRS (duplicates summed)."""
        rows_all, cols_all, vals_all = [], [], []
        b = np.arange(self.n)

        def term(H, r, colmap, sign=None):
            H = H.tocsr()
            cnt = (H.indptr[r + 1] - H.indptr[r]).astype(np.int64)
            rr = np.repeat(b, cnt)
            start = np.repeat(H.indptr[r], cnt)
            off = np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt)
            k = start + off
            c = H.indices[k]
            v = H.data[k].copy()
            inv = colmap(rr, c)
            if sign is not None:
                v = v * sign[rr]
            keep = inv >= 0
            rows_all.append(rr[keep])
            cols_all.append(inv[keep])
            vals_all.append(v[keep])

        LL, LR, RR, RL = (x.astype(np.int64) for x in (self.LL, self.LR, self.RR, self.RL))
        r1 = self.inv_lllr[LL, LR]
        term(self.H_LLLR, r1, lambda rr, c: self.inv[self._sup(self.lllr[c, 0], self.lllr[c, 1], RR[rr], RL[rr])])
        r2 = self.inv_lrrl[LR, RL]
        f2 = lambda rr, c: self.inv[self._sup(LL[rr], self.lrrl[c, 0], RR[rr], self.lrrl[c, 1])]  # noqa: E731
        term(self.H_LRRL, r2, f2)
        if self.H_LRRL_Sign.nnz:
            sign = np.where(self.ele_rr[RR] % 2 == 1, -1.0, 1.0)
            term(self.H_LRRL_Sign, r2, f2, sign)
        r3 = self.inv_rrrl[RR, RL]
        term(self.H_RRRL, r3, lambda rr, c: self.inv[self._sup(LL[rr], LR[rr], self.rrrl[c, 0], self.rrrl[c, 1])])
        A = sp.coo_matrix((np.concatenate(vals_all), (np.concatenate(rows_all), np.concatenate(cols_all))),
                          shape=(self.n, self.n)).tocsr()
        A.sum_duplicates()
        A.sort_indices()
        return A

    def explicit_lower(self) -> Crs:
        """Lower triangle with the diagonal stored last (explicit zero when absent), entries
        with |v| <= 1e-15 dropped off the diagonal (GET_HAM_LLLRRRRL.c:51)."""
        A = self.explicit()
        L = sp.tril(A, k=-1).tocsr()
        L.data[np.abs(L.data) <= 1e-15] = 0.0
        L.eliminate_zeros()
        L.sort_indices()
        diag = A.diagonal()
        n = self.n
        cnt = np.diff(L.indptr) + 1
        row = np.zeros(n + 1, np.int64)
        np.cumsum(cnt, out=row[1:])
        col = np.empty(row[-1], np.int32)
        val = np.empty(row[-1], np.float64)
        pos_diag = row[1:] - 1
        mask = np.ones(row[-1], bool)
        mask[pos_diag] = False
        col[mask] = L.indices
        val[mask] = L.data
        col[pos_diag] = np.arange(n)
        val[pos_diag] = diag
        return Crs(row, col, val, n=n)


def synthetic_superblock(dim_LL: int, d: int, qn_block, qn_site, target: int, nnz_lllr: float, nnz_lrrl: float,
                         seed: int = 0, dim_RR: int | None = None, qn_block_r=None, with_sign: bool = False,
                         diag_shift: float = 0.0) -> Superblock:
    """Seeded random superblock operator in one symmetry sector.

    qn_block / qn_site: integer quantum number of every block / site state (several
    conserved quantities can be packed into one integer, e.g. N*1000 + 2Sz, which keeps the
    reference's key order N first).  nnz_lllr / nnz_lrrl: target stored entries per row of
    the pair-space operators."""
    rng = np.random.default_rng(seed)
    dim_RR = dim_LL if dim_RR is None else dim_RR
    qb = np.asarray(qn_block, np.int64)
    qr = qb if qn_block_r is None else np.asarray(qn_block_r, np.int64)
    qs = np.asarray(qn_site, np.int64)
    LL, LR, RR, RL = np.meshgrid(np.arange(dim_LL), np.arange(d), np.arange(dim_RR), np.arange(d), indexing="ij")
    LL, LR, RR, RL = (x.ravel() for x in (LL, LR, RR, RL))
    tot = qb[LL] + qs[LR] + qr[RR] + qs[RL]
    keep = tot == target
    LL, LR, RR, RL = LL[keep], LR[keep], RR[keep], RL[keep]
    q_lllr = qb[LL] + qs[LR]
    order = np.lexsort((RL, RR, LR, LL, q_lllr))   # primary key last
    LL, LR, RR, RL = LL[order], LR[order], RR[order], RL[order]
    n = len(LL)
    if n == 0:
        raise ValueError("empty superblock sector")
    inv = -np.ones(dim_LL * d * dim_RR * d, np.int32)
    inv[((LL * d + LR) * dim_RR + RR) * d + RL] = np.arange(n, dtype=np.int32)

    def pairs(a, b, da, db):
        key = a * db + b
        _, first = np.unique(key, return_index=True)
        first = np.sort(first)
        pr = np.stack([a[first], b[first]], axis=1)
        table = -np.ones((da, db), np.int32)
        table[pr[:, 0], pr[:, 1]] = np.arange(len(pr), dtype=np.int32)
        return pr, table

    lllr, inv_lllr = pairs(LL, LR, dim_LL, d)
    lrrl, inv_lrrl = pairs(LR, RL, d, d)
    rrrl, inv_rrrl = pairs(RR, RL, dim_RR, d)
    H_LLLR = _random_sym_block(qb[lllr[:, 0]] + qs[lllr[:, 1]], nnz_lllr, rng)
    H_LRRL = _random_sym_block(qs[lrrl[:, 0]] + qs[lrrl[:, 1]], nnz_lrrl, rng)
    H_RRRL = _random_sym_block(qr[rrrl[:, 0]] + qs[rrrl[:, 1]], nnz_lllr, rng)
    if diag_shift:
        H_LLLR = (H_LLLR + sp.identity(H_LLLR.shape[0]) * diag_shift).tocsr()
    if with_sign:
        H_sign = _random_sym_block(qs[lrrl[:, 0]] + qs[lrrl[:, 1]], max(1.0, nnz_lrrl / 2), rng, scale=0.5)
        ele_rr = rng.integers(0, 4, size=dim_RR).astype(np.int32)
    else:
        H_sign = sp.csr_matrix((len(lrrl), len(lrrl)))
        ele_rr = np.zeros(dim_RR, np.int32)
    return Superblock(n, dim_LL, dim_RR, d, LL, LR, RR, RL, inv, lllr, lrrl, rrrl, inv_lllr, inv_lrrl, inv_rrrl, H_LLLR,
                      H_LRRL, H_sign, H_RRRL, ele_rr)


def spin_block_labels(dim: int, n_sites: int, seed: int = 0) -> np.ndarray:
    """2Sz labels for a block of `dim` kept states of an n_sites spin-1/2 block: sampled
    from the binomial distribution of 2Sz over the full block space (seeded)."""
    rng = np.random.default_rng(seed)
    k = rng.binomial(n_sites, 0.5, size=dim)
    return np.sort(2 * k - n_sites)
