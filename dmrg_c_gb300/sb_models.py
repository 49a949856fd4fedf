"""Superblock Hamiltonians as dg_sb_model term lists (the GPU superblock CRS build).

A term applies one operator to one of the positions LL, LR, RR, RL of a superblock state, or
two operators to two positions, with an optional fermionic sign from the electron numbers
of chosen positions -- the primitives of dmrg/DMRG_MAKE_ELEM_*_LLLRRRRL.c.  The list order
is the order a model's MAKE_ELEMENT_HAM_LLLRRRRL applies them, e.g. the 1D Hubbard model's
(main/dmrg/hubbard_vf/src/*/MAKE_ELEMENT_HAM_LLLRRRRL.c:16-45): block and site
Hamiltonians, then hopping across LL-LR, RR-RL and LR-RL.

``hubbard_superblock_model`` fills that term list with seeded random block operators that
change the block quantum numbers as c^dagger / c do (they stand in for the renormalised
block operators of a DMRG sweep) on the basis of a ``superblock.Superblock``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp

from .abi import CRS1, Crs, dg_sb_model, dg_sb_term, ptr
from .workloads import QN_SCALE

LL, LR, RR, RL = 0, 1, 2, 3
M_LL, M_LR, M_RR, M_RL = 1, 2, 4, 8


@dataclass
class SBModel:
    """A dg_sb_model with the numpy storage it points into."""
    n: int
    dim_LL: int
    dim_RR: int
    d: int
    LL: np.ndarray
    LR: np.ndarray
    RR: np.ndarray
    RL: np.ndarray
    inv: np.ndarray
    ops: list
    terms: list
    ele: list            # 4 arrays or None
    _keep: list = field(default_factory=list, repr=False)

    def __post_init__(self):
        sh = lambda a: np.ascontiguousarray(a, np.int16)  # noqa: E731
        self.LL, self.LR, self.RR, self.RL = sh(self.LL), sh(self.LR), sh(self.RR), sh(self.RL)
        self.inv = np.ascontiguousarray(self.inv, np.int32)
        self.ele = [None if e is None else np.ascontiguousarray(e, np.int32) for e in self.ele]
        ops_arr = (CRS1 * len(self.ops))(*[o.struct for o in self.ops])
        terms_arr = (dg_sb_term * max(len(self.terms), 1))(*[dg_sb_term(*t) for t in self.terms])
        eles = (C.POINTER(C.c_int) * 4)(*[ptr(e, C.c_int) if e is not None else None for e in self.ele])
        self._keep = [ops_arr, terms_arr]
        self.struct = dg_sb_model(
            n=self.n, dim_LL=self.dim_LL, dim_RR=self.dim_RR, dim_onsite=self.d, LL=ptr(self.LL, C.c_short),
            LR=ptr(self.LR, C.c_short), RR=ptr(self.RR, C.c_short), RL=ptr(self.RL, C.c_short), inv=ptr(self.inv, C.c_int),
            n_ops=len(self.ops), ops=C.cast(ops_arr, C.POINTER(CRS1)), n_terms=len(self.terms),
            terms=C.cast(terms_arr, C.POINTER(dg_sb_term)), ele=eles)


def _crs(M: sp.csr_matrix) -> Crs:
    M = M.tocsr()
    M.sort_indices()
    return Crs(M.indptr.astype(np.int64), M.indices.astype(np.int32), M.data.astype(np.float64), n=M.shape[0])


def _random_shift_op(qn, delta, per_row, rng) -> sp.csr_matrix:
    """Block operator that takes a state with quantum number q to states with q + delta."""
    n = len(qn)
    rows, cols, vals = [], [], []
    for r in range(n):
        cand = np.flatnonzero(qn == qn[r] + delta)
        if len(cand) == 0:
            continue
        k = min(len(cand), per_row)
        c = rng.choice(cand, size=k, replace=False)
        rows.extend([r] * k)
        cols.extend(c.tolist())
        vals.extend(rng.standard_normal(k).tolist())
    return sp.csr_matrix((vals, (rows, cols)), shape=(n, n))


def _random_sym_op(qn, per_row, rng) -> sp.csr_matrix:
    A = _random_shift_op(qn, 0, per_row, rng)
    A = (A + A.T) * 0.5
    A.sum_duplicates()
    A.eliminate_zeros()
    return A.tocsr()


def hubbard_superblock_model(sb, qn_block, qn_block_r=None, seed=0, per_row=4, t1=-1.0, U=4.0, pbc=False) -> SBModel:
    """Hubbard-type superblock term list on the basis of Superblock `sb` (site dimension 4,
    local states empty / up / down / up+down; quantum numbers packed N * QN_SCALE + 2Sz)."""
    assert sb.d == 4
    rng = np.random.default_rng(seed)
    qb = np.asarray(qn_block, np.int64)
    qr = qb if qn_block_r is None else np.asarray(qn_block_r, np.int64)
    up, dn = QN_SCALE + 1, QN_SCALE - 1          # c^dagger_up / c^dagger_down shifts
    # site operators; row = current local state, column = new one (the element builders'
    # convention): c^dagger_up takes empty -> up and down -> up+down, c^dagger_down takes
    # empty -> down and up -> up+down with the fermionic minus sign
    cupd = np.zeros((4, 4))
    cupd[0, 1] = 1.0
    cupd[2, 3] = 1.0
    cdnd = np.zeros((4, 4))
    cdnd[0, 2] = 1.0
    cdnd[1, 3] = -1.0
    ham_on = np.diag([0.0, 0.0, 0.0, U])
    site = lambda M: _crs(sp.csr_matrix(M))  # noqa: E731
    ops = []

    def add(M):
        ops.append(M if isinstance(M, Crs) else _crs(M))
        return len(ops) - 1

    H_S = add(_random_sym_op(qb, per_row, rng))
    H_E = add(_random_sym_op(qr, per_row, rng))
    H_On = add(site(ham_on))
    CupD_S = _random_shift_op(qb, up, per_row, rng)
    CdnD_S = _random_shift_op(qb, dn, per_row, rng)
    CupD_E = _random_shift_op(qr, up, per_row, rng)
    CdnD_E = _random_shift_op(qr, dn, per_row, rng)
    iCupD_S, iCup_S = add(CupD_S), add(CupD_S.T.tocsr())
    iCdnD_S, iCdn_S = add(CdnD_S), add(CdnD_S.T.tocsr())
    iCupD_E, iCup_E = add(CupD_E), add(CupD_E.T.tocsr())
    iCdnD_E, iCdn_E = add(CdnD_E), add(CdnD_E.T.tocsr())
    iCupD_On, iCup_On = add(site(cupd)), add(site(cupd.T))
    iCdnD_On, iCdn_On = add(site(cdnd)), add(site(cdnd.T))
    terms = [(LL, -1, H_S, 0, 1.0, 0, 1), (RR, -1, H_E, 0, 1.0, 0, 1), (LR, -1, H_On, 0, 1.0, 0, 1),
             (RL, -1, H_On, 0, 1.0, 0, 1)]
    for a, b, ev in ((iCupD_S, iCup_On, -1), (iCup_S, iCupD_On, 1), (iCdnD_S, iCdn_On, -1), (iCdn_S, iCdnD_On, 1)):
        terms.append((LL, LR, a, b, t1, M_LL, ev))
    for a, b, ev in ((iCupD_E, iCup_On, -1), (iCup_E, iCupD_On, 1), (iCdnD_E, iCdn_On, -1), (iCdn_E, iCdnD_On, 1)):
        terms.append((RR, RL, a, b, t1, M_RR, ev))
    for a, b, ev in ((iCupD_On, iCup_On, -1), (iCup_On, iCupD_On, 1), (iCdnD_On, iCdn_On, -1), (iCdn_On, iCdnD_On, 1)):
        terms.append((LR, RL, a, b, t1, M_RR | M_LR, ev))
    if pbc:
        # closing bond between the two block edges and the sites (the PBC branches of the
        # model drivers: LRRR, LLRL, LLRR element builders)
        terms.append((LR, RR, iCupD_On, iCup_E, t1, M_LR, -1))
        terms.append((LR, RR, iCup_On, iCupD_E, t1, M_LR, 1))
        terms.append((LL, RL, iCupD_S, iCup_On, t1, M_LL | M_RR | M_LR, -1))
        terms.append((LL, RL, iCup_S, iCupD_On, t1, M_LL | M_RR | M_LR, 1))
        terms.append((LL, RR, iCdnD_S, iCdn_E, t1, M_LL | M_LR, -1))
        terms.append((LL, RR, iCdn_S, iCdnD_E, t1, M_LL | M_LR, 1))
    ele_b = np.rint(qb / QN_SCALE).astype(np.int32)
    ele_r = np.rint(qr / QN_SCALE).astype(np.int32)
    ele_site = np.array([0, 1, 1, 2], np.int32)
    return SBModel(sb.n, sb.dim_LL, sb.dim_RR, 4, sb.LL, sb.LR, sb.RR, sb.RL, sb.inv, ops, terms,
                   [ele_b, ele_site, ele_r, ele_site])


def small_hubbard_model(pbc=False) -> SBModel:
    """A seeded 600-state Hubbard-type superblock (blocks of 40 states, 7 sites, N = 14):
    small enough for the CPU oracle and the reference's own builders in seconds."""
    from . import superblock, workloads
    qb = workloads._block_labels(40, 7, 7.0, 1.0, 0.9, 3)
    sb = superblock.synthetic_superblock(40, 4, qb, workloads.hubbard_site_labels(), 14 * QN_SCALE, nnz_lllr=1, nnz_lrrl=1,
                                         seed=4, with_sign=True)
    return hubbard_superblock_model(sb, qb, seed=5, per_row=3, pbc=pbc)
