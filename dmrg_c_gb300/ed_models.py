"""Exact-diagonalisation Hamiltonians as dg_ed_model term lists.

The reference ships one ED model program (the 1D Kondo lattice,
main/exact_diag/klm_vf/src/MAKE_ELEMENT_HAM.c:11-76).  Its term order is: the on-site
Hamiltonian on every site, then per bond the spin-exchange terms and the four hopping
terms with the Jordan-Wigner sign of the left site, then (PBC) the closing bond, then a
zero-valued diagonal.  The XXZ and Hubbard chains below follow the same recipe with the
reference's own site-operator conventions:

* spin-1/2 (onsite_op/ONSITE_SZ_SZBASIS_HB.c, ONSITE_SP_SZBASIS_HB.c): local state 0 = up
  (2Sz = +1), 1 = down; on-site term D_z Sz^2 + h_z Sz
  (main/dmrg/xxz_vf/src/main/MAKE_ONSITE_HAM.c:11-43);
* Hubbard (onsite_op/ONSITE_CUP_SZBASIS_HUBBARD.c, ONSITE_CDOWN_SZBASIS_HUBBARD.c): local
  states 0 empty, 1 up, 2 down, 3 up+down; on-site term h_z Sz + U n_up n_down + mu n
  (onsite_op/ONSITE_MAKE_HAM_SZBASIS_HUBBARD.c:5-26); hopping coefficient ``t`` enters as
  in the KLM driver (Model->t multiplies c^dagger c; t = -1 is the usual -|t| hopping).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from .abi import CRS1, Crs, dg_ed_model, dg_ed_term, ptr

ONSITE, INTER = 0, 1
SIGN_NONE, SIGN_SITE1, SIGN_SITE1_NEG, SIGN_RANGE, SIGN_RANGE_NEG = 0, 1, 2, 3, 4
ZERO = 1e-15


def dense_to_crs(M: np.ndarray) -> Crs:
    """Small dense site operator -> CRS keeping |v| > 1e-15 (as the onsite_op builders do)."""
    M = np.asarray(M, dtype=np.float64)
    rows, cols, vals = [0], [], []
    for r in range(M.shape[0]):
        for c in range(M.shape[1]):
            if abs(M[r, c]) > ZERO:
                cols.append(c)
                vals.append(M[r, c])
        rows.append(len(cols))
    return Crs(np.array(rows), np.array(cols, dtype=np.int32), np.array(vals), n=M.shape[0])


@dataclass
class EDModel:
    """A dg_ed_model with the numpy storage it points into."""
    n_sites: int
    dim_onsite: int
    qn1: np.ndarray
    qn2: np.ndarray
    use_qn1: bool
    use_qn2: bool
    target_qn1: int
    target_qn2: int
    ops: list
    terms: list
    n_ele: np.ndarray | None = None
    name: str = "model"
    _keep: list = field(default_factory=list, repr=False)

    def __post_init__(self):
        self.qn1 = np.ascontiguousarray(self.qn1, np.int32)
        self.qn2 = np.ascontiguousarray(self.qn2, np.int32)
        ops_arr = (CRS1 * len(self.ops))(*[o.struct for o in self.ops])
        terms_arr = (dg_ed_term * len(self.terms))(*[dg_ed_term(*t) for t in self.terms])
        ne = None if self.n_ele is None else np.ascontiguousarray(self.n_ele, np.int32)
        self.n_ele = ne
        self._keep = [ops_arr, terms_arr]
        self.struct = dg_ed_model(
            n_sites=self.n_sites, dim_onsite=self.dim_onsite, qn1=ptr(self.qn1, C.c_int), qn2=ptr(self.qn2, C.c_int),
            use_qn1=int(self.use_qn1), use_qn2=int(self.use_qn2), target_qn1=self.target_qn1,
            target_qn2=self.target_qn2, n_ops=len(self.ops), ops=C.cast(ops_arr, C.POINTER(CRS1)),
            n_terms=len(self.terms), terms=C.cast(terms_arr, C.POINTER(dg_ed_term)),
            n_ele=ptr(ne, C.c_int) if ne is not None else None)

    @property
    def dim_full(self) -> int:
        return self.dim_onsite ** self.n_sites


def xxz_chain(L: int, Jxy: float = 1.0, Jz: float = 1.0, hz: float = 0.0, Dz: float = 0.0, twoSz: int = 0,
              bc: str = "OBC") -> EDModel:
    """Spin-1/2 XXZ chain H = sum Jz Sz Sz + Jxy/2 (S+S- + S-S+) + sum (Dz Sz^2 + hz Sz)."""
    sz = np.diag([0.5, -0.5])
    onsite = np.diag([0.25 * Dz + 0.5 * hz, 0.25 * Dz + (-0.5) * hz])
    sp = np.array([[0.0, 1.0], [0.0, 0.0]])
    sm = sp.T.copy()
    zero = np.zeros((2, 2))
    ops = [dense_to_crs(onsite), dense_to_crs(sz), dense_to_crs(sp), dense_to_crs(sm),
           Crs(np.array([0, 1, 2]), np.array([0, 1], np.int32), np.array([0.0, 0.0]), n=2)]
    H, SZ, SP, SM, Z = 0, 1, 2, 3, 4
    del zero
    terms = []
    for s in range(L):
        terms.append((ONSITE, s, 0, H, 0, 1.0, SIGN_NONE))
    bonds = [(s, s + 1) for s in range(L - 1)] + ([(0, L - 1)] if bc == "PBC" else [])
    for a, b in bonds:
        terms.append((INTER, a, b, SZ, SZ, Jz, SIGN_NONE))
        terms.append((INTER, a, b, SP, SM, 0.5 * Jxy, SIGN_NONE))
        terms.append((INTER, a, b, SM, SP, 0.5 * Jxy, SIGN_NONE))
    terms.append((ONSITE, 0, 0, Z, 0, 0.0, SIGN_NONE))
    return EDModel(L, 2, qn1=np.zeros(2), qn2=np.array([1, -1]), use_qn1=False, use_qn2=True, target_qn1=0,
                   target_qn2=twoSz, ops=ops, terms=terms, name=f"xxz_L{L}")


def hubbard_chain(L: int, t: float = -1.0, U: float = 0.0, hz: float = 0.0, mu: float = 0.0, n_ele: int | None = None,
                  twoSz: int = 0, bc: str = "OBC") -> EDModel:
    """1D Hubbard chain H = t sum (c^dag_i c_i+1 + h.c.) + sum (U n_up n_dn + hz Sz + mu n)."""
    n_ele = L if n_ele is None else n_ele
    d = 4
    cup = np.zeros((d, d))
    cup[0, 1] = 1.0
    cup[2, 3] = 1.0
    cdn = np.zeros((d, d))
    cdn[0, 2] = 1.0
    cdn[1, 3] = -1.0
    # on-site: (h_z Szc + U NcNc) + mu N, summed in the order of ONSITE_MAKE_HAM_SZBASIS_HUBBARD
    szc = [0.0, 0.5, -0.5, 0.0]
    ncnc = [0.0, 0.0, 0.0, 1.0]
    nc = [0.0, 1.0, 1.0, 2.0]
    diag = []
    for k in range(d):
        a = szc[k] * hz
        b = ncnc[k] * U
        v = (a + b) if (abs(a) > ZERO and abs(b) > ZERO) else (a if abs(a) > ZERO else b)
        c = nc[k] * mu
        v = (v + c) if (abs(v) > ZERO and abs(c) > ZERO) else (v if abs(v) > ZERO else c)
        diag.append(v)
    ops = [dense_to_crs(np.diag(diag)), dense_to_crs(cup.T), dense_to_crs(cup), dense_to_crs(cdn.T), dense_to_crs(cdn),
           Crs(np.arange(d + 1), np.arange(d, dtype=np.int32), np.zeros(d), n=d)]
    H, CUPD, CUP, CDND, CDN, Z = range(6)
    terms = [(ONSITE, s, 0, H, 0, 1.0, SIGN_NONE) for s in range(L)]
    for s in range(L - 1):
        terms.append((INTER, s, s + 1, CUPD, CUP, t, SIGN_SITE1))
        terms.append((INTER, s, s + 1, CUP, CUPD, t, SIGN_SITE1_NEG))
        terms.append((INTER, s, s + 1, CDND, CDN, t, SIGN_SITE1))
        terms.append((INTER, s, s + 1, CDN, CDND, t, SIGN_SITE1_NEG))
    if bc == "PBC":
        terms.append((INTER, 0, L - 1, CUPD, CUP, t, SIGN_RANGE))
        terms.append((INTER, 0, L - 1, CUP, CUPD, t, SIGN_RANGE_NEG))
        terms.append((INTER, 0, L - 1, CDND, CDN, t, SIGN_RANGE))
        terms.append((INTER, 0, L - 1, CDN, CDND, t, SIGN_RANGE_NEG))
    terms.append((ONSITE, 0, 0, Z, 0, 0.0, SIGN_NONE))
    return EDModel(L, d, qn1=np.array([0, 1, 1, 2]), qn2=np.array([0, 1, -1, 0]), use_qn1=True, use_qn2=True,
                   target_qn1=n_ele, target_qn2=twoSz, ops=ops, terms=terms, n_ele=np.array([0, 1, 1, 2]),
                   name=f"hubbard_L{L}")


def klm_chain_from_tables(L: int, tables: list, n_ele: int, twoSz: int, t: float, I_z: float = 0.0, I_xy: float = 0.0,
                          bc: str = "OBC", spin_loc: int = 1) -> EDModel:
    """1D Kondo lattice with site operators given as (row, col, val) tables in the order
    Ham_On, SpL, SmL, SzL, CUp, CUp_D, CDown, CDown_D, Zero (the operator set of the
    reference's HAM_BOX), term order of main/exact_diag/klm_vf/src/MAKE_ELEMENT_HAM.c."""
    dim_spin = spin_loc + 1
    d = 4 * dim_spin
    ops = [Crs(r, c, v, n=d) for (r, c, v) in tables]
    HAM, SPL, SML, SZL, CUP, CUPD, CDN, CDND, Z = range(9)
    # local state = charge * dim_spin + spin; charge 0 empty, 1 up, 2 down, 3 up+down
    ele = np.array([[0, 1, 1, 2][k // dim_spin] for k in range(d)])
    sz_c = np.array([[0, 1, -1, 0][k // dim_spin] for k in range(d)])
    sz_l = np.array([spin_loc - 2 * (k % dim_spin) for k in range(d)])
    terms = [(ONSITE, s, 0, HAM, 0, 1.0, SIGN_NONE) for s in range(L)]
    bonds = [(s, s + 1) for s in range(L - 1)]
    for a, b in bonds:
        terms.append((INTER, a, b, SZL, SZL, I_z * 1.0, SIGN_NONE))
        terms.append((INTER, a, b, SPL, SML, 0.5 * I_xy * 1.0, SIGN_NONE))
        terms.append((INTER, a, b, SML, SPL, 0.5 * I_xy * 1.0, SIGN_NONE))
        terms.append((INTER, a, b, CUPD, CUP, t * 1.0, SIGN_SITE1))
        terms.append((INTER, a, b, CUP, CUPD, t * 1.0, SIGN_SITE1_NEG))
        terms.append((INTER, a, b, CDND, CDN, t * 1.0, SIGN_SITE1))
        terms.append((INTER, a, b, CDN, CDND, t * 1.0, SIGN_SITE1_NEG))
    if bc == "PBC":
        terms.append((INTER, 0, L - 1, SZL, SZL, I_z, SIGN_NONE))
        terms.append((INTER, 0, L - 1, SPL, SML, 0.5 * I_xy, SIGN_NONE))
        terms.append((INTER, 0, L - 1, SML, SPL, 0.5 * I_xy, SIGN_NONE))
        terms.append((INTER, 0, L - 1, CUPD, CUP, t, SIGN_RANGE))
        terms.append((INTER, 0, L - 1, CUP, CUPD, t, SIGN_RANGE_NEG))
        terms.append((INTER, 0, L - 1, CDND, CDN, t, SIGN_RANGE))
        terms.append((INTER, 0, L - 1, CDN, CDND, t, SIGN_RANGE_NEG))
    terms.append((ONSITE, 0, 0, Z, 0, 0.0, SIGN_NONE))
    return EDModel(L, d, qn1=ele, qn2=sz_c + sz_l, use_qn1=True, use_qn2=True, target_qn1=n_ele, target_qn2=twoSz,
                   ops=ops, terms=terms, n_ele=ele, name=f"klm_L{L}")


def free_fermion_energy(L: int, n_up: int, n_dn: int, t: float = -1.0) -> float:
    """OBC tight-binding ground-state energy: eps_k = 2 t cos(pi k/(L+1)), lowest n per spin."""
    eps = np.sort(2.0 * t * np.cos(np.pi * np.arange(1, L + 1) / (L + 1)))
    return float(eps[:n_up].sum() + eps[:n_dn].sum())
