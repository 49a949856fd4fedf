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


# ---------------------------------------------------------------------------------------
# Observables: block operators on a superblock whose sectors are all laid out (the inputs of
# DMRG_V_M_* and DMRG_EXPECTATION_*).
# ---------------------------------------------------------------------------------------
def sector_states(q_LL, q_RR, q_site, target):
    """States (LL, LR, RR, RL) of one sector in the reference's order (GET_BASIS_SUPERBLOCK then
    DMRG_QUICK_SORT_BASIS: by the label of LL+LR, then LL, LR, RR, RL), labels packed N*QN_SCALE+2Sz."""
    q_LL, q_RR, q_site = (np.asarray(a, np.int64) for a in (q_LL, q_RR, q_site))
    d = len(q_site)
    LL, LR, RR, RL = (x.ravel() for x in np.meshgrid(np.arange(len(q_LL)), np.arange(d), np.arange(len(q_RR)),
                                                     np.arange(d), indexing="ij"))
    k1 = q_LL[LL] + q_site[LR]
    keep = k1 + q_RR[RR] + q_site[RL] == target
    LL, LR, RR, RL, k1 = (x[keep] for x in (LL, LR, RR, RL, k1))
    order = np.lexsort((RL, RR, LR, LL, k1))
    return tuple(x[order].astype(np.int16) for x in (LL, LR, RR, RL))


@dataclass
class ObservableProblem:
    """Block labels, every sector of the superblock and the block operators of a few sites.

    ``inv`` is the whole Inv_LLLRRRRL table: each state's index inside its own sector (the
    DMRG_WHOLE_BASIS_Qk layout); ``inv_sector(q)`` is the single-sector table of a DMRG_BASIS.
    Operators: ``M_LL`` / ``M_RR`` conserve the block labels (site observables carried by the
    blocks), ``M_CF`` too (correlations inside LL), ``M_On`` is a site observable, and
    ``Cd_LL`` / ``Cd_On`` / ``Cd_RR`` raise the label by one up electron (c^dagger_up)."""
    q_LL: np.ndarray
    q_RR: np.ndarray
    q_site: np.ndarray
    ops: dict                      # name -> Crs or list of Crs
    target: int

    def __post_init__(self):
        self.d, self.dim_LL, self.dim_RR = len(self.q_site), len(self.q_LL), len(self.q_RR)
        k = (self.q_LL[:, None, None, None] + self.q_site[None, :, None, None] + self.q_RR[None, None, :, None]
             + self.q_site[None, None, None, :]).ravel()
        self.labels = np.unique(k)
        self.sectors = {int(t): sector_states(self.q_LL, self.q_RR, self.q_site, int(t)) for t in self.labels}
        self.inv = -np.ones(self.dim_LL * self.d * self.dim_RR * self.d, np.int32)
        for st in self.sectors.values():
            self.inv[self.sup(st)] = np.arange(len(st[0]), dtype=np.int32)
        self.ele = tuple(np.rint(np.asarray(a) / QN_SCALE).astype(np.int32) for a in (self.q_LL, self.q_site, self.q_RR))

    def sup(self, st):
        d, R = self.d, self.dim_RR
        return ((st[0].astype(np.int64) * d + st[1]) * R + st[2]) * d + st[3]

    def inv_sector(self, q):
        out = -np.ones_like(self.inv)
        st = self.sectors[q]
        out[self.sup(st)] = np.arange(len(st[0]), dtype=np.int32)
        return out

    def index(self, q, k):
        """Non-negative k-tuple naming sector q in a DMRG_WHOLE_BASIS_Qk: (rank of the label) for
        k = 1, (N - N_min, (2Sz - 2Sz_min) / 2) for k = 2, padded with zeros for k = 3, 4."""
        if k == 1:
            return (int(np.searchsorted(self.labels, q)),)
        N = np.rint(self.labels / QN_SCALE).astype(np.int64)
        sz = self.labels - N * QN_SCALE
        n, s = int(round(q / QN_SCALE)), q - int(round(q / QN_SCALE)) * QN_SCALE
        return (n - int(N.min()), (s - int(sz.min())) // 2) + (0,) * (k - 2)

    def shape(self, k):
        if k == 1:
            return (len(self.labels),)
        idx = [self.index(int(q), 2) for q in self.labels]
        return (max(i[0] for i in idx) + 1, max(i[1] for i in idx) + 1) + (1,) * (k - 2)

    def whole_basis(self, k):
        from .abi import WholeBasis
        return WholeBasis({self.index(q, k): st for q, st in self.sectors.items()}, self.shape(k), self.inv, self.dim_RR,
                          self.d)

    def arrays(self) -> dict:
        """Flat arrays (labels, target and every operator's CRS) for a fixture."""
        out = dict(q_LL=self.q_LL, q_RR=self.q_RR, q_site=self.q_site, target=np.int64(self.target))
        for name, o in self.ops.items():
            for i, c in enumerate(o if isinstance(o, list) else [o]):
                out[f"op_{name}_{i}_row"], out[f"op_{name}_{i}_col"], out[f"op_{name}_{i}_val"] = c.row, c.col[:c.nnz], c.val[:c.nnz]
        return out

    @classmethod
    def from_arrays(cls, a) -> "ObservableProblem":
        ops = {}
        for key in sorted(k for k in a.keys() if k.startswith("op_") and k.endswith("_row")):
            _, name, i, _ = key.split("_")
            c = Crs(a[key], a[f"op_{name}_{i}_col"], a[f"op_{name}_{i}_val"])
            ops.setdefault(name, {})[int(i)] = c
        ops = {n: (v[0] if n in ("On", "CdOn") else [v[i] for i in sorted(v)]) for n, v in ops.items()}
        return cls(np.asarray(a["q_LL"]), np.asarray(a["q_RR"]), np.asarray(a["q_site"]), ops, int(a["target"]))


def random_observable_problem(dim_LL=16, dim_RR=14, n_LL=3, n_RR=3, per_row=4, seed=0, n_sites=5) -> ObservableProblem:
    """Hubbard-type blocks (labels of n_sites sites) with seeded random block operators; the
    target is the half-filled Sz = 0 sector of 2 n_sites + 2 sites."""
    rng = np.random.default_rng(seed)
    from .workloads import _block_labels, hubbard_site_labels
    qL = _block_labels(dim_LL, n_sites, n_sites, 1.0, 0.9, seed + 1)
    qR = _block_labels(dim_RR, n_sites, n_sites, 1.0, 0.9, seed + 2)
    qs = hubbard_site_labels()
    up = QN_SCALE + 1
    cupd = np.zeros((4, 4))
    cupd[0, 1] = 1.0
    cupd[2, 3] = 1.0
    ops = dict(LL=[_crs(_random_sym_op(qL, per_row, rng)) for _ in range(n_LL)],
               RR=[_crs(_random_sym_op(qR, per_row, rng)) for _ in range(n_RR)],
               CF=[_crs(_random_sym_op(qL, per_row, rng)) for _ in range(n_LL)],
               On=_crs(sp.csr_matrix(np.diag(rng.standard_normal(4)))),
               CdLL=[_crs(_random_shift_op(qL, up, per_row, rng))],
               CdRR=[_crs(_random_shift_op(qR, up, per_row, rng))],
               CdOn=_crs(sp.csr_matrix(cupd)))
    return ObservableProblem(qL, qR, qs, ops, (2 * n_sites + 2) * QN_SCALE)


# ---------------------------------------------------------------------------------------
# Superblocks recorded from the reference's own DMRG runs
# ---------------------------------------------------------------------------------------
@dataclass
class DmrgSuperblock:
    """One superblock of a reference DMRG run: the term list (``model``) and what the reference's
    solve returned for it (``gs_val``, ``gs_error``, ``gs_vec``), with the dg64 checksums of the
    reference's lower-triangle CRS (``crs_dg64``: Row, Col, Val) and its stored element count."""
    name: str
    model: SBModel
    sweep: int
    LL_site: int
    RR_site: int
    nnz: int
    crs_dg64: tuple
    gs_val: float
    gs_error: float
    gs_vec: np.ndarray


def load_dmrg_superblock(path) -> DmrgSuperblock:
    """Term list and reference results from a ``dmrg_<model>_sweep<k>.npz`` file (written by
    the fixture generator that runs main/dmrg/<model>; the terms are in the order the model's
    MAKE_ELEMENT_HAM_LLLRRRRL applies them, e.g. main/dmrg/hubbard_vf/src/main/
    MAKE_ELEMENT_HAM_LLLRRRRL.c:16-45)."""
    z = np.load(path)
    n, d, dim_LL, dim_RR = int(z["n"]), int(z["dim_onsite"]), int(z["dim_LL"]), int(z["dim_RR"])
    LL, LR, RR, RL = (np.ascontiguousarray(z["states"][k]) for k in range(4))
    inv = -np.ones(dim_LL * d * dim_RR * d, np.int32)
    sup = ((LL.astype(np.int64) * d + LR) * dim_RR + RR) * d + RL
    inv[sup] = np.arange(n, dtype=np.int32)
    ops = [Crs(z[f"op{k}_row"], z[f"op{k}_col"], z[f"op{k}_val"]) for k in range(int(z["n_ops"]))]
    ti, tc = z["term_int"], z["term_coef"]
    terms = [(int(a[0]), int(a[1]), int(a[2]), int(a[3]), float(c), int(a[4]), int(a[5])) for a, c in zip(ti, tc)]
    ele = [np.asarray(z[f"ele{p}"]) if f"ele{p}" in z.files else None for p in range(4)]
    model = SBModel(n, dim_LL, dim_RR, d, LL, LR, RR, RL, inv, ops, terms, ele)
    name = f"{z['model']} sweep {int(z['sweep'])} ({int(z['LL_site']) + 1},1,1,{int(z['RR_site']) + 1})"
    return DmrgSuperblock(name, model, int(z["sweep"]), int(z["LL_site"]), int(z["RR_site"]), int(z["nnz"]),
                          (np.uint64(z["row_dg64"]), np.uint64(z["col_dg64"]), np.uint64(z["val_dg64"])),
                          float(z["gs_val"]), float(z["gs_error"]), np.asarray(z["gs_vec"], np.float64))
