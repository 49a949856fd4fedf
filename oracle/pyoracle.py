"""ctypes front end of the checker libraries.

TEST INFRASTRUCTURE ONLY (imported by tests/, __graft_entry__.smoke() and the CPU-baseline
leg of bench.py).  Two libraries:

* ``liboracle.so``: the project's CPU restatement of the hot path (oracle.c);
* ``_ref/libdmrg_ref.so``: the reference's own C sources compiled where they lie (only
  where the reference tree is present; see the Makefile).  Its functions print progress
  and append to ./SML_out/, so calls into it run inside a scratch working directory.
"""
from __future__ import annotations

import contextlib
import ctypes as C
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

from dmrg_c_gb300 import abi
from dmrg_c_gb300.abi import (BOX_CG, BOX_II, BOX_LAN, CRS1, DMRG_BASIS, EXACT_BASIS_INFO, MODEL_1DKLM_VF, dg_ed_model, ptr)

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libdmrg_ref.so"
REF_SRC = Path(os.environ.get("DMRG_REF", "/root/reference"))

P = C.POINTER
dp, ip, lp = P(C.c_double), P(C.c_int), P(C.c_long)


class or_lanczos_cfg(C.Structure):
    _fields_ = [("acc", C.c_double), ("min_step", C.c_int), ("max_step", C.c_int), ("max_block_step", C.c_int),
                ("tight", C.c_int), ("slow", C.c_int), ("guess", C.c_int), ("seed", C.c_ulonglong),
                ("dense_below", C.c_int), ("threads", C.c_int)]


class or_lanczos_out(C.Structure):
    _fields_ = [("eig_val", C.c_double), ("steps", C.c_int), ("converged", C.c_int), ("dense", C.c_int),
                ("spmv", C.c_int)]


class or_ii_cfg(C.Structure):
    _fields_ = [("ii_acc", C.c_double), ("ii_diag_add", C.c_double), ("ii_max_step", C.c_int), ("cg_acc", C.c_double),
                ("cg_max_step", C.c_int), ("minres", C.c_int), ("threads", C.c_int)]


class or_ii_out(C.Structure):
    _fields_ = [("error", C.c_double), ("iters", C.c_int), ("cg_total", C.c_int), ("converged", C.c_int),
                ("spmv", C.c_int)]


class or_obc(C.Structure):
    _fields_ = [("M_LLLR", P(CRS1)), ("M_LRRL", P(CRS1)), ("M_LRRL_Sign", P(CRS1)), ("M_RRRL", P(CRS1)),
                ("Ele_RR", ip), ("Basis", P(DMRG_BASIS))]


_lib = None
_ref = None


def build_oracle() -> None:
    subprocess.run(["make", "-s", "-C", str(HERE), "oracle"], check=True)


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists() or LIB.stat().st_mtime < (HERE / "oracle.c").stat().st_mtime:
            build_oracle()
        lib = C.CDLL(str(LIB))
        sig = {
            "or_spmv": (C.c_int, [P(CRS1), C.c_int, dp, dp, C.c_int]),
            "or_tridiag_eig": (C.c_int, [dp, dp, C.c_int, dp, dp]),
            "or_dense_lowest": (C.c_int, [dp, C.c_int, dp, dp]),
            "or_lanczos": (C.c_int, [P(CRS1), C.c_int, P(or_lanczos_cfg), dp, P(or_lanczos_out)]),
            "or_inverse_iteration": (C.c_int, [P(CRS1), C.c_int, P(or_ii_cfg), C.c_double, dp, P(or_ii_out)]),
            "or_cg": (C.c_int, [P(CRS1), C.c_int, C.c_double, dp, dp, C.c_double, C.c_int, C.c_int, ip, ip]),
            "or_minres": (C.c_int, [P(CRS1), C.c_int, C.c_double, dp, dp, C.c_double, C.c_int, C.c_int, ip, ip]),
            "or_converge_check": (C.c_double, [P(CRS1), C.c_int, dp, C.c_double, C.c_int]),
            "or_obc_spmv": (C.c_int, [P(or_obc), dp, dp, C.c_int]),
            "or_obc_lanczos_slow": (C.c_int, [P(or_obc), P(or_lanczos_cfg), dp, P(or_lanczos_out)]),
            "or_obc_inverse_iteration": (C.c_int, [P(or_obc), P(or_ii_cfg), C.c_double, dp, P(or_ii_out)]),
            "or_obc_cg": (C.c_int, [P(or_obc), C.c_double, dp, dp, C.c_double, C.c_int, C.c_int, ip, ip]),
            "or_ed_dim": (C.c_long, [P(dg_ed_model), C.c_int]),
            "or_ed_basis": (C.c_int, [P(dg_ed_model), lp, C.c_long, C.c_int]),
            "or_ed_count": (C.c_int, [P(dg_ed_model), lp, C.c_long, lp, C.c_int]),
            "or_ed_fill": (C.c_int, [P(dg_ed_model), lp, C.c_long, lp, ip, dp, C.c_int]),
            "or_site_apply": (C.c_int, [P(CRS1), lp, C.c_long, lp, C.c_long, C.c_int, C.c_int, ip, dp, dp, C.c_int]),
            "or_sb_count": (C.c_int, [P(abi.dg_sb_model), lp, C.c_int]),
            "or_sb_fill": (C.c_int, [P(abi.dg_sb_model), lp, ip, dp, C.c_int]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype, f.argtypes = res, args
        _lib = lib
    return _lib


def threads_default() -> int:
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


# ---------------------------------------------------------------------------------------
# oracle (restatement)
# ---------------------------------------------------------------------------------------
def spmv(crs: abi.Crs, x: np.ndarray, sym: bool, threads: int | None = None) -> np.ndarray:
    y = np.empty(crs.n)
    x = np.ascontiguousarray(x, np.float64)
    assert load().or_spmv(crs.ref, int(sym), ptr(x, C.c_double), ptr(y, C.c_double), threads or threads_default()) == 0
    return y


def tridiag_eig(d, e, vectors=True):
    d = np.ascontiguousarray(d, np.float64)
    e = np.ascontiguousarray(e, np.float64)
    n = len(d)
    w = np.empty(n)
    z = np.empty(n * n) if vectors else None
    rc = load().or_tridiag_eig(ptr(d, C.c_double), ptr(e, C.c_double), n, ptr(w, C.c_double),
                               ptr(z, C.c_double) if vectors else None)
    assert rc == 0
    return (w, z.reshape(n, n).T) if vectors else w     # columns = eigenvectors


def lanczos(crs: abi.Crs, sym: bool, guess=None, acc=1e-14, min_step=1, max_step=800, max_block_step=None, tight=False,
            slow=False, seed=0, dense_below=1000, threads=None):
    cfg = or_lanczos_cfg(acc=acc, min_step=min_step, max_step=max_step,
                         max_block_step=max_step if max_block_step is None else max_block_step, tight=int(tight),
                         slow=int(slow), guess=int(guess is not None), seed=seed, dense_below=dense_below,
                         threads=threads or threads_default())
    v = np.array(guess, dtype=np.float64) if guess is not None else np.zeros(crs.n)
    out = or_lanczos_out()
    rc = load().or_lanczos(crs.ref, int(sym), C.byref(cfg), ptr(v, C.c_double), C.byref(out))
    return rc, out, v


def inverse_iteration(crs, sym, eig_val, vec, ii_acc=1e-9, ii_diag_add=1e-11, ii_max_step=3, cg_acc=1e-7,
                      cg_max_step=1000, minres=False, threads=None):
    cfg = or_ii_cfg(ii_acc=ii_acc, ii_diag_add=ii_diag_add, ii_max_step=ii_max_step, cg_acc=cg_acc,
                    cg_max_step=cg_max_step, minres=int(minres), threads=threads or threads_default())
    v = np.array(vec, dtype=np.float64)
    out = or_ii_out()
    rc = load().or_inverse_iteration(crs.ref, int(sym), C.byref(cfg), eig_val, ptr(v, C.c_double), C.byref(out))
    return rc, out, v


def linear_solve(crs, sym, b, x0, sigma=0.0, acc=1e-7, max_step=1000, minres=False, threads=None):
    b = np.ascontiguousarray(b, np.float64)
    x = np.array(x0, dtype=np.float64)
    it, cv = C.c_int(), C.c_int()
    f = load().or_minres if minres else load().or_cg
    rc = f(crs.ref, int(sym), sigma, ptr(b, C.c_double), ptr(x, C.c_double), acc, max_step,
           threads or threads_default(), C.byref(it), C.byref(cv))
    return rc, it.value, bool(cv.value), x


def converge_check(crs, sym, x, lam, threads=None) -> float:
    x = np.ascontiguousarray(x, np.float64)
    return load().or_converge_check(crs.ref, int(sym), ptr(x, C.c_double), lam, threads or threads_default())


def ed_build(model, threads=None):
    """Basis and full CRS (row, col, val) of an ED model (see dmrg_c_gb300.ed_models)."""
    th = threads or threads_default()
    lib = load()
    m = C.byref(model.struct)
    dim = lib.or_ed_dim(m, th)
    basis = np.empty(dim, np.int64)
    assert lib.or_ed_basis(m, ptr(basis, C.c_long), dim, th) == 0
    row = np.zeros(dim + 1, np.int64)
    assert lib.or_ed_count(m, ptr(basis, C.c_long), dim, ptr(row, C.c_long), th) == 0
    col = np.empty(max(row[-1], 1), np.int32)
    val = np.empty(max(row[-1], 1), np.float64)
    assert lib.or_ed_fill(m, ptr(basis, C.c_long), dim, ptr(row, C.c_long), ptr(col, C.c_int), ptr(val, C.c_double),
                          th) == 0
    return basis, row, col[:row[-1]], val[:row[-1]]


def sb_build(model, threads=None):
    """Superblock lower-triangle CRS (row, col, val) of a dmrg_c_gb300.sb_models.SBModel."""
    th = threads or threads_default()
    lib = load()
    n = model.n
    row = np.zeros(n + 1, np.int64)
    assert lib.or_sb_count(C.byref(model.struct), ptr(row, C.c_long), th) == 0
    col = np.empty(max(row[-1], 1), np.int32)
    val = np.empty(max(row[-1], 1), np.float64)
    assert lib.or_sb_fill(C.byref(model.struct), ptr(row, C.c_long), ptr(col, C.c_int), ptr(val, C.c_double), th) == 0
    return row, col[:row[-1]], val[:row[-1]]


def dg64(a: np.ndarray) -> np.uint64:
    """Checksum of an array's bytes shared with ref_dmrg_dump.c: the bytes as little-endian 64-bit
    words (the last zero-padded), word i contributing mix64(w_i + (i + 1) * 0x9E3779B97F4A7C15)
    (the splitmix64 finaliser), summed modulo 2**64."""
    b = np.ascontiguousarray(a).view(np.uint8).ravel()
    pad = (-len(b)) % 8
    if pad:
        b = np.concatenate([b, np.zeros(pad, np.uint8)])
    w = b.view("<u8").astype(np.uint64)
    with np.errstate(over="ignore"):
        z = w + (np.arange(1, len(w) + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
        return np.uint64(np.sum(z, dtype=np.uint64))


def ref_sb_build(model, cap=None):
    """The same through the reference's own DMRG_MAKE_ELEM_*_LLLRRRRL builders (oracle/_ref)."""
    lib = load_ref()
    lib.ref_sb_build.restype = C.c_int
    lib.ref_sb_build.argtypes = [P(abi.dg_sb_model), lp, ip, dp, C.c_long]
    n = model.n
    cap = cap or n * 64
    row = np.zeros(n + 1, np.int64)
    col = np.empty(cap, np.int32)
    val = np.empty(cap, np.float64)
    rc = lib.ref_sb_build(C.byref(model.struct), ptr(row, C.c_long), ptr(col, C.c_int), ptr(val, C.c_double), cap)
    assert rc == 0, rc
    return row, col[:row[-1]].copy(), val[:row[-1]].copy()


def sb_basis(dim_LL, dim_RR, d, qn1, qn2, targets):
    """Superblock basis restated with numpy (GET_BASIS_SUPERBLOCK + DMRG_QUICK_SORT_BASIS_Q1/Q2):
    qn1 = (LL, RR, site) quantum-number arrays, qn2 the same or None; states ordered by
    (qn1 of LL+LR, qn2 of LL+LR, LL, LR, RR, RL).  Returns (LL, LR, RR, RL, inv)."""
    LL, LR, RR, RL = (x.ravel() for x in np.meshgrid(np.arange(dim_LL), np.arange(d), np.arange(dim_RR), np.arange(d),
                                                     indexing="ij"))
    q = [np.asarray(a, np.int64) for a in qn1]
    keep = q[0][LL] + q[2][LR] + q[1][RR] + q[2][RL] == targets[0]
    k1 = q[0][LL] + q[2][LR]
    k2 = np.zeros_like(k1)
    if qn2 is not None:
        r = [np.asarray(a, np.int64) for a in qn2]
        keep &= r[0][LL] + r[2][LR] + r[1][RR] + r[2][RL] == targets[1]
        k2 = r[0][LL] + r[2][LR]
    LL, LR, RR, RL, k1, k2 = (x[keep] for x in (LL, LR, RR, RL, k1, k2))
    order = np.lexsort((RL, RR, LR, LL, k2, k1))   # primary key last
    LL, LR, RR, RL = (x[order].astype(np.int16) for x in (LL, LR, RR, RL))
    inv = -np.ones(dim_LL * d * dim_RR * d, np.int32)
    inv[((LL.astype(np.int64) * d + LR) * dim_RR + RR) * d + RL] = np.arange(len(LL), dtype=np.int32)
    return LL, LR, RR, RL, inv


def ref_sb_basis(dim_LL, dim_RR, d, qn1, qn2, targets):
    """The same with the reference's own DMRG_QUICK_SORT_BASIS_Q1 / _Q2 ordering (oracle/_ref)."""
    lib = load_ref()
    sp, ip_ = P(C.c_short), P(C.c_int)
    lib.ref_sb_basis.restype = C.c_int
    lib.ref_sb_basis.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int] + [ip_] * 6 + [C.c_int, C.c_int] + [sp] * 4 + [ip_, C.c_int]
    arr = lambda a: np.ascontiguousarray(a, np.int32)   # noqa: E731
    q1 = [arr(a) for a in qn1]
    q2 = [arr(a) for a in qn2] if qn2 is not None else [None] * 3
    cap = dim_LL * d * dim_RR * d
    st = [np.empty(cap, np.int16) for _ in range(4)]
    inv = np.empty(cap, np.int32)
    n = lib.ref_sb_basis(dim_LL, dim_RR, d, 2 if qn2 is not None else 1, *(ptr(a, C.c_int) if a is not None else None for a in q1 + q2),
                         int(targets[0]), int(targets[1]) if qn2 is not None else 0, *(ptr(a, C.c_short) for a in st),
                         ptr(inv, C.c_int), cap)
    assert n > 0, n
    return (*(a[:n].copy() for a in st), inv)


SB_LL, SB_LR, SB_RR, SB_RL = 0, 1, 2, 3
SB_NAMES = ("LL", "LR", "RR", "RL")


def sb_vm(states, inv, dim_RR, d, op: abi.Crs, pos, v, ele=None):
    """Block operator on one sector's superblock states, restated with numpy from DMRG_V_M_<pos>_Q*
    (dmrg/DMRG_V_M_LL_Q0.c:13-28, dmrg/DMRG_V_M_LR_Q1.c:23-52, dmrg/DMRG_V_M_RR_Q2.c:23-52): for
    state i the sum over the operator row of its pos coordinate, in storage order, of
    (sign_i * v[Inv(i with that coordinate set to the column)]) * value, Inv = -1 entries skipped;
    sign_i = (-1)^(electrons at the positions before pos) when ele = (ele_LL, ele_LR, ele_RR) is
    given (Sign_Flag "Yes").  Each step is rounded as the reference's loop rounds it."""
    c = [np.asarray(a, np.int64) for a in states]
    n = len(c[0])
    strides = [d * dim_RR * d, dim_RR * d, d, 1]
    full = ((c[0] * d + c[1]) * dim_RR + c[2]) * d + c[3]
    s = c[pos]
    base = full - s * strides[pos]
    sgn = np.ones(n)
    if ele is not None and pos != SB_LL:
        ne = np.asarray(ele[0], np.int64)[c[0]]
        if pos >= SB_RR:
            ne = ne + np.asarray(ele[1], np.int64)[c[1]]
        if pos >= SB_RL:
            ne = ne + np.asarray(ele[2], np.int64)[c[2]]
        sgn = np.where(ne % 2 == 0, 1.0, -1.0)
    v = np.asarray(v, np.float64)
    start = op.row[s]
    length = op.row[s + 1] - start
    acc = np.zeros(n)
    for k in range(int(length.max()) if n else 0):
        live = np.flatnonzero(length > k)
        idx = start[live] + k
        j = inv[base[live] + op.col[idx].astype(np.int64) * strides[pos]]
        ok = j >= 0
        li = live[ok]
        acc[li] = acc[li] + (sgn[li] * v[j[ok]]) * op.val[idx[ok]]
    return acc


def sb_expect(states, inv, dim_RR, d, terms, v, weights, ele=None):
    """<w|O|v> for each term (op, pos, weight index) over one sector: the sb_vm product dotted
    with weights[weight] (DMRG_EXPECTATION_ONSITE.c:12-29 is V_M then INNER_PRODUCT per site)."""
    return np.array([float(np.dot(weights[w], sb_vm(states, inv, dim_RR, d, op, pos, v, ele))) for op, pos, w in terms])


def _crs_array(ops):
    arr = (P(CRS1) * max(len(ops), 1))(*[o.ref for o in ops])
    return arr


def _q0_basis(states, inv, dim_LL, dim_RR, d):
    st = [np.ascontiguousarray(a, np.int16) for a in states]
    inv = np.ascontiguousarray(inv, np.int32)
    B = DMRG_BASIS(LL_LLLRRRRL=ptr(st[0], C.c_short), LR_LLLRRRRL=ptr(st[1], C.c_short), RR_LLLRRRRL=ptr(st[2], C.c_short),
                   RL_LLLRRRRL=ptr(st[3], C.c_short), Inv_LLLRRRRL=ptr(inv, C.c_int), dim_LLLRRRRL=len(st[0]),
                   dim_LL=dim_LL, dim_RR=dim_RR, dim_onsite=d)
    return B, (st, inv)


def call_vm_q0(lib, states, inv, dim_LL, dim_RR, d, op: abi.Crs, pos, v):
    """DMRG_V_M_<pos>_Q0 of lib (the reference build or libdmrg_gb300) on host arrays."""
    B, keep = _q0_basis(states, inv, dim_LL, dim_RR, d)
    v = np.ascontiguousarray(v, np.float64)
    out = np.full(len(states[0]), np.nan)
    getattr(lib, f"DMRG_V_M_{SB_NAMES[pos]}_Q0")(op.ref, ptr(v, C.c_double), ptr(out, C.c_double), len(out), 1, C.byref(B))
    return out


def call_vm_whole(lib, wb, q, op: abi.Crs, pos, v, ele=None, sign=False):
    """DMRG_V_M_<pos>_Q<k> of lib on a whole basis (abi.WholeBasis) for output sector q (a k-tuple)."""
    k = len(q)
    v = np.ascontiguousarray(v, np.float64)
    dim = wb.struct.Dim
    for i in q:
        dim = dim[i]
    out = np.full(int(dim), np.nan)
    e = [np.ascontiguousarray(a, np.int32) if a is not None else None for a in (ele or (None, None, None))]
    ep = [ptr(a, C.c_int) if a is not None else None for a in e]
    flag = b"Yes" if sign else b"No"
    args = [op.ref, *[C.c_int(i) for i in q], ptr(v, C.c_double)]
    if pos == SB_LR:
        args += [ep[0], flag]
    elif pos == SB_RR:
        args += [ep[0], ep[1], flag]
    elif pos == SB_RL:
        args += [ep[0], ep[1], ep[2], flag]
    args += [ptr(out, C.c_double), C.c_int(1), wb.ref]
    getattr(lib, f"DMRG_V_M_{SB_NAMES[pos]}_Q{k}")(*args)
    return out


def call_expectation_onsite(lib, states, inv, dim_LL, dim_RR, d, M_LL, M_On, M_RR, v):
    """DMRG_EXPECTATION_ONSITE of lib: returns (Out, Temp_V)."""
    B, keep = _q0_basis(states, inv, dim_LL, dim_RR, d)
    S = abi.DMRG_STATUS(LL_site=len(M_LL) - 1, RR_site=len(M_RR) - 1, dim_LLLRRRRL=len(states[0]))
    v = np.ascontiguousarray(v, np.float64)
    out = np.full(len(M_LL) + len(M_RR) + 2, np.nan)
    temp = np.full(len(v), np.nan)
    lib.DMRG_EXPECTATION_ONSITE(_crs_array(M_LL), M_On.ref, _crs_array(M_RR), ptr(out, C.c_double), ptr(v, C.c_double),
                                ptr(temp, C.c_double), 1, C.byref(B), C.byref(S))
    return out, temp


def call_expectation_intersite_q0(lib, states, inv, dim_LL, dim_RR, d, M_CF, M_LL, M_On, M_RR, origin, v):
    """DMRG_EXPECTATION_INTERSITE_Q0 of lib: returns (Out, Temp_V1, Temp_V2)."""
    B, keep = _q0_basis(states, inv, dim_LL, dim_RR, d)
    LL_site, RR_site = len(M_LL) - 1, len(M_RR) - 1
    S = abi.DMRG_STATUS(LL_site=LL_site, RR_site=RR_site, dim_LLLRRRRL=len(states[0]))
    v = np.ascontiguousarray(v, np.float64)
    out = np.full(LL_site + RR_site + 4, np.nan)
    t1, t2 = np.full(len(v), np.nan), np.full(len(v), np.nan)
    lib.DMRG_EXPECTATION_INTERSITE_Q0(_crs_array(M_CF), _crs_array(M_LL), M_On.ref, _crs_array(M_RR), ptr(out, C.c_double),
                                      origin, ptr(v, C.c_double), ptr(t1, C.c_double), ptr(t2, C.c_double), 1, C.byref(B),
                                      C.byref(S))
    return out, t1, t2


def lllr_list(q_LL, q_site, states):
    """The DMRG_BASIS LLLR list of a sector in the reference's order: every (LL, LR) pair sorted by
    the label of LL+LR (then LL, LR), the number of superblock states of each pair (Sum_LLLR), the
    pair labels and the block sizes of DMRG_GET_DENSITY_MATRIX_INFO_Q1 (runs of equal labels)."""
    q_LL, q_site = np.asarray(q_LL, np.int64), np.asarray(q_site, np.int64)
    d = len(q_site)
    LL, LR = (x.ravel() for x in np.meshgrid(np.arange(len(q_LL)), np.arange(d), indexing="ij"))
    lab = q_LL[LL] + q_site[LR]
    order = np.lexsort((LR, LL, lab))
    LL, LR, lab = LL[order], LR[order], lab[order]
    cnt = np.zeros(len(q_LL) * d, np.int64)
    np.add.at(cnt, np.asarray(states[0], np.int64) * d + np.asarray(states[1], np.int64), 1)
    sums = cnt[LL * d + LR].astype(np.int32)
    _, dim_block = np.unique(lab, return_counts=True)
    return LL.astype(np.int16), LR.astype(np.int16), sums, lab, dim_block.astype(np.int32)


def density_matrix_blocks(states, inv, d, dim_RR, v, lllr):
    """DMRG_GET_DENSITY_MATRIX restated for every block (dmrg/DMRG_GET_DENSITY_MATRIX.c:36-100):
    M[row][col] = sum over the row pair's states t of v[state t of row] * v[state t of col], the
    sum taken in t order and rounded as written.  lllr = lllr_list(...)."""
    LLl, LRl, sums, _, dim_block = lllr
    base = np.concatenate([[0], np.cumsum(sums)])
    out, b0 = [], 0
    for dim in dim_block:
        rows = np.arange(b0, b0 + dim)
        Q = int(sums[b0])
        X = np.zeros((dim, Q))
        for t in range(Q):
            s = base[rows] + t
            sup = ((LLl[rows].astype(np.int64) * d + LRl[rows]) * dim_RR + states[2][s]) * d + states[3][s]
            X[:, t] = v[inv[sup]]
        M = np.zeros((dim, dim))
        for t in range(Q):
            M = M + X[:, t, None] * X[None, :, t]
        out.append(M)
        b0 += dim
    return out


def call_density_matrix(lib, states, inv, dim_LL, dim_RR, d, v, lllr, free):
    """DMRG_GET_DENSITY_MATRIX of lib for every block; free(ptr) releases a row / the row array."""
    LLl, LRl, sums, _, dim_block = lllr
    st = [np.ascontiguousarray(a, np.int16) for a in states]
    inv = np.ascontiguousarray(inv, np.int32)
    LLl, LRl, sums, dim_block = (np.ascontiguousarray(a) for a in (LLl, LRl, sums, dim_block))
    B = DMRG_BASIS(LL_LLLRRRRL=ptr(st[0], C.c_short), LR_LLLRRRRL=ptr(st[1], C.c_short), RR_LLLRRRRL=ptr(st[2], C.c_short),
                   RL_LLLRRRRL=ptr(st[3], C.c_short), Inv_LLLRRRRL=ptr(inv, C.c_int), dim_LLLRRRRL=len(st[0]), dim_LL=dim_LL,
                   dim_RR=dim_RR, dim_onsite=d, LL_LLLR=ptr(LLl, C.c_short), LR_LLLR=ptr(LRl, C.c_short), dim_LLLR=len(LLl),
                   Sum_LLLR=ptr(sums, C.c_int))
    v = np.ascontiguousarray(v, np.float64)
    fn = lib.DMRG_GET_DENSITY_MATRIX
    fn.restype = P(dp)
    out = []
    for blk, dim in enumerate(dim_block):
        M = fn(blk, ptr(dim_block, C.c_int), C.byref(B), ptr(v, C.c_double), 1)
        out.append(np.array([[M[r][c] for c in range(dim)] for r in range(dim)]).reshape(dim, dim))
        for r in range(dim):
            free(C.cast(M[r], C.c_void_p))
        free(C.cast(M, C.c_void_p))
    return out


def system_info(qns, states, inv, d, dim_RR, v, lllr, max_dim):
    """DMRG_GET_SYSTEM_INFO_Q<k> restated (dmrg/DMRG_GET_SYSTEM_INFO_Q1.c:8-213): the density
    blocks (density_matrix_blocks), numpy's symmetric eigensolver in place of LAPACK's dsyev
    (ascending values), a stable descending sort of all eigenvalues, the cut (max_dim, no cut
    inside a degenerate multiplet, nothing at or below 1e-15), a stable sort of the kept states by
    the quantum numbers qns (a list of per-pair arrays, primary first).  Returns a dict."""
    blocks = density_matrix_blocks(states, inv, d, dim_RR, v, lllr)
    dim_block = lllr[4]
    starts = np.concatenate([[0], np.cumsum(dim_block)])
    vals, vecs = zip(*[np.linalg.eigh(M) if len(M) else (np.zeros(0), np.zeros((0, 0))) for M in blocks])
    items = [(g, i) for g in range(len(blocks)) for i in range(len(blocks[g]))]
    order = sorted(range(len(items)), key=lambda e: -vals[items[e][0]][items[e][1]])   # stable
    val = np.array([vals[items[e][0]][items[e][1]] for e in order])
    dim_LLLR = len(val)
    zero = 1e-15
    dim_renorm = 0
    if dim_LLLR <= max_dim:
        for i in range(dim_LLLR, 0, -1):
            if val[i - 1] > zero:
                dim_renorm = i
                break
    else:
        for i in range(max_dim, 0, -1):
            if abs(val[i - 1] - val[i]) > zero and val[i - 1] > zero:
                dim_renorm = i
                break
    # per block: the distance between its kept and its dropped eigenvalues, and its norm (the kept
    # subspace of a block is determined to about 1e-16 * norm / gap)
    kept_set = set(order[:dim_renorm])
    gaps = {}
    for g in range(len(blocks)):
        if len(blocks[g]) == 0:
            continue
        es = [e for e in range(len(items)) if items[e][0] == g]
        kv = [vals[g][items[e][1]] for e in es if e in kept_set]
        dv = [vals[g][items[e][1]] for e in es if e not in kept_set]
        gap = min((abs(a - b) for a in kv for b in dv), default=np.inf)
        gaps[int(starts[g])] = (gap, float(np.abs(vals[g]).max()))
    kept = sorted(order[:dim_renorm], key=lambda e: tuple(int(q[starts[items[e][0]]]) for q in qns))
    cols, rows, qn_out = [], [], [[] for _ in qns]
    for e in kept:
        g, i = items[e]
        cols.append(vecs[g][:, i])
        rows.append(np.arange(starts[g], starts[g + 1]))
        for k, q in enumerate(qns):
            qn_out[k].append(int(q[starts[g]]))
    return dict(dim_renorm=dim_renorm, val=val, sum_val=float(np.sum(val)), tr_error=float(np.sum(val) - np.sum(val[:dim_renorm])),
                gaps=gaps,
                qn=[np.array(x, np.int32) for x in qn_out], col_ptr=np.concatenate([[0], np.cumsum([len(r) for r in rows])]),
                rows=np.concatenate(rows) if rows else np.zeros(0, int), vals=np.concatenate(cols) if cols else np.zeros(0))


def call_system_info(lib, qns, states, inv, dim_LL, dim_RR, d, v, lllr, max_dim, free):
    """DMRG_GET_SYSTEM_INFO_Q<len(qns)> of lib; returns the dict of system_info and releases the
    structure as DMRG_FREE_SYSTEM_INFO does (free(ptr) on every array)."""
    LLl, LRl, sums, _, dim_block = lllr
    st = [np.ascontiguousarray(a, np.int16) for a in states]
    inv = np.ascontiguousarray(inv, np.int32)
    LLl, LRl, sums = (np.ascontiguousarray(a) for a in (LLl, LRl, sums))
    q = [np.ascontiguousarray(a, np.int32) for a in qns]
    B = DMRG_BASIS(LL_LLLRRRRL=ptr(st[0], C.c_short), LR_LLLRRRRL=ptr(st[1], C.c_short), RR_LLLRRRRL=ptr(st[2], C.c_short),
                   RL_LLLRRRRL=ptr(st[3], C.c_short), Inv_LLLRRRRL=ptr(inv, C.c_int), dim_LLLRRRRL=len(st[0]), dim_LL=dim_LL,
                   dim_RR=dim_RR, dim_onsite=d, LL_LLLR=ptr(LLl, C.c_short), LR_LLLR=ptr(LRl, C.c_short), dim_LLLR=len(LLl),
                   Sum_LLLR=ptr(sums, C.c_int))
    T = abi.DMRG_TIME()
    v = np.ascontiguousarray(v, np.float64)
    fn = getattr(lib, f"DMRG_GET_SYSTEM_INFO_Q{len(q)}")
    fn.restype = P(abi.DMRG_SYSTEM_INFO)
    S = fn(*[ptr(a, C.c_int) for a in q], C.byref(B), ptr(v, C.c_double), max_dim, 1, C.byref(T)).contents
    n, dl = S.dim_renorm, S.dim_LLLR
    TM, TD = S.Trans_Matrix.contents, S.Trans_Matrix_Dagger.contents
    nnz = TM.Col[n]
    out = dict(dim_renorm=n, val=np.array(S.Val_DM_Dist[:dl]), sum_val=S.sum_val_dm, tr_error=S.tr_error,
               qn=[np.array(S.Q_Number1[:n], np.int32), np.array(S.Q_Number2[:n], np.int32), np.array(S.Q_Number3[:n], np.int32)][:len(q)],
               col_ptr=np.array(TM.Col[:n + 1]), rows=np.array(TM.Row[:nnz]), vals=np.array(TM.Val[:nnz]),
               d_row_ptr=np.array(TD.Row[:n + 1]), d_cols=np.array(TD.Col[:nnz]), d_vals=np.array(TD.Val[:nnz]),
               shape=(TM.row_dim, TM.col_dim, TD.row_dim, TD.col_dim), time=T.make_dens_mat,
               q2_sentinel=S.Q_Number2[0] if len(q) < 2 else None)
    for m in (TM, TD):
        for a in (m.Val, m.Row, m.Col):
            free(C.cast(a, C.c_void_p))
    free(C.cast(S.Trans_Matrix, C.c_void_p))
    free(C.cast(S.Trans_Matrix_Dagger, C.c_void_p))
    for a in (S.Val_DM_Dist, S.Q_Number1, S.Q_Number2, S.Q_Number3):
        free(C.cast(a, C.c_void_p))
    free(C.cast(C.pointer(S), C.c_void_p))
    return out


def same_truncation(a, b, tol_val=1e-13, tol_proj=1e-9):
    """Two system_info results describe the same truncation: the same kept dimension, quantum
    numbers and sparsity; spectra within tol_val; and, per block of equal quantum numbers, the
    same kept subspace (projectors within tol_proj -- eigenvectors are fixed only up to sign and,
    inside a degenerate multiplet, up to rotation).  Where b carries the oracle's per-block gaps
    between kept and dropped eigenvalues, a block's projector tolerance grows by 1e-13 * norm / gap:
    two correct eigensolvers may differ by that much on a subspace whose cut falls into a narrow
    gap.  Returns a list of differences (empty: same)."""
    bad = []
    tol_val = tol_val * max(1.0, abs(a["sum_val"]))
    if a["dim_renorm"] != b["dim_renorm"]:
        return [f"dim_renorm {a['dim_renorm']} != {b['dim_renorm']}"]
    for k, (x, y) in enumerate(zip(a["qn"], b["qn"])):
        if not np.array_equal(x, y):
            bad.append(f"Q_Number{k + 1}")
    if not (np.array_equal(a["col_ptr"], b["col_ptr"]) and np.array_equal(a["rows"], b["rows"])):
        return bad + ["sparsity"]
    if np.abs(a["val"] - b["val"]).max() > tol_val:
        bad.append(f"spectrum {np.abs(a['val'] - b['val']).max():.2e}")
    for key in ("sum_val", "tr_error"):
        if abs(a[key] - b[key]) > tol_val:
            bad.append(key)
    n = a["dim_renorm"]
    cp = a["col_ptr"]
    j = 0
    while j < n:
        r0 = a["rows"][cp[j]]
        j1 = j
        while j1 < n and a["rows"][cp[j1]] == r0:
            j1 += 1
        dim = cp[j + 1] - cp[j]
        Ta = np.stack([a["vals"][cp[c]:cp[c + 1]] for c in range(j, j1)], axis=1)
        Tb = np.stack([b["vals"][cp[c]:cp[c + 1]] for c in range(j, j1)], axis=1)
        tol = tol_proj
        if "gaps" in b and int(r0) in b["gaps"]:
            gap, norm = b["gaps"][int(r0)]
            tol = tol_proj + (1e-13 * norm / gap if gap > 0 else np.inf)
        if np.abs(Ta @ Ta.T - Tb @ Tb.T).max() > tol or dim != Ta.shape[0]:
            bad.append(f"subspace of the block at row {r0}")
        j = j1
    return bad


def call_exact_expectation(lib, op_o, op_r, start, end, basis, vec, d):
    """EXACT_EXPECTATION_ONSITE (op_o None: sites 0..end-1 of op_r) or _INTERSITE_Q0 of lib on a Q0
    basis; returns (Out, work vector 1, work vector 2)."""
    basis = np.ascontiguousarray(basis, np.int64)
    vec = np.ascontiguousarray(vec, np.float64)
    info = EXACT_BASIS_INFO(dim=len(basis), Basis=ptr(basis, C.c_long))
    n = end - start
    out = np.full(max(n, 1), np.nan)
    t1, t2 = np.full(len(basis), np.nan), np.full(len(basis), np.nan)
    if op_o is None:
        lib.EXACT_EXPECTATION_ONSITE(op_r.ref, ptr(out, C.c_double), ptr(vec, C.c_double), ptr(t1, C.c_double), d, end, 1,
                                     C.byref(info))
    else:
        lib.EXACT_EXPECTATION_INTERSITE_Q0(op_o.ref, op_r.ref, start, end, ptr(out, C.c_double), ptr(vec, C.c_double),
                                           ptr(t1, C.c_double), ptr(t2, C.c_double), d, 1, C.byref(info))
    return out[:max(n, 0)], t1, t2


def crs_crs_ccs(M1: abi.Crs, M2: abi.Crs, M3: abi.Ccs):
    """CRS_CRS_CCS_PRODUCT restated with numpy (sml/CRS_CRS_CCS_PRODUCT.c:42-121): W = M2 M3 by
    columns (each row of M2 summed in storage order against the dense column of M3), Out = M1 W by
    rows (each column of W summed in its storage order against the dense row of M1), entries with
    |v| > 1e-15 kept, every step rounded as the reference's loops round it.  Returns
    (W_col, W_row, W_val, Out_row, Out_col, Out_val)."""
    r1, r2 = M1.struct.row_dim, M2.struct.row_dim
    r3, c3 = M3.struct.row_dim, M3.struct.col_dim
    D3 = np.zeros((c3, r3))
    for c in range(c3):
        for e in range(M3.col[c], M3.col[c + 1]):
            D3[c, M3.row[e]] = M3.val[e]
    start, length = M2.row[:r2], M2.row[1:r2 + 1] - M2.row[:r2]
    W = np.zeros((c3, r2))
    for k in range(int(length.max()) if r2 else 0):
        live = np.flatnonzero(length > k)
        e = start[live] + k
        W[:, live] = W[:, live] + D3[:, M2.col[e]] * M2.val[e][None, :]
    keep = np.abs(W) > 1e-15
    w_col = np.concatenate([[0], np.cumsum(keep.sum(axis=1))])
    w_row = np.concatenate([np.flatnonzero(keep[c]) for c in range(c3)]) if c3 else np.zeros(0, int)
    w_val = W[keep]
    D1 = np.zeros((r1, r2))
    for r in range(r1):
        for e in range(M1.row[r], M1.row[r + 1]):
            D1[r, M1.col[e]] = M1.val[e]
    O = np.zeros((r1, c3))
    for c in range(c3):
        for e in range(w_col[c], w_col[c + 1]):
            O[:, c] = O[:, c] + D1[:, w_row[e]] * w_val[e]
    keep = np.abs(O) > 1e-15
    o_row = np.concatenate([[0], np.cumsum(keep.sum(axis=1))])
    o_col = np.concatenate([np.flatnonzero(keep[r]) for r in range(r1)]) if r1 else np.zeros(0, int)
    return w_col, w_row, w_val, o_row, o_col, O[keep]


def call_crs_crs_ccs(lib, M1: abi.Crs, M2: abi.Crs, M3: abi.Ccs, max_w, max_o):
    """CRS_CRS_CCS_PRODUCT of lib into fresh outputs of the given capacities; returns the same tuple
    as crs_crs_ccs and the work vector."""
    r1, r2, r3, c3 = M1.struct.row_dim, M2.struct.row_dim, M3.struct.row_dim, M3.struct.col_dim
    work = abi.Ccs.empty(c3, max_w)
    out = abi.Crs(np.zeros(r1 + 1, np.int64), np.zeros(max(max_o, 1), np.int32), np.zeros(max(max_o, 1)), n=r1)
    out.struct.max_val = max_o
    wv = np.full(max(r2, r3), np.nan)
    lib.CRS_CRS_CCS_PRODUCT(M1.ref, M2.ref, M3.ref, out.ref, work.ref, ptr(wv, C.c_double))
    nw, no = int(work.col[c3]), int(out.row[r1])
    return (work.col.copy(), work.row[:nw].copy(), work.val[:nw].copy(), out.row.copy(), out.col[:no].copy(), out.val[:no].copy(),
            wv, (work.struct.row_dim, work.struct.col_dim, out.struct.row_dim, out.struct.col_dim))


def site_apply(op: abi.Crs, out_basis, in_basis, d, site, vec, n_ele=None, threads=None):
    out_basis = np.ascontiguousarray(out_basis, np.int64)
    in_basis = np.ascontiguousarray(in_basis, np.int64)
    vec = np.ascontiguousarray(vec, np.float64)
    out = np.empty(len(out_basis))
    ne = np.ascontiguousarray(n_ele, np.int32) if n_ele is not None else None
    rc = load().or_site_apply(op.ref, ptr(out_basis, C.c_long), len(out_basis), ptr(in_basis, C.c_long), len(in_basis), d,
                              site, ptr(ne, C.c_int) if ne is not None else None, ptr(vec, C.c_double),
                              ptr(out, C.c_double), threads or threads_default())
    assert rc == 0
    return out


def obc_struct(sb):
    """or_obc view of a superblock operator built by dmrg_c_gb300.superblock."""
    return or_obc(M_LLLR=sb.M_LLLR.ref, M_LRRL=sb.M_LRRL.ref, M_LRRL_Sign=sb.M_LRRL_Sign.ref, M_RRRL=sb.M_RRRL.ref,
                  Ele_RR=ptr(sb.ele_rr, C.c_int), Basis=C.pointer(sb.basis))


def obc_spmv(sb, x, threads=None):
    x = np.ascontiguousarray(x, np.float64)
    y = np.empty(sb.n)
    o = obc_struct(sb)
    assert load().or_obc_spmv(C.byref(o), ptr(x, C.c_double), ptr(y, C.c_double), threads or threads_default()) == 0
    return y


def obc_lanczos_slow(sb, guess=None, acc=1e-14, min_step=1, max_step=800, tight=False, seed=0, threads=None):
    cfg = or_lanczos_cfg(acc=acc, min_step=min_step, max_step=max_step, max_block_step=max_step, tight=int(tight),
                         slow=1, guess=int(guess is not None), seed=seed, dense_below=0,
                         threads=threads or threads_default())
    v = np.array(guess, dtype=np.float64) if guess is not None else np.zeros(sb.n)
    out = or_lanczos_out()
    o = obc_struct(sb)
    rc = load().or_obc_lanczos_slow(C.byref(o), C.byref(cfg), ptr(v, C.c_double), C.byref(out))
    return rc, out, v


def obc_inverse_iteration(sb, eig_val, vec, ii_acc=1e-9, ii_diag_add=1e-11, ii_max_step=3, cg_acc=1e-7, cg_max_step=1000,
                          threads=None):
    cfg = or_ii_cfg(ii_acc=ii_acc, ii_diag_add=ii_diag_add, ii_max_step=ii_max_step, cg_acc=cg_acc,
                    cg_max_step=cg_max_step, minres=0, threads=threads or threads_default())
    v = np.array(vec, dtype=np.float64)
    out = or_ii_out()
    o = obc_struct(sb)
    rc = load().or_obc_inverse_iteration(C.byref(o), C.byref(cfg), eig_val, ptr(v, C.c_double), C.byref(out))
    return rc, out, v


# ---------------------------------------------------------------------------------------
# reference build (oracle/_ref), available only where the reference tree exists
# ---------------------------------------------------------------------------------------
def ref_available() -> bool:
    return REF_LIB.exists() or (REF_SRC / "sml" / "LANCZOS_SYM.c").exists()


def load_ref() -> C.CDLL:
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            subprocess.run(["make", "-s", "-j8", "-C", str(HERE), "ref", f"REF={REF_SRC}"], check=True)
        _ref = C.CDLL(str(REF_LIB))
    return _ref


@contextlib.contextmanager
def scratch_cwd():
    old = os.getcwd()
    with tempfile.TemporaryDirectory(prefix="dmrg_ref_") as d:
        os.chdir(d)
        try:
            yield Path(d)
        finally:
            os.chdir(old)


def ref_spmv(crs: abi.Crs, x, sym: bool, threads: int = 1):
    lib = load_ref()
    x = np.ascontiguousarray(x, np.float64)
    y = np.zeros(crs.n)
    if sym:
        temp = [np.zeros(crs.n) for _ in range(threads)]
        arr = (dp * threads)(*[ptr(t, C.c_double) for t in temp])
        lib.MATRIX_VECTOR_PRODUCT_SYM(crs.ref, ptr(x, C.c_double), ptr(y, C.c_double), arr, threads)
    else:
        lib.MATRIX_VECTOR_PRODUCT(crs.ref, ptr(x, C.c_double), ptr(y, C.c_double), threads)
    return y


def _box_lan(crs, vec, val, acc, min_step, max_step, max_block_step, guess, typ, threads):
    return BOX_LAN(M=crs.ref, Eig_Vec=ptr(vec, C.c_double), eig_val=ptr(val, C.c_double), acc=acc, min_step=min_step,
                   max_step=max_step, max_block_step=max_block_step, p_threads=threads, Guess=guess.encode(),
                   Type=typ.encode())


def ref_lanczos(crs, sym, guess, slow=False, acc=1e-14, min_step=1, max_step=800, max_block_step=None, tight=False,
                threads=1):
    """Run the reference LANCZOS[_SLOW][_SYM] with Guess "Yes"; returns (eig_val, vec, steps)."""
    lib = load_ref()
    vec = np.array(guess, dtype=np.float64)
    val = np.zeros(1)
    box = _box_lan(crs, vec, val, acc, min_step, max_step, max_step if max_block_step is None else max_block_step,
                   "Yes", "Tight" if tight else "Normal", threads)
    name = ("LANCZOS_SLOW" if slow else "LANCZOS") + ("_SYM" if sym else "")
    with scratch_cwd() as d:
        getattr(lib, name)(C.byref(box))
        steps = None
        for f in d.glob("SML_out/LANCZOS*"):
            line = f.read_text().strip().splitlines()[-1]
            steps = int(line.split()[0])
    return float(val[0]), vec, steps


def ref_inverse_iteration(crs, sym, eig_val, vec, ii_acc=1e-9, ii_diag_add=1e-11, ii_max_step=3, cg_acc=1e-7,
                          cg_max_step=1000, typ="CG", threads=1):
    lib = load_ref()
    v = np.array(vec, dtype=np.float64)
    ev = np.array([eig_val])
    box = BOX_II(M=crs.ref, ii_acc=ii_acc, ii_diag_add=ii_diag_add, ii_max_step=ii_max_step, cg_acc=cg_acc,
                 cg_max_step=cg_max_step, error=0.0, Eig_Vec=ptr(v, C.c_double), Eig_Val=ptr(ev, C.c_double),
                 p_threads=threads, Type=typ.encode())
    with scratch_cwd() as d:
        getattr(lib, "INVERSE_ITERATION_SYM" if sym else "INVERSE_ITERATION")(C.byref(box))
        f = d / "SML_out" / "Inv_iter_step.txt"
        iters = int(f.read_text().split()[-1]) if f.exists() else None
    return box.error, v, iters


def ref_linear_solve(crs, sym, b, x0, acc=1e-7, max_step=1000, minres=False, threads=1):
    lib = load_ref()
    b = np.ascontiguousarray(b, np.float64)
    x = np.array(x0, dtype=np.float64)
    box = BOX_CG(M=crs.ref, acc=acc, Vec=ptr(b, C.c_double), Out_Vec=ptr(x, C.c_double), max_step=max_step,
                 p_threads=threads)
    name = ("MINIMUM_RESIDUAL" if minres else "CONJUGATE_GRADIENT") + ("_SYM" if sym else "")
    with scratch_cwd() as d:
        getattr(lib, name)(C.byref(box))
        files = list(d.glob("SML_out/*_Step.txt"))
        iters = int(files[0].read_text().split()[-1]) if files else None
    return x, iters


def ref_converge_check(crs, sym, x, lam, threads=1):
    lib = load_ref()
    f = lib.CONVERGE_CHECK_SYM if sym else lib.CONVERGE_CHECK
    f.restype = C.c_double
    x = np.ascontiguousarray(x, np.float64)
    return f(crs.ref, ptr(x, C.c_double), C.c_double(lam), threads)


def ref_tridiag(d, e):
    """The reference's LAPACK dstev_ (through the shim) on (d, e): (w, z columns)."""
    lib = load_ref()
    n = len(d)
    D = np.array(d, dtype=np.float64)
    E = np.zeros(max(n, 1))
    E[:n - 1] = e
    Z = np.zeros(n * n)
    W = np.zeros(2 * n)
    info = C.c_int()
    nn, ldz = C.c_int(n), C.c_int(n)
    lib.dstev_(C.c_char_p(b"V"), C.byref(nn), ptr(D, C.c_double), ptr(E, C.c_double), ptr(Z, C.c_double), C.byref(ldz),
               ptr(W, C.c_double), C.byref(info))
    return D, Z.reshape(n, n).T


def ref_klm_model(L, n_ele, tot_sz, t=-1.0, J=1.0, D_z=0.0, I_xy=0.0, I_z=0.0, h_z=0.0, mu=0.0, spin_loc=1, bc="OBC"):
    m = MODEL_1DKLM_VF()
    m.BC = bc.encode()
    m.p_threads = 1
    m.spin_loc = spin_loc
    m.tot_site = L
    m.tot_sz = tot_sz
    m.tot_ele = n_ele
    m.dim_charge = 4
    m.dim_lspin = spin_loc + 1
    m.dim_onsite = 4 * (spin_loc + 1)
    m.t, m.J, m.D_z, m.I_xy, m.I_z, m.h_z, m.mu = t, J, D_z, I_xy, I_z, h_z, mu
    return m


def ref_klm_ed(model: MODEL_1DKLM_VF, est_max_row=10000):
    """The reference's own FIND_DIM / GET_BASIS / GET_HAM for the 1D KLM."""
    from dmrg_c_gb300.abi import EXACT_PARAMETER, EXACT_TIME
    lib = load_ref()
    lib.FIND_DIM.restype = C.c_int
    lib.GET_BASIS.restype = lp
    lib.GET_HAM.restype = P(CRS1)
    tm = EXACT_TIME()
    dim = lib.FIND_DIM(C.byref(model), C.byref(tm))
    bptr = lib.GET_BASIS(C.byref(model), C.byref(tm), dim)
    basis = np.ctypeslib.as_array(bptr, shape=(dim,)).copy()
    info = EXACT_BASIS_INFO(dim=dim, Basis=bptr, tot_sz=model.tot_sz, tot_ele=model.tot_ele, tot_parity=0)
    par = EXACT_PARAMETER()
    par.est_max_row_elem_num = est_max_row
    with scratch_cwd():
        H = lib.GET_HAM(C.byref(model), C.byref(info), C.byref(par), C.byref(tm)).contents
    row = np.ctypeslib.as_array(H.Row, shape=(dim + 1,)).copy()
    nnz = int(row[-1])
    col = np.ctypeslib.as_array(H.Col, shape=(nnz,)).copy()
    val = np.ctypeslib.as_array(H.Val, shape=(nnz,)).copy()
    return basis, row, col, val


def ref_klm_site_ops(model: MODEL_1DKLM_VF):
    """The reference's KLM site operators (Ham_On, SpL, SmL, SzL, CUp, CUp_D, CDown, CDown_D, Zero)."""
    lib = load_ref()
    d = model.dim_onsite
    out = []
    for which in range(9):
        row = np.zeros(d + 1, np.int64)
        col = np.zeros(d * d, np.int32)
        val = np.zeros(d * d)
        nnz = lib.ref_klm_site_op(C.byref(model), which, ptr(row, C.c_long), ptr(col, C.c_int), ptr(val, C.c_double))
        out.append((row, col[:nnz].copy(), val[:nnz].copy()))
    return out


def ref_site_apply(op: abi.Crs, basis, d, site, vec):
    lib = load_ref()
    basis = np.ascontiguousarray(basis, np.int64)
    # The reference's binary search may read one element past the table (its end bound is
    # inclusive, exact/EXACT_V_M_Q0.c:29): pad with a sentinel no code can equal.
    padded = np.concatenate([basis, [np.iinfo(np.int64).max]])
    vec = np.ascontiguousarray(vec, np.float64)
    out = np.zeros(len(basis))
    info = EXACT_BASIS_INFO(dim=len(basis), Basis=ptr(padded, C.c_long), tot_sz=0, tot_ele=0, tot_parity=0)
    lib.EXACT_V_M_Q0(op.ref, ptr(vec, C.c_double), ptr(out, C.c_double), d, site, 1, C.byref(info))
    return out


def ref_vm_q1(op: abi.Crs, sectors, shape, qn_out, qn_in, vec, d, site):
    """The reference's EXACT_V_M_Q1 (exact/EXACT_V_M_Q1.c:8-38) between two sectors of a whole basis."""
    lib = load_ref()
    W = abi.ExactWholeBasis(sectors, shape, pad=True)
    vec = np.ascontiguousarray(vec, np.float64)
    out = np.zeros(len(sectors[(qn_out,)]))
    lib.EXACT_V_M_Q1(op.ref, C.c_int(qn_out), ptr(vec, C.c_double), C.c_int(qn_in), ptr(out, C.c_double), C.c_int(d),
                     C.c_int(site), C.c_int(1), W.ref)
    return out


def ref_vm_q3(op: abi.Crs, sectors, shape, q_out, q_in, vec, sign, n_ele, d, site):
    """The reference's EXACT_V_M_Q3 (exact/EXACT_V_M_Q3.c:10-60) between two sectors (3-index labels)."""
    lib = load_ref()
    W = abi.ExactWholeBasis(sectors, shape, pad=True)
    vec = np.ascontiguousarray(vec, np.float64)
    ne = np.ascontiguousarray(n_ele, np.int32)
    out = np.zeros(len(sectors[tuple(q_out)]))
    lib.EXACT_V_M_Q3(op.ref, *(C.c_int(q) for q in q_out), ptr(vec, C.c_double), *(C.c_int(q) for q in q_in),
                     ptr(out, C.c_double), b"Yes" if sign else b"No", ptr(ne, C.c_int), C.c_int(d), C.c_int(site), C.c_int(1),
                     W.ref)
    return out


def ref_obc_spmv(sb, x, threads=1):
    lib = load_ref()
    x = np.ascontiguousarray(x, np.float64)
    y = np.zeros(sb.n)
    lib.DMRG_MATRIX_VECTOR_PRODUCT_OBC(sb.M_LLLR.ref, sb.M_LRRL.ref, sb.M_LRRL_Sign.ref, sb.M_RRRL.ref,
                                       ptr(x, C.c_double), ptr(y, C.c_double), ptr(sb.ele_rr, C.c_int), threads,
                                       C.byref(sb.basis))
    return y
