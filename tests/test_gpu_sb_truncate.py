"""Truncation of the LL+LR block on the GPU (DMRG_GET_SYSTEM_INFO_Q1 / _Q2 / _Q3: density
matrices and their batched Jacobi eigen-decompositions on the device, the reference's ordering and
cut on the host) against the reference-made fixture and the oracle.

The kept dimension, quantum numbers and sparsity of the transformation matrix must be identical;
spectra agree within 1e-13 of |v|^2 and the kept subspace of every block within 1e-9 (eigenvectors
are fixed only up to sign, and up to rotation inside a degenerate multiplet)."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden
from dmrg_c_gb300 import sb_models, workloads

pytestmark = pytest.mark.gpu


def _free():
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    return libc.free


def _qns(lab, k):
    N = np.rint(lab / sb_models.QN_SCALE).astype(np.int32)
    sz = (lab - N * sb_models.QN_SCALE).astype(np.int32)
    return {1: [lab.astype(np.int32)], 2: [N, sz], 3: [N, sz, np.zeros_like(N)]}[k]


@pytest.mark.parametrize("tag", ["q1", "q2"])
@pytest.mark.parametrize("max_dim", [20, 10000])
def test_system_info_vs_reference_golden(gpu, oracle, tag, max_dim):
    g = golden("sb_obs.npz")
    p = sb_models.ObservableProblem.from_arrays(g)
    st, inv0 = p.sectors[p.target], p.inv_sector(p.target)
    lllr = oracle.lllr_list(p.q_LL, p.q_site, st)
    got = oracle.call_system_info(gpu.load(), _qns(lllr[3], 1 if tag == "q1" else 2), st, inv0, p.dim_LL, p.dim_RR, p.d,
                                  g["v_unit"], lllr, max_dim, _free())
    pre = f"si_{tag}_{max_dim}_"
    want = dict(dim_renorm=int(g[pre + "dim_renorm"]), val=g[pre + "val"], sum_val=float(g[pre + "sum_val"]),
                tr_error=float(g[pre + "tr_error"]), col_ptr=g[pre + "col_ptr"], rows=g[pre + "rows"], vals=g[pre + "vals"],
                qn=[g[pre + f"qn{k}"] for k in range(1 if tag == "q1" else 2)])
    assert oracle.same_truncation(got, want) == []
    n, L = got["dim_renorm"], p.dim_LL * p.d
    assert got["shape"] == (L, n, n, L)
    assert np.array_equal(got["d_row_ptr"], got["col_ptr"]) and np.array_equal(got["d_cols"], got["rows"])
    assert np.array_equal(got["d_vals"], got["vals"])
    if tag == "q1":
        assert got["q2_sentinel"] == -2**31


def _columns(r):
    cp = r["col_ptr"]
    return [(r["rows"][cp[j]:cp[j + 1]], r["vals"][cp[j]:cp[j + 1]]) for j in range(r["dim_renorm"])]


def test_system_info_q3_and_orthonormal_columns(gpu, oracle):
    """The three-label variant (a constant third label) keeps what the two-label one keeps; the
    kept eigenvectors are orthonormal."""
    g = golden("sb_obs.npz")
    p = sb_models.ObservableProblem.from_arrays(g)
    st, inv0 = p.sectors[p.target], p.inv_sector(p.target)
    lllr = oracle.lllr_list(p.q_LL, p.q_site, st)
    want = oracle.system_info(_qns(lllr[3], 3), st, inv0, p.d, p.dim_RR, g["v_unit"], lllr, 30)
    got = oracle.call_system_info(gpu.load(), _qns(lllr[3], 3), st, inv0, p.dim_LL, p.dim_RR, p.d, g["v_unit"], lllr, 30, _free())
    assert oracle.same_truncation(got, want) == []
    L = p.dim_LL * p.d
    T = np.zeros((L, got["dim_renorm"]))
    for j, (rows, vals) in enumerate(_columns(got)):
        T[rows, j] = vals
    assert np.abs(T.T @ T - np.eye(got["dim_renorm"])).max() < 1e-12


def test_system_info_hubbard_m512_vs_oracle(gpu, oracle):
    """The Hubbard m=512 superblock (L=64, half filling): 57 density blocks of up to 216 pairs (16-CTA
    clusters); keep 512 states."""
    qb = workloads._block_labels(512, 31, 31.0, 1.25, 0.9, 0)
    qs = workloads.hubbard_site_labels()
    st = sb_models.sector_states(qb, qb, qs, 64 * sb_models.QN_SCALE)
    d = 4
    inv = -np.ones(512 * d * 512 * d, np.int32)
    inv[((st[0].astype(np.int64) * d + st[1]) * 512 + st[2]) * d + st[3]] = np.arange(len(st[0]), dtype=np.int32)
    lllr = oracle.lllr_list(qb, qs, st)
    assert lllr[4].max() > 160
    v = np.random.default_rng(21).standard_normal(len(st[0]))
    v /= np.linalg.norm(v)
    qns = _qns(lllr[3], 2)
    want = oracle.system_info(qns, st, inv, d, 512, v, lllr, 512)
    got = oracle.call_system_info(gpu.load(), qns, st, inv, 512, 512, d, v, lllr, 512, _free())
    assert oracle.same_truncation(got, want) == []
    assert got["time"] > 0


def test_system_info_block_beyond_shared_memory(gpu, oracle):
    """One density block of 400 pairs (every state with one label): too large for the CTAs' shared
    memory, so the eigensolver keeps its rows in a global workspace."""
    dim, d = 200, 2
    qb, qs = np.zeros(dim, np.int64), np.zeros(d, np.int64)
    st = sb_models.sector_states(qb, qb, qs, 0)
    inv = -np.ones(dim * d * dim * d, np.int32)
    inv[((st[0].astype(np.int64) * d + st[1]) * dim + st[2]) * d + st[3]] = np.arange(len(st[0]), dtype=np.int32)
    lllr = oracle.lllr_list(qb, qs, st)
    assert len(lllr[4]) == 1 and lllr[4][0] == 400
    v = np.random.default_rng(23).standard_normal(len(st[0]))
    v /= np.linalg.norm(v)
    qns = [np.zeros(dim * d, np.int32)]
    want = oracle.system_info(qns, st, inv, d, dim, v, lllr, 100)
    got = oracle.call_system_info(gpu.load(), qns, st, inv, dim, dim, d, v, lllr, 100, _free())
    assert oracle.same_truncation(got, want) == []


def test_system_info_mixed_block_sizes_with_global_workspace(gpu, oracle):
    """One density block beyond the CTAs' shared memory (400 pairs) beside small blocks, several
    with fewer pairs than a cluster has CTAs (2 and 6 pairs), in one call: the large block runs
    from the global workspace and the small ones from shared memory."""
    d = 2
    qb = np.array([0] * 200 + [1] * 3 + [-1] * 3 + [2] + [-2], np.int64)
    dim = len(qb)
    qs = np.zeros(d, np.int64)
    st = sb_models.sector_states(qb, qb, qs, 0)
    inv = -np.ones(dim * d * dim * d, np.int32)
    inv[((st[0].astype(np.int64) * d + st[1]) * dim + st[2]) * d + st[3]] = np.arange(len(st[0]), dtype=np.int32)
    lllr = oracle.lllr_list(qb, qs, st)
    sizes = sorted(int(x) for x in lllr[4])
    assert sizes[-1] == 400 and sizes[0] < 8 and len(sizes) >= 4
    v = np.random.default_rng(29).standard_normal(len(st[0]))
    v /= np.linalg.norm(v)
    qns = _qns(lllr[3], 1)   # the LLLR labels in the basis' ascending order
    for keep in (30, 404):
        want = oracle.system_info(qns, st, inv, d, dim, v, lllr, keep)
        got = oracle.call_system_info(gpu.load(), qns, st, inv, dim, dim, d, v, lllr, keep, _free())
        assert oracle.same_truncation(got, want) == []
