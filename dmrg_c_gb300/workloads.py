"""Seeded synthetic inputs with the shapes of the benchmark configurations.

The DMRG configurations solve superblock Hamiltonians whose block operators come out of a
DMRG sweep.  No sweep is run here: blocks of ``m`` kept states get seeded quantum-number
labels drawn around the sector a sweep keeps, random symmetric block operators conserve
them, and the superblock of the target sector is assembled in the reference's layout
(dmrg_c_gb300.superblock).  Sizes are tuned so that the superblock dimension and stored
entries per row match the configurations' largest step (n / nnz figures of the reference
runs: XXZ m=64 n~3.7e3, ~66 entries/row; KLM m=128 n~5.8e4, ~63 entries/row; Hubbard
m=512 n~2.4e5, ~235 entries/row).
"""
from __future__ import annotations

import numpy as np

from . import superblock
from .ed_models import hubbard_chain, xxz_chain

QN_SCALE = 1000   # pack (N_e, 2Sz) into one integer N_e*1000 + 2Sz (N_e is the primary key)


def _block_labels(m, n_sites, n_mean, n_sd, sz_sd, seed, fermions=True):
    rng = np.random.default_rng(seed)
    if fermions:
        N = np.clip(np.rint(rng.normal(n_mean, n_sd, size=m)), 0, 2 * n_sites).astype(np.int64)
        par = N % 2 if n_sites % 2 == 0 else (N + n_sites) % 2
    else:
        N = np.zeros(m, np.int64)
        par = np.full(m, n_sites % 2)
    sz = par + 2 * np.rint(rng.normal(0.0, sz_sd, size=m)).astype(np.int64)
    sz = np.clip(sz, -n_sites, n_sites)
    return np.sort(N * QN_SCALE + sz)


def klm_site_labels():
    """KLM site (spin_loc = 1): state = charge*2 + s; N_e = [0,1,1,2][charge],
    2Sz = [0,1,-1,0][charge] + (1 - 2s) (onsite_op/ONSITE_FIND_SITE_*_SZBASIS_KLM.c)."""
    out = []
    for k in range(8):
        c, s = k // 2, k % 2
        out.append([0, 1, 1, 2][c] * QN_SCALE + [0, 1, -1, 0][c] + (1 - 2 * s))
    return np.array(out)


def hubbard_site_labels():
    return np.array([0 * QN_SCALE + 0, 1 * QN_SCALE + 1, 1 * QN_SCALE - 1, 2 * QN_SCALE + 0])


def xxz_superblock_m64(seed=0):
    """Largest superblock of the XXZ DMRG run: L=32, m=64 (block of 15 sites), 2Sz = 0."""
    qb = _block_labels(64, 15, 0, 0, 0.95, seed, fermions=False)
    return superblock.synthetic_superblock(64, 2, qb, np.array([1, -1]), 0, nnz_lllr=29, nnz_lrrl=2, seed=seed + 1)


def klm_superblock_m128(seed=0):
    """Largest superblock of the Kondo-lattice DMRG run: L=24, N_e=12, 2Sz=0, m=128 (block of 11 sites, d=8)."""
    qb = _block_labels(128, 11, 5.0, 0.95, 0.85, seed)
    return superblock.synthetic_superblock(128, 8, qb, klm_site_labels(), 12 * QN_SCALE, nnz_lllr=18, nnz_lrrl=3,
                                           seed=seed + 1, with_sign=True)


def hubbard_superblock_m512(seed=0):
    """Largest superblock of the Hubbard DMRG run: L=64, half filling, 2Sz=0, m=512 (block of 31 sites, d=4)."""
    qb = _block_labels(512, 31, 31.0, 1.25, 0.9, seed)
    return superblock.synthetic_superblock(512, 4, qb, hubbard_site_labels(), 64 * QN_SCALE, nnz_lllr=100, nnz_lrrl=3,
                                           seed=seed + 1, with_sign=True)


def superblock_labels(name, seed=0):
    """(block labels, site labels, target, kept states m) of the synthetic superblock `name` (the
    labels the generators above draw, so the sector and its order are the same)."""
    if name == "klm_m128":
        return _block_labels(128, 11, 5.0, 0.95, 0.85, seed), klm_site_labels(), 12 * QN_SCALE, 128
    if name == "hubbard_m512":
        return _block_labels(512, 31, 31.0, 1.25, 0.9, seed), hubbard_site_labels(), 64 * QN_SCALE, 512
    if name == "xxz_m64":
        return _block_labels(64, 15, 0, 0, 0.95, seed, fermions=False), np.array([1, -1]), 0, 64
    raise KeyError(name)


def xxz_ed_batch(count=256, seed=0):
    """Batched XXZ ED instances: L uniform in {12,...,22}, Jz ~ U[0,2], hz ~ U[0,1], Jxy = 1, 2Sz = 0, OBC."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        L = int(rng.choice(np.arange(12, 23, 2)))
        Jz = float(rng.uniform(0, 2))
        hz = float(rng.uniform(0, 1))
        out.append(dict(L=L, Jz=Jz, hz=hz, model=lambda L=L, Jz=Jz, hz=hz: xxz_chain(L, Jxy=1.0, Jz=Jz, hz=hz)))
    return out


def hubbard_request_trace(rate=200.0, duration=60.0, seed=1):
    """Served Hubbard ED request trace: Poisson arrivals at `rate`/s for `duration` s; L in
    {8,10,12}, t=1 (coefficient -1), U ~ U[0,8], h ~ U[0,0.5], half filling, 2Sz = 0, OBC."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        L = int(rng.choice([8, 10, 12]))
        U = float(rng.uniform(0, 8))
        h = float(rng.uniform(0, 0.5))
        out.append(dict(t=t, L=L, U=U, h=h, model=lambda L=L, U=U, h=h: hubbard_chain(L, t=-1.0, U=U, hz=h)))
    return out


def hubbard_sb_model_m512(seed=0, per_row=24):
    """Term-list form (block and site operators) of a Hubbard m=512 superblock of the same
    basis as ``hubbard_superblock_m512``, for the GPU superblock CRS build."""
    from . import sb_models
    qb = _block_labels(512, 31, 31.0, 1.25, 0.9, seed)
    sb = superblock.synthetic_superblock(512, 4, qb, hubbard_site_labels(), 64 * QN_SCALE, nnz_lllr=1, nnz_lrrl=1,
                                         seed=seed + 1, with_sign=True)
    return sb_models.hubbard_superblock_model(sb, qb, seed=seed + 2, per_row=per_row)
