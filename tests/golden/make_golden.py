"""Regenerate the golden fixtures in this folder from the reference implementation.

Runs the reference's own C code (compiled from the dmrg_C sources into oracle/_ref by
oracle/Makefile) on seeded inputs and stores inputs and outputs as compressed .npz files.
Needs the reference source tree (env DMRG_REF, default /root/reference); the fixtures are
committed so that tests on machines without it still check against the reference.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np
import scipy.sparse as sp

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import pyoracle as po  # noqa: E402

from dmrg_c_gb300 import abi, ed_models, superblock  # noqa: E402


def quiet():
    """Silence the reference's progress output on fd 1 while it runs."""
    devnull = os.open(os.devnull, os.O_WRONLY)
    saved = os.dup(1)
    os.dup2(devnull, 1)
    return saved


def loud(saved):
    os.dup2(saved, 1)


def random_sym(n, density, seed, diag_scale=1.0):
    rng = np.random.default_rng(seed)
    A = sp.random(n, n, density=density, random_state=seed, data_rvs=rng.standard_normal)
    A = (A + A.T).tocsr()
    A.setdiag(rng.standard_normal(n) * diag_scale)
    A.eliminate_zeros()
    return A.tocsr()


def sml_fixture():
    """SpMV / Lanczos / inverse iteration / CG / MINRES on a random symmetric matrix."""
    A = random_sym(1500, 0.008, seed=11)
    low = abi.lower_diag_last(A)
    full = abi.Crs.from_scipy(A)
    rng = np.random.default_rng(12)
    x = rng.standard_normal(A.shape[0])
    guess = rng.standard_normal(A.shape[0])
    out = dict(low_row=low.row, low_col=low.col[:low.nnz], low_val=low.val[:low.nnz], full_row=full.row,
               full_col=full.col[:full.nnz], full_val=full.val[:full.nnz], x=x, guess=guess)
    s = quiet()
    try:
        out["spmv_sym"] = po.ref_spmv(low, x, True, 1)
        out["spmv_full"] = po.ref_spmv(full, x, False, 1)
        for name, sym, slow in (("lanczos_sym", True, False), ("lanczos_slow_sym", True, True), ("lanczos", False, False),
                                ("lanczos_slow", False, True)):
            E, v, steps = po.ref_lanczos(low if sym else full, sym, guess, slow=slow)
            out[name + "_E"], out[name + "_vec"], out[name + "_steps"] = E, v, steps
        E, v = out["lanczos_sym_E"], out["lanczos_sym_vec"]
        err, vv, it = po.ref_inverse_iteration(low, True, E, v)
        out["ii_sym_err"], out["ii_sym_vec"], out["ii_sym_iters"] = err, vv, it
        err, vv, it = po.ref_inverse_iteration(full, False, E, v)
        out["ii_err"], out["ii_vec"], out["ii_iters"] = err, vv, it
        # CG / MINRES on a positive definite shift of A
        B = (A + sp.identity(A.shape[0]) * (abs(E) + 1.0)).tocsr()
        lowB = abi.lower_diag_last(B)
        b = rng.standard_normal(A.shape[0])
        x0 = rng.standard_normal(A.shape[0])
        out.update(B_row=lowB.row, B_col=lowB.col[:lowB.nnz], B_val=lowB.val[:lowB.nnz], b=b, x0=x0)
        xs, it = po.ref_linear_solve(lowB, True, b, x0, acc=1e-10, max_step=1000)
        out["cg_x"], out["cg_iters"] = xs, it
        xs, it = po.ref_linear_solve(lowB, True, b, x0, acc=1e-6, max_step=1000, minres=True)
        out["mr_x"], out["mr_iters"] = xs, it
        out["conv_sym"] = po.ref_converge_check(low, True, out["lanczos_sym_vec"], E)
        out["conv_full"] = po.ref_converge_check(full, False, out["lanczos_sym_vec"], E)
    finally:
        loud(s)
    np.savez_compressed(HERE / "sml_random1500.npz", **out)


def tridiag_fixture():
    rng = np.random.default_rng(21)
    d = rng.standard_normal(120)
    e = np.abs(rng.standard_normal(119))
    w, z = po.ref_tridiag(d, e)
    np.savez_compressed(HERE / "tridiag120.npz", d=d, e=e, w=w, z0=z[:, 0])


def klm_ed_fixture():
    """The reference's own KLM ED basis and CRS (FIND_DIM / GET_BASIS / GET_HAM) and site
    operator tables, for two small chains."""
    out = {}
    for tag, (L, ne, sz, bc, kw) in {
        "obc": (4, 4, 0, "OBC", dict(t=-1.0, J=1.5, D_z=-1.0, I_z=-1.0, I_xy=0.0, h_z=0.1)),
        "pbc": (4, 3, 1, "PBC", dict(t=-1.0, J=1.0, D_z=0.0, I_z=0.5, I_xy=0.3, h_z=0.0, mu=0.2)),
    }.items():
        m = po.ref_klm_model(L, ne, sz, bc=bc, **kw)
        basis, row, col, val = po.ref_klm_ed(m)
        tabs = po.ref_klm_site_ops(m)
        out[f"{tag}_params"] = np.array([L, ne, sz, kw["t"], kw.get("I_z", 0.0), kw.get("I_xy", 0.0)])
        # every MODEL_1DKLM_VF parameter: L, N_e, 2Sz, t, J, D_z, I_xy, I_z, h_z, mu, PBC
        out[f"{tag}_model"] = np.array([L, ne, sz, kw["t"], kw.get("J", 0.0), kw.get("D_z", 0.0), kw.get("I_xy", 0.0),
                                        kw.get("I_z", 0.0), kw.get("h_z", 0.0), kw.get("mu", 0.0), bc == "PBC"])
        out[f"{tag}_basis"], out[f"{tag}_row"], out[f"{tag}_col"], out[f"{tag}_val"] = basis, row, col, val
        for k, (r, c, v) in enumerate(tabs):
            out[f"{tag}_op{k}_row"], out[f"{tag}_op{k}_col"], out[f"{tag}_op{k}_val"] = r, c, v
    np.savez_compressed(HERE / "klm_ed.npz", **out)


def sb_fixture():
    """The reference's superblock element builders (DMRG_MAKE_ELEM_*_LLLRRRRL) driven over a
    seeded Hubbard-type term list (OBC and PBC bonds): lower-triangle CRS arrays."""
    from dmrg_c_gb300 import sb_models
    out = {}
    for tag, pbc in (("obc", False), ("pbc", True)):
        m = sb_models.small_hubbard_model(pbc)
        row, col, val = po.ref_sb_build(m)
        out[f"{tag}_row"], out[f"{tag}_col"], out[f"{tag}_val"] = row, col, val
        out[f"{tag}_inv_checksum"] = np.int64(int(m.inv.astype(np.int64).sum()))
    np.savez_compressed(HERE / "sb_hubbard.npz", **out)


def sb_basis_fixture():
    """Superblock bases in the reference's order (states collected as GET_BASIS_SUPERBLOCK does,
    sorted by the reference's DMRG_QUICK_SORT_BASIS_Q1 / _Q2): a spin-1/2 case with one
    conserved quantity (2Sz) and a Hubbard-type case with two (N_e first, then 2Sz)."""
    rng = np.random.default_rng(11)
    out = {}
    # Q1: spin-1/2 sites (2Sz = +1 / -1), blocks of 40 / 36 states with 2Sz labels of 9 / 8 sites
    q1 = (rng.choice(np.arange(-9, 10, 2), 40), rng.choice(np.arange(-8, 9, 2), 36), np.array([1, -1]))
    LL, LR, RR, RL, inv = po.ref_sb_basis(40, 36, 2, q1, None, (1, 0))
    out.update(q1_LL=q1[0], q1_RR=q1[1], q1_site=q1[2], q1_target=np.int32(1), q1_states=np.stack([LL, LR, RR, RL]),
               q1_inv=inv)
    # Q2: Hubbard sites (empty, up, down, double) as (N_e, 2Sz); blocks of 48 / 44 states
    ne_s, sz_s = np.array([0, 1, 1, 2]), np.array([0, 1, -1, 0])
    def block(dim):
        ne = rng.integers(2, 9, dim)
        sz = np.array([rng.choice(np.arange(-min(k, 8 - k), min(k, 8 - k) + 1, 2)) for k in ne])
        return ne, sz
    (nl, sl), (nr, sr) = block(48), block(44)
    LL, LR, RR, RL, inv = po.ref_sb_basis(48, 44, 4, (nl, nr, ne_s), (sl, sr, sz_s), (12, 0))
    out.update(q2_ne_LL=nl, q2_ne_RR=nr, q2_ne_site=ne_s, q2_sz_LL=sl, q2_sz_RR=sr, q2_sz_site=sz_s,
               q2_targets=np.array([12, 0], np.int32), q2_states=np.stack([LL, LR, RR, RL]), q2_inv=inv)
    np.savez_compressed(HERE / "sb_basis.npz", **out)


def vm_fixture():
    """EXACT_V_M_Q0 on a Hubbard basis with the reference's C^dagger_up site operator."""
    model = ed_models.hubbard_chain(6, t=-1.0, U=2.0, n_ele=6, twoSz=0)
    basis, row, col, val = po.ed_build(model)
    rng = np.random.default_rng(31)
    vec = rng.standard_normal(len(basis))
    op = model.ops[1]
    out = dict(basis=basis, vec=vec, op_row=op.row, op_col=op.col[:op.nnz], op_val=op.val[:op.nnz])
    for site in (0, 2, 5):
        out[f"out_site{site}"] = po.ref_site_apply(op, basis, 4, site, vec)
    np.savez_compressed(HERE / "vm_hubbard6.npz", **out)


def vm_q13_fixture():
    """The reference's EXACT_V_M_Q1 (spin-1/2 chain: a sector-raising and a diagonal site operator)
    and EXACT_V_M_Q3 (Hubbard chain: c^dagger_up with and without the fermion sign)."""
    sys.path.insert(0, str(HERE.parent))
    from conftest import vm_whole_sectors
    q1, s1, q3, s3 = vm_whole_sectors()
    rng = np.random.default_rng(41)
    out = {}
    raise_op = abi.Crs(np.array([0, 0, 1]), np.array([0], np.int32), np.array([1.5]), n=2)   # row: output local state
    diag_op = abi.Crs(np.array([0, 1, 2]), np.array([0, 1], np.int32), np.array([-0.5, 0.75]), n=2)
    v3, v4 = rng.standard_normal(len(q1[(3,)])), rng.standard_normal(len(q1[(4,)]))
    out.update(q1_v3=v3, q1_v4=v4)
    for site in (0, 3, 7):
        out[f"q1_raise_site{site}"] = po.ref_vm_q1(raise_op, q1, s1, 4, 3, v3, 2, site)
        out[f"q1_diag_site{site}"] = po.ref_vm_q1(diag_op, q1, s1, 4, 4, v4, 2, site)
    model = ed_models.hubbard_chain(4, t=-1.0, U=2.0, n_ele=2, twoSz=0)
    cdu = model.ops[1]                                   # c^dagger_up (row: output local state)
    out.update(q3_op_row=cdu.row, q3_op_col=cdu.col[:cdu.nnz], q3_op_val=cdu.val[:cdu.nnz])
    vin = rng.standard_normal(len(q3[(1, 1, 0)]))
    out["q3_v"] = vin
    n_ele = np.array([0, 1, 1, 2], np.int32)
    for site in (0, 2, 3):
        for sign in (False, True):
            out[f"q3_site{site}_sign{int(sign)}"] = po.ref_vm_q3(cdu, q3, s3, (2, 1, 0), (1, 1, 0), vin, sign, n_ele, 4, site)
    np.savez_compressed(HERE / "vm_q13.npz", **out)


def sb_obs_fixture():
    """The reference's DMRG_V_M_{LL,LR,RR,RL}_Q0..Q4 and DMRG_EXPECTATION_ONSITE /
    _INTERSITE_Q0 on a seeded Hubbard-type superblock with every sector laid out: block
    observables, a c^dagger_up-type operator on each position (with and without the fermion
    sign) and site-by-site expectation values."""
    from dmrg_c_gb300 import sb_models
    p = sb_models.random_observable_problem(seed=5)
    ref = po.load_ref()
    rng = np.random.default_rng(61)
    q0 = p.target
    st, inv0 = p.sectors[q0], p.inv_sector(q0)
    v = rng.standard_normal(len(st[0]))
    out = dict(p.arrays(), v=v)
    ops = p.ops
    for pos, op in ((po.SB_LL, ops["LL"][0]), (po.SB_LR, ops["On"]), (po.SB_RR, ops["RR"][1]), (po.SB_RL, ops["On"])):
        out[f"q0_{po.SB_NAMES[pos]}"] = po.call_vm_q0(ref, st, inv0, p.dim_LL, p.dim_RR, p.d, op, pos, v)
    # sector-changing operator: the output sector is the input's label minus one up electron
    q_out = q0 - (sb_models.QN_SCALE + 1)
    shift = {po.SB_LL: ops["CdLL"][0], po.SB_LR: ops["CdOn"], po.SB_RR: ops["CdRR"][0], po.SB_RL: ops["CdOn"]}
    for k in (1, 2, 3, 4):
        wb = p.whole_basis(k)
        for pos, op in shift.items():
            if k == 4 and pos in (po.SB_LL, po.SB_LR):
                continue
            for sign in (False, True):
                if sign and pos == po.SB_LL:
                    continue
                out[f"q{k}_{po.SB_NAMES[pos]}_{int(sign)}"] = po.call_vm_whole(ref, wb, p.index(q_out, k), op, pos, v,
                                                                              ele=p.ele, sign=sign)
    o, t = po.call_expectation_onsite(ref, st, inv0, p.dim_LL, p.dim_RR, p.d, ops["LL"], ops["On"], ops["RR"], v)
    out.update(onsite=o, onsite_temp=t)
    for origin in (0, 1, len(ops["LL"])):
        o, t1, t2 = po.call_expectation_intersite_q0(ref, st, inv0, p.dim_LL, p.dim_RR, p.d, ops["CF"][origin:] if origin < len(ops["LL"]) else ops["CF"][:1],
                                                     ops["LL"], ops["On"], ops["RR"], origin, v)
        out.update({f"inter{origin}": o, f"inter{origin}_t1": t1, f"inter{origin}_t2": t2})
    # DMRG_GET_DENSITY_MATRIX for every block of the target sector's LLLR list
    import ctypes as C
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    lllr = po.lllr_list(p.q_LL, p.q_site, st)
    blocks = po.call_density_matrix(ref, st, inv0, p.dim_LL, p.dim_RR, p.d, v, lllr, libc.free)
    out["dm_blocks"] = np.concatenate([b.ravel() for b in blocks])
    # DMRG_GET_SYSTEM_INFO_Q1 (packed labels) and _Q2 (N_e, 2Sz) at two kept dimensions, on the
    # normalised vector (a ground state's): the cut at 1e-15 then sits far above the eigensolvers'
    # rounding of the zero eigenvalues
    vu = v / np.linalg.norm(v)
    out["v_unit"] = vu
    lab = lllr[3]
    N = np.rint(lab / sb_models.QN_SCALE).astype(np.int32)
    for tag, qns in (("q1", [lab.astype(np.int32)]), ("q2", [N, (lab - N * sb_models.QN_SCALE).astype(np.int32)])):
        for max_dim in (20, 10000):
            r = po.call_system_info(ref, qns, st, inv0, p.dim_LL, p.dim_RR, p.d, vu, lllr, max_dim, libc.free)
            for k in ("dim_renorm", "val", "sum_val", "tr_error", "col_ptr", "rows", "vals"):
                out[f"si_{tag}_{max_dim}_{k}"] = r[k]
            for k, q in enumerate(r["qn"]):
                out[f"si_{tag}_{max_dim}_qn{k}"] = q
    np.savez_compressed(HERE / "sb_obs.npz", **out)


def ed_obs_fixture():
    """The reference's EXACT_EXPECTATION_ONSITE / _INTERSITE_Q0 on the Hubbard L=6 basis: site
    densities and density correlations."""
    model = ed_models.hubbard_chain(6, t=-1.0, U=2.0, n_ele=6, twoSz=0)
    basis, row, col, val = po.ed_build(model)
    rng = np.random.default_rng(33)
    vec = rng.standard_normal(len(basis))
    dens = abi.Crs(np.arange(5), np.arange(4, dtype=np.int32), np.array([0.0, 1.0, 1.0, 2.0]))
    nup = abi.Crs(np.arange(5), np.arange(4, dtype=np.int32), np.array([0.0, 1.0, 0.0, 1.0]))
    ref = po.load_ref()
    out = dict(basis=basis, vec=vec)
    out["onsite"], out["onsite_t"], _ = po.call_exact_expectation(ref, None, dens, 0, 6, basis, vec, 4)
    for start, end in ((0, 6), (2, 5), (3, 3)):
        o, t1, t2 = po.call_exact_expectation(ref, nup, dens, start, end, basis, vec, 4)
        out[f"inter_{start}_{end}"], out[f"inter_{start}_{end}_t1"], out[f"inter_{start}_{end}_t2"] = o, t1, t2
    np.savez_compressed(HERE / "ed_obs_hubbard6.npz", **out)


def renorm_operands(seed=71, r3=60, c3=24, per_row=7):
    """Operands of a renormalisation T^dagger O T: T (r3 x c3, CCS) with each column supported on one
    block of rows, T^dagger as CRS, O (r3 x r3, CRS) with a row whose products cancel exactly."""
    rng = np.random.default_rng(seed)
    blocks = np.sort(rng.integers(0, 6, r3))
    T = np.zeros((r3, c3))
    for j in range(c3):
        rows = np.flatnonzero(blocks == j % 6)
        T[rows, j] = rng.standard_normal(len(rows))
    O = sp.random(r3, r3, density=per_row / r3, random_state=seed, data_rvs=rng.standard_normal).toarray()
    O[O == 0] = 0.0
    # row 0: +x on row a and -x on row b of T, where T's rows a and b are equal -> exact zeros
    a, b = 1, 2
    T[b] = T[a]
    O[0] = 0.0
    O[0, a], O[0, b] = 0.75, -0.75
    M3 = sp.csc_matrix(T)
    return abi.Crs.from_scipy(sp.csr_matrix(T.T)), abi.Crs.from_scipy(sp.csr_matrix(O)), abi.Ccs.from_scipy(M3)


def renorm_fixture():
    """The reference's CRS_CRS_CCS_PRODUCT on seeded renormalisation operands."""
    M1, M2, M3 = renorm_operands()
    ref = po.load_ref()
    r = po.call_crs_crs_ccs(ref, M1, M2, M3, 60 * 24, 24 * 24)
    names = ("w_col", "w_row", "w_val", "o_row", "o_col", "o_val")
    ops = dict(m1_row=M1.row, m1_col=M1.col[:M1.nnz], m1_val=M1.val[:M1.nnz], m2_row=M2.row, m2_col=M2.col[:M2.nnz],
               m2_val=M2.val[:M2.nnz], m3_col=M3.col, m3_row=M3.row[:M3.col[-1]], m3_val=M3.val[:M3.col[-1]],
               dims=np.array([M1.struct.row_dim, M2.struct.row_dim, M3.struct.row_dim, M3.struct.col_dim]))
    np.savez_compressed(HERE / "renorm.npz", **dict(zip(names, r[:6])), shape=np.array(r[7]), **ops)


def obc_fixture():
    """The reference's matrix-free superblock product and OBC Lanczos on a seeded
    synthetic superblock (spin-1/2 sites, one block quantum number)."""
    qb = superblock.spin_block_labels(40, 9, seed=41)
    sb = superblock.synthetic_superblock(40, 2, qb, [1, -1], 0, nnz_lllr=6, nnz_lrrl=2, seed=42, with_sign=True)
    rng = np.random.default_rng(43)
    x = rng.standard_normal(sb.n)
    s = quiet()
    try:
        y = po.ref_obc_spmv(sb, x)
    finally:
        loud(s)
    out = dict(x=x, y=y, n=sb.n)
    np.savez_compressed(HERE / "obc_synthetic.npz", **out)


def xxz_energy_fixture():
    """Reference LANCZOS + INVERSE_ITERATION on the XXZ L=16 Heisenberg chain (Sz=0)."""
    model = ed_models.xxz_chain(16, Jxy=1.0, Jz=1.0)
    basis, row, col, val = po.ed_build(model)
    H = abi.Crs(row, col, val)
    guess = np.random.default_rng(51).standard_normal(len(basis))
    s = quiet()
    try:
        E, v, steps = po.ref_lanczos(H, False, guess)
        err, vv, it = po.ref_inverse_iteration(H, False, E, v)
    finally:
        loud(s)
    np.savez_compressed(HERE / "xxz16.npz", E=E, steps=steps, guess=guess, ii_err=err, dim=len(basis), nnz=row[-1])


def main():
    if not po.ref_available():
        raise SystemExit("reference sources not found (set DMRG_REF)")
    po.load_ref()
    sml_fixture()
    tridiag_fixture()
    klm_ed_fixture()
    sb_fixture()
    sb_basis_fixture()
    vm_fixture()
    vm_q13_fixture()
    sb_obs_fixture()
    ed_obs_fixture()
    renorm_fixture()
    obc_fixture()
    xxz_energy_fixture()
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
