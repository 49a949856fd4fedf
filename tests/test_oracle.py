"""The oracle (CPU restatement) pinned against the reference: golden fixtures produced by
the reference's own code (always), the live reference build (where its sources exist),
and closed-form answers."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import golden, klm_model_from_golden, renorm_operands_from_golden
from dmrg_c_gb300 import abi, ed_models, superblock


def sml_inputs():
    g = golden("sml_random1500.npz")
    low = abi.Crs(g["low_row"], g["low_col"], g["low_val"])
    full = abi.Crs(g["full_row"], g["full_col"], g["full_val"])
    return g, low, full


# ---- golden fixtures (reference outputs) ---------------------------------------------------

def test_spmv_matches_reference_golden(oracle):
    g, low, full = sml_inputs()
    np.testing.assert_allclose(oracle.spmv(low, g["x"], True), g["spmv_sym"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(oracle.spmv(full, g["x"], False), g["spmv_full"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("name,sym,slow", [("lanczos_sym", True, False), ("lanczos_slow_sym", True, True),
                                           ("lanczos", False, False), ("lanczos_slow", False, True)])
def test_lanczos_matches_reference_golden(oracle, name, sym, slow):
    g, low, full = sml_inputs()
    rc, out, v = oracle.lanczos(low if sym else full, sym, guess=g["guess"], slow=slow)
    assert rc == 0 and out.converged
    E = float(g[name + "_E"])
    assert abs(out.eig_val - E) <= 1e-12 * abs(E)
    assert abs(out.steps - int(g[name + "_steps"])) <= 2
    assert abs(abs(v @ g[name + "_vec"]) - 1) < 1e-9


def test_inverse_iteration_matches_reference_golden(oracle):
    g, low, full = sml_inputs()
    for sym, tag in ((True, "ii_sym"), (False, "ii")):
        rc, out, v = oracle.inverse_iteration(low if sym else full, sym, float(g["lanczos_sym_E"]), g["lanczos_sym_vec"])
        assert out.converged and out.iters == int(g[tag + "_iters"])
        assert out.error < 1e-9
        assert abs(abs(v @ g[tag + "_vec"]) - 1) < 1e-12


def test_cg_minres_match_reference_golden(oracle):
    g = golden("sml_random1500.npz")
    B = abi.Crs(g["B_row"], g["B_col"], g["B_val"])
    rc, it, cv, x = oracle.linear_solve(B, True, g["b"], g["x0"], acc=1e-10, max_step=1000)
    assert cv and abs(it - int(g["cg_iters"])) <= 1
    np.testing.assert_allclose(x, g["cg_x"], rtol=0, atol=1e-8)
    rc, it, cv, x = oracle.linear_solve(B, True, g["b"], g["x0"], acc=1e-6, max_step=1000, minres=True)
    assert cv and abs(it - int(g["mr_iters"])) <= 1
    np.testing.assert_allclose(x, g["mr_x"], rtol=0, atol=1e-6)


def test_converge_check_golden(oracle):
    g, low, full = sml_inputs()
    E = float(g["lanczos_sym_E"])
    assert oracle.converge_check(low, True, g["lanczos_sym_vec"], E) == pytest.approx(float(g["conv_sym"]), rel=1e-6)
    assert oracle.converge_check(full, False, g["lanczos_sym_vec"], E) == pytest.approx(float(g["conv_full"]), rel=1e-6)


def test_tridiag_matches_dstev_golden(oracle):
    g = golden("tridiag120.npz")
    w, z = oracle.tridiag_eig(g["d"], g["e"])
    np.testing.assert_allclose(w, g["w"], rtol=0, atol=1e-12)
    assert abs(abs(z[:, 0] @ g["z0"]) - 1) < 1e-12


@pytest.mark.parametrize("tag", ["obc", "pbc"])
def test_ed_build_bit_exact_vs_reference_golden(oracle, tag):
    """Basis table and CRS arrays (row_ptr, col_idx and values) identical to the reference's
    FIND_DIM / GET_BASIS / GET_HAM on the KLM chain."""
    g = golden("klm_ed.npz")
    model = klm_model_from_golden(g, tag)
    basis, row, col, val = oracle.ed_build(model)
    assert np.array_equal(basis, g[f"{tag}_basis"])
    assert np.array_equal(row, g[f"{tag}_row"])
    assert np.array_equal(col, g[f"{tag}_col"])
    assert np.array_equal(val.view(np.int64), g[f"{tag}_val"].view(np.int64))


def test_site_apply_matches_reference_golden(oracle):
    g = golden("vm_hubbard6.npz")
    op = abi.Crs(g["op_row"], g["op_col"], g["op_val"], n=4)
    for site in (0, 2, 5):
        out = oracle.site_apply(op, g["basis"], g["basis"], 4, site, g["vec"])
        np.testing.assert_array_equal(out, g[f"out_site{site}"])


def test_obc_spmv_matches_reference_golden(oracle):
    g = golden("obc_synthetic.npz")
    qb = superblock.spin_block_labels(40, 9, seed=41)
    sb = superblock.synthetic_superblock(40, 2, qb, [1, -1], 0, nnz_lllr=6, nnz_lrrl=2, seed=42, with_sign=True)
    assert sb.n == int(g["n"])
    np.testing.assert_array_equal(oracle.obc_spmv(sb, g["x"]), g["y"])
    np.testing.assert_allclose(sb.explicit() @ g["x"], g["y"], rtol=0, atol=1e-12)


def test_heisenberg16_energy_golden(oracle):
    g = golden("xxz16.npz")
    model = ed_models.xxz_chain(16)
    basis, row, col, val = oracle.ed_build(model)
    assert len(basis) == int(g["dim"]) and row[-1] == int(g["nnz"])
    rc, out, v = oracle.lanczos(abi.Crs(row, col, val), False, guess=g["guess"])
    assert abs(out.eig_val - float(g["E"])) < 1e-12 * abs(float(g["E"]))


# ---- closed-form answers ----------------------------------------------------------------------

@pytest.mark.parametrize("L", [6, 8, 10])
def test_free_fermion_hubbard_u0(oracle, L):
    model = ed_models.hubbard_chain(L, t=-1.0, U=0.0, n_ele=L, twoSz=0)
    basis, row, col, val = oracle.ed_build(model)
    H = abi.Crs(row, col, val)
    rc, out, v = oracle.lanczos(H, False, seed=3, dense_below=0)
    assert out.converged
    assert abs(out.eig_val - ed_models.free_fermion_energy(L, L // 2, L // 2)) < 1e-10


def test_two_site_hubbard(oracle):
    U = 3.0
    model = ed_models.hubbard_chain(2, t=-1.0, U=U, n_ele=2, twoSz=0)
    basis, row, col, val = oracle.ed_build(model)
    A = sp.csr_matrix((val, col, row), shape=(len(basis), len(basis))).toarray()
    assert np.allclose(A, A.T)
    assert np.linalg.eigvalsh(A)[0] == pytest.approx((U - np.sqrt(U * U + 16.0)) / 2.0, abs=1e-12)


@pytest.mark.parametrize("L", [8, 12])
def test_xx_chain_free_fermions(oracle, L):
    """Jz = 0: XX chain = free spinless fermions with hopping Jxy/2."""
    model = ed_models.xxz_chain(L, Jxy=1.0, Jz=0.0)
    basis, row, col, val = oracle.ed_build(model)
    rc, out, v = oracle.lanczos(abi.Crs(row, col, val), False, seed=5, dense_below=0)
    eps = np.sort(np.cos(np.pi * np.arange(1, L + 1) / (L + 1)))
    assert abs(out.eig_val - eps[:L // 2].sum()) < 1e-10


def test_dense_path_small(oracle):
    A = sp.random(300, 300, density=0.05, random_state=7)
    A = (A + A.T).tocsr()
    low = abi.lower_diag_last(A)
    rc, out, v = oracle.lanczos(low, True, seed=1)
    assert out.dense and abs(out.eig_val - np.linalg.eigvalsh(A.toarray())[0]) < 1e-12
    assert np.linalg.norm(A @ v - out.eig_val * v) < 1e-10


# ---- live reference (where its sources are present) ------------------------------------------

def test_live_reference_lanczos_cases(ref, rng):
    for n, dens in ((1200, 0.01), (2500, 0.004)):
        A = sp.random(n, n, density=dens, random_state=int(rng.integers(1 << 30)))
        A = (A + A.T).tocsr()
        A.setdiag(rng.standard_normal(n))
        low = abi.lower_diag_last(A)
        g = rng.standard_normal(n)
        s = __import__("os").dup(1)
        E, v, st = ref.ref_lanczos(low, True, g)
        rc, out, vo = ref.lanczos(low, True, guess=g)
        assert abs(out.eig_val - E) < 1e-12 * abs(E)
        assert abs(abs(v @ vo) - 1) < 1e-9
        del s


def test_live_reference_klm_ed_random(ref):
    for L, ne, sz in ((3, 3, 0), (4, 5, 1)):   # 2Sz has the parity of ne + L
        m = ref.ref_klm_model(L, ne, sz, t=-1.0, J=0.7, D_z=0.2, I_z=0.3, h_z=0.05)
        basis, row, col, val = ref.ref_klm_ed(m)
        tabs = ref.ref_klm_site_ops(m)
        model = ed_models.klm_chain_from_tables(L, tabs, ne, sz, t=-1.0, I_z=0.3)
        b2, r2, c2, v2 = ref.ed_build(model)
        assert np.array_equal(basis, b2) and np.array_equal(row, r2) and np.array_equal(col, c2)
        assert np.array_equal(val.view(np.int64), v2.view(np.int64))


@pytest.mark.parametrize("tag", ["obc", "pbc"])
def test_superblock_build_bit_exact_vs_reference_golden(oracle, tag):
    """Superblock CRS (lower triangle, diagonal last) identical to the reference's element
    builders DMRG_MAKE_ELEM_*_LLLRRRRL with GET_HAM_LLLRRRRL's keep rule and column sort."""
    from dmrg_c_gb300 import sb_models
    g = golden("sb_hubbard.npz")
    m = sb_models.small_hubbard_model(tag == "pbc")
    assert int(m.inv.astype(np.int64).sum()) == int(g[f"{tag}_inv_checksum"])
    row, col, val = oracle.sb_build(m)
    assert np.array_equal(row, g[f"{tag}_row"])
    assert np.array_equal(col, g[f"{tag}_col"])
    assert np.array_equal(val.view(np.int64), g[f"{tag}_val"].view(np.int64))


def test_live_reference_superblock_build(ref):
    from dmrg_c_gb300 import sb_models, superblock, workloads
    qb = workloads._block_labels(30, 5, 5.0, 1.0, 0.8, 11)
    sb = superblock.synthetic_superblock(30, 4, qb, workloads.hubbard_site_labels(), 10 * workloads.QN_SCALE, nnz_lllr=1,
                                         nnz_lrrl=1, seed=12, with_sign=True)
    m = sb_models.hubbard_superblock_model(sb, qb, seed=13, per_row=4, pbc=True, U=2.5, t1=-0.7)
    a = ref.sb_build(m)
    b = ref.ref_sb_build(m)
    assert all(np.array_equal(x.view(np.int64) if x.dtype == np.float64 else x,
                              y.view(np.int64) if y.dtype == np.float64 else y) for x, y in zip(a, b))


@pytest.mark.parametrize("case", ["q1", "q2"])
def test_superblock_basis_matches_reference_golden(oracle, case):
    """The numpy restatement of GET_BASIS_SUPERBLOCK orders the states exactly as the reference's
    DMRG_QUICK_SORT_BASIS_Q1 / _Q2 do (fixture made by the reference's own sort)."""
    g = golden("sb_basis.npz")
    if case == "q1":
        a = oracle.sb_basis(40, 36, 2, (g["q1_LL"], g["q1_RR"], g["q1_site"]), None, (int(g["q1_target"]), 0))
    else:
        a = oracle.sb_basis(48, 44, 4, (g["q2_ne_LL"], g["q2_ne_RR"], g["q2_ne_site"]),
                            (g["q2_sz_LL"], g["q2_sz_RR"], g["q2_sz_site"]), tuple(int(t) for t in g["q2_targets"]))
    assert np.array_equal(np.stack(a[:4]), g[f"{case}_states"])
    assert np.array_equal(a[4], g[f"{case}_inv"])


def _obs_problem():
    from dmrg_c_gb300 import sb_models
    g = golden("sb_obs.npz")
    return sb_models.ObservableProblem.from_arrays(g), g


def test_observable_sectors_in_reference_order(oracle):
    """Every sector of the observable problem is laid out in the order the reference's sort gives
    (the numpy restatement of GET_BASIS_SUPERBLOCK is pinned by the basis fixture above)."""
    p, _ = _obs_problem()
    for q in (p.target, p.target - 1001, p.target + 999):
        LL, LR, RR, RL, inv = oracle.sb_basis(p.dim_LL, p.dim_RR, p.d, (p.q_LL, p.q_RR, p.q_site), None, (q, 0))
        assert np.array_equal(np.stack([LL, LR, RR, RL]), np.stack(p.sectors[q]))
        assert np.array_equal(inv, p.inv_sector(q))


def test_sb_vm_matches_reference_golden(oracle):
    """DMRG_V_M_*_Q0..Q4 restated (numpy) equal the reference's outputs bit for bit: in-sector
    block observables, and a c^dagger_up-type operator on each position with and without the
    fermion sign through a whole basis."""
    p, g = _obs_problem()
    v = g["v"]
    q0 = p.target
    st, inv0 = p.sectors[q0], p.inv_sector(q0)
    for pos, op in ((0, p.ops["LL"][0]), (1, p.ops["On"]), (2, p.ops["RR"][1]), (3, p.ops["On"])):
        y = oracle.sb_vm(st, inv0, p.dim_RR, p.d, op, pos, v)
        assert np.array_equal(y.view(np.int64), g[f"q0_{oracle.SB_NAMES[pos]}"].view(np.int64))
    q_out = q0 - 1001
    shift = {0: p.ops["CdLL"][0], 1: p.ops["CdOn"], 2: p.ops["CdRR"][0], 3: p.ops["CdOn"]}
    checked = 0
    for key in g.keys():
        if key[0] == "q" and key[1] in "1234" and key.count("_") == 2:
            _, name, sign = key.split("_")
            pos = oracle.SB_NAMES.index(name)
            y = oracle.sb_vm(p.sectors[q_out], p.inv, p.dim_RR, p.d, shift[pos], pos, v, ele=p.ele if sign == "1" else None)
            assert np.array_equal(y.view(np.int64), g[key].view(np.int64)), key
            checked += 1
    assert checked == 25
    # the sign matters in this case
    assert not np.array_equal(g["q1_RL_0"], g["q1_RL_1"])


def test_sb_expectation_matches_reference_golden(oracle):
    """DMRG_EXPECTATION_ONSITE / _INTERSITE_Q0 restated: the V_M products dotted with the
    vector (or with the origin's product); within 1e-12 of the reference's sums."""
    p, g = _obs_problem()
    v = g["v"]
    st, inv0 = p.sectors[p.target], p.inv_sector(p.target)
    LLs, RRs, On = p.ops["LL"], p.ops["RR"], p.ops["On"]
    terms = [(o, 0, 0) for o in LLs] + [(On, 1, 0), (On, 3, 0)] + [(o, 2, 0) for o in RRs[::-1]]
    e = oracle.sb_expect(st, inv0, p.dim_RR, p.d, terms, v, [v])
    scale = float(np.dot(np.abs(v), np.abs(v))) * 10
    assert np.allclose(e, g["onsite"], rtol=0, atol=1e-12 * scale)
    for origin in (0, 1, len(LLs)):
        t1 = oracle.sb_vm(st, inv0, p.dim_RR, p.d, LLs[origin] if origin < len(LLs) else On, 0 if origin < len(LLs) else 1, v)
        assert np.array_equal(t1, g[f"inter{origin}_t1"])
        cf = p.ops["CF"][origin:] if origin < len(LLs) else []
        terms = [(o, 0, 0) for o in cf] + [(On, 1, 1), (On, 3, 1)] + [(o, 2, 1) for o in RRs[::-1]]
        e = oracle.sb_expect(st, inv0, p.dim_RR, p.d, terms, v, [v, t1])
        ref = g[f"inter{origin}"][:len(terms)]
        assert np.allclose(e, ref, rtol=0, atol=1e-12 * scale), origin


def test_density_matrix_matches_reference_golden(oracle):
    """DMRG_GET_DENSITY_MATRIX restated (numpy, sums in the reference's order) equals the
    reference's blocks bit for bit on the observable problem's target sector."""
    p, g = _obs_problem()
    st, inv0 = p.sectors[p.target], p.inv_sector(p.target)
    lllr = oracle.lllr_list(p.q_LL, p.q_site, st)
    blocks = oracle.density_matrix_blocks(st, inv0, p.d, p.dim_RR, g["v"], lllr)
    got = np.concatenate([b.ravel() for b in blocks])
    assert np.array_equal(got.view(np.int64), g["dm_blocks"].view(np.int64))
    assert sum(b.shape[0] for b in blocks) == p.dim_LL * p.d


def _golden_system_info(g, tag, max_dim):
    pre = f"si_{tag}_{max_dim}_"
    nq = 1 if tag == "q1" else 2
    return dict(dim_renorm=int(g[pre + "dim_renorm"]), val=g[pre + "val"], sum_val=float(g[pre + "sum_val"]),
                tr_error=float(g[pre + "tr_error"]), col_ptr=g[pre + "col_ptr"], rows=g[pre + "rows"], vals=g[pre + "vals"],
                qn=[g[pre + f"qn{k}"] for k in range(nq)])


def _system_info_qns(p, lllr, tag):
    lab = lllr[3]
    N = np.rint(lab / 1000).astype(np.int32)
    return [lab.astype(np.int32)] if tag == "q1" else [N, (lab - N * 1000).astype(np.int32)]


@pytest.mark.parametrize("tag", ["q1", "q2"])
@pytest.mark.parametrize("max_dim", [20, 10000])
def test_system_info_matches_reference_golden(oracle, tag, max_dim):
    """DMRG_GET_SYSTEM_INFO_Q1 / _Q2 restated (numpy's eigensolver for LAPACK's): the same kept
    dimension, quantum numbers and sparsity as the reference, spectra within 1e-13 * |v|^2 and
    the same kept subspace in every block."""
    p, g = _obs_problem()
    st, inv0 = p.sectors[p.target], p.inv_sector(p.target)
    lllr = oracle.lllr_list(p.q_LL, p.q_site, st)
    got = oracle.system_info(_system_info_qns(p, lllr, tag), st, inv0, p.d, p.dim_RR, g["v_unit"], lllr, max_dim)
    assert oracle.same_truncation(got, _golden_system_info(g, tag, max_dim)) == []


def test_ed_expectation_matches_reference_golden(oracle):
    """EXACT_EXPECTATION_ONSITE / _INTERSITE_Q0: the oracle's site products dotted with the vector
    (or with the origin's product) agree with the reference within 1e-12 of |v|^2; the work
    vectors are the products themselves."""
    g = golden("ed_obs_hubbard6.npz")
    basis, vec = g["basis"], g["vec"]
    dens = abi.Crs(np.arange(5), np.arange(4, dtype=np.int32), np.array([0.0, 1.0, 1.0, 2.0]))
    nup = abi.Crs(np.arange(5), np.arange(4, dtype=np.int32), np.array([0.0, 1.0, 0.0, 1.0]))
    tol = 1e-12 * float(vec @ vec) * 4
    on = [vec @ oracle.site_apply(dens, basis, basis, 4, s, vec) for s in range(6)]
    assert np.allclose(on, g["onsite"], rtol=0, atol=tol)
    assert np.array_equal(oracle.site_apply(dens, basis, basis, 4, 5, vec), g["onsite_t"])
    for start, end in ((0, 6), (2, 5), (3, 3)):
        t1 = oracle.site_apply(nup, basis, basis, 4, start, vec)
        assert np.array_equal(t1, g[f"inter_{start}_{end}_t1"])
        got = [t1 @ oracle.site_apply(dens, basis, basis, 4, s, vec) for s in range(start, end)]
        assert np.allclose(got, g[f"inter_{start}_{end}"], rtol=0, atol=tol)


def test_renorm_product_matches_reference_golden(oracle):
    """CRS_CRS_CCS_PRODUCT restated (numpy, the reference's summation order) equals the reference's
    intermediate (CCS) and result (CRS) bit for bit, exact cancellations dropped."""
    g = golden("renorm.npz")
    M1, M2, M3 = renorm_operands_from_golden(g)
    got = oracle.crs_crs_ccs(M1, M2, M3)
    for a, name in zip(got, ("w_col", "w_row", "w_val", "o_row", "o_col", "o_val")):
        a = np.asarray(a)
        b = g[name]
        assert a.shape == b.shape, name
        assert np.array_equal(a.view(np.int64) if a.dtype == np.float64 else a.astype(np.int64),
                              b.view(np.int64) if b.dtype == np.float64 else b.astype(np.int64)), name


def test_dmrg_step_lllr_list_is_the_oracles(oracle):
    """The post-solve driver lays out the LLLR list exactly as the oracle (pinned to the reference)
    does."""
    from dmrg_c_gb300 import dmrg_step, superblock, workloads
    qb = workloads._block_labels(48, 9, 9.0, 1.0, 0.9, 7)
    qs = workloads.hubbard_site_labels()
    sb = superblock.synthetic_superblock(48, 4, qb, qs, 20 * workloads.QN_SCALE, nnz_lllr=6, nnz_lrrl=2, seed=8)
    states = (sb.LL, sb.LR, sb.RR, sb.RL)
    a, b = dmrg_step.lllr_list(qb, qs, states), oracle.lllr_list(qb, qs, states)
    for x, y in zip(a, b[:4]):
        assert np.array_equal(x, y)


def test_live_reference_vm_whole_basis(ref):
    """The reference's DMRG_V_M_*_Q1..Q4 on another seeded problem, called through the ctypes
    DMRG_WHOLE_BASIS_Qk mirrors, equal the numpy restatement bit for bit (signs included)."""
    from dmrg_c_gb300 import sb_models
    p = sb_models.random_observable_problem(dim_LL=20, dim_RR=18, seed=13)
    lib = ref.load_ref()
    v = np.random.default_rng(5).standard_normal(len(p.sectors[p.target][0]))
    q_out = p.target - 1001
    shift = {0: p.ops["CdLL"][0], 1: p.ops["CdOn"], 2: p.ops["CdRR"][0], 3: p.ops["CdOn"]}
    n = 0
    for k in (1, 2, 3, 4):
        wb = p.whole_basis(k)
        for pos, op in shift.items():
            if k == 4 and pos < 2:
                continue
            for sign in ((False,) if pos == 0 else (False, True)):
                got = ref.call_vm_whole(lib, wb, p.index(q_out, k), op, pos, v, ele=p.ele, sign=sign)
                want = ref.sb_vm(p.sectors[q_out], p.inv, p.dim_RR, p.d, op, pos, v, ele=p.ele if sign else None)
                assert np.array_equal(got.view(np.int64), want.view(np.int64)), (k, pos, sign)
                n += 1
    assert n == 25


def test_live_reference_truncation_and_renorm(ref):
    """The reference's DMRG_GET_SYSTEM_INFO_Q2 and CRS_CRS_CCS_PRODUCT on a superblock ground state:
    the restatements agree (the truncation as a truncation, the product bit for bit)."""
    import scipy.sparse as sp
    from dmrg_c_gb300 import superblock, workloads
    qb = workloads._block_labels(40, 8, 8.0, 1.0, 0.9, 17)
    qs = workloads.hubbard_site_labels()
    sb = superblock.synthetic_superblock(40, 4, qb, qs, 18 * workloads.QN_SCALE, nnz_lllr=6, nnz_lrrl=2, seed=19)
    w, V = np.linalg.eigh(sb.explicit().toarray())
    psi = V[:, 0]
    states = (sb.LL, sb.LR, sb.RR, sb.RL)
    lllr = ref.lllr_list(qb, qs, states)
    N = np.rint(lllr[3] / 1000).astype(np.int32)
    qns = [N, (lllr[3] - N * 1000).astype(np.int32)]
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    got = ref.call_system_info(ref.load_ref(), qns, states, sb.inv, 40, 40, 4, psi, lllr, 30, libc.free)
    assert ref.same_truncation(got, ref.system_info(qns, states, sb.inv, 4, 40, psi, lllr, 30)) == []
    nr, L = got["dim_renorm"], len(lllr[0])
    T = sp.csc_matrix((got["vals"], got["rows"], got["col_ptr"]), shape=(L, nr))
    O = sp.random(L, L, density=0.05, random_state=3, format="csr")
    M1, M2, M3 = abi.Crs.from_scipy(sp.csr_matrix(T.T)), abi.Crs.from_scipy(O + O.T), abi.Ccs.from_scipy(T)
    r = ref.call_crs_crs_ccs(ref.load_ref(), M1, M2, M3, L * nr, nr * nr)
    for x, y in zip(r[:6], ref.crs_crs_ccs(M1, M2, M3)):
        x, y = np.asarray(x), np.asarray(y)
        assert np.array_equal(x.astype(np.float64).view(np.int64), y.astype(np.float64).view(np.int64))


def test_oracle_site_apply_matches_reference_q1_q3_golden(oracle):
    """The oracle's site-operator application against the reference's EXACT_V_M_Q1 / _Q3 (golden)."""
    from conftest import vm_whole_sectors
    g = golden("vm_q13.npz")
    q1, _, q3, _ = vm_whole_sectors()
    raise_op = abi.Crs(np.array([0, 0, 1]), np.array([0], np.int32), np.array([1.5]), n=2)
    diag_op = abi.Crs(np.array([0, 1, 2]), np.array([0, 1], np.int32), np.array([-0.5, 0.75]), n=2)
    for site in (0, 3, 7):
        np.testing.assert_array_equal(oracle.site_apply(raise_op, q1[(4,)], q1[(3,)], 2, site, g["q1_v3"]),
                                      g[f"q1_raise_site{site}"])
        np.testing.assert_array_equal(oracle.site_apply(diag_op, q1[(4,)], q1[(4,)], 2, site, g["q1_v4"]),
                                      g[f"q1_diag_site{site}"])
    op = abi.Crs(g["q3_op_row"], g["q3_op_col"], g["q3_op_val"], n=4)
    for site in (0, 2, 3):
        for sign in (0, 1):
            ne = np.array([0, 1, 1, 2], np.int32) if sign else None
            np.testing.assert_array_equal(oracle.site_apply(op, q3[(2, 1, 0)], q3[(1, 1, 0)], 4, site, g["q3_v"], n_ele=ne),
                                          g[f"q3_site{site}_sign{sign}"])
