"""GPU parity of the SML path (SpMV, Lanczos, inverse iteration, CG, MINRES, residual) through
the C-ABI, against the reference's golden outputs and the oracle.

Tolerances: SpMV results within 1e-13 relative to max|y| (different summation order);
eigenvalues within 1e-12 relative; eigenvectors |<psi|psi_ref>| >= 1 - 1e-9; structure
(row offsets, columns) bit-exact."""
import ctypes as C
import subprocess
import sys
import textwrap

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import ROOT, golden
from dmrg_c_gb300 import abi, ed_models

pytestmark = pytest.mark.gpu


def sml_inputs():
    g = golden("sml_random1500.npz")
    return g, abi.Crs(g["low_row"], g["low_col"], g["low_val"]), abi.Crs(g["full_row"], g["full_col"], g["full_val"])


def rel_close(a, b, tol=1e-13):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() <= tol * scale


def test_spmv_golden(gpu):
    g, low, full = sml_inputs()
    ms = gpu.DeviceMatrix(low, gpu.DG_STORE_LOWER_DIAG_LAST)
    mf = gpu.DeviceMatrix(full, gpu.DG_STORE_FULL)
    assert ms.nnz == full.nnz and mf.nnz == full.nnz
    assert rel_close(ms.spmv(g["x"]), g["spmv_sym"])
    assert rel_close(mf.spmv(g["x"]), g["spmv_full"])


def test_lower_to_full_expansion_bit_exact(gpu, rng):
    A = sp.random(3000, 3000, density=0.003, random_state=5)
    A = (A + A.T).tocsr()
    A.setdiag(rng.standard_normal(3000))
    A.sort_indices()
    m = gpu.DeviceMatrix(abi.lower_diag_last(A), gpu.DG_STORE_LOWER_DIAG_LAST)
    row, col, val = m.download()
    assert np.array_equal(row, A.indptr) and np.array_equal(col, A.indices)
    assert np.array_equal(val, A.data)


@pytest.mark.parametrize("lanes", [1, 2, 4, 8, 16, 32])
def test_spmv_all_launch_shapes_and_determinism(gpu, oracle, rng, lanes):
    A = sp.random(4097, 4097, density=0.01, random_state=lanes)
    A = (A + A.T).tocsr()
    full = abi.Crs.from_scipy(A)
    m = gpu.DeviceMatrix(full)
    m.set_shape(lanes, 37)
    x = rng.standard_normal(4097)
    y1, y2 = m.spmv(x), m.spmv(x)
    assert np.array_equal(y1, y2)
    assert rel_close(y1, oracle.spmv(full, x, False))
    ys = m.spmv(x, sigma=0.75)
    assert rel_close(ys, y1 + 0.75 * x, 1e-13)


@pytest.mark.parametrize("n", [1, 2, 3, 31, 33, 1000])
def test_spmv_edge_sizes(gpu, oracle, rng, n):
    A = sp.random(n, n, density=min(1.0, 5.0 / n), random_state=n)
    A = (A + A.T).tocsr()
    A.setdiag(rng.standard_normal(n))
    low = abi.lower_diag_last(A)
    x = rng.standard_normal(n)
    m = gpu.DeviceMatrix(low, gpu.DG_STORE_LOWER_DIAG_LAST)
    assert rel_close(m.spmv(x), oracle.spmv(low, x, True))


def test_spmv_device_pointers(gpu, rng):
    torch = pytest.importorskip("torch")
    g, low, full = sml_inputs()
    m = gpu.DeviceMatrix(full)
    x = torch.tensor(g["x"], device="cuda")
    y = torch.empty_like(x)
    m.spmv(x, y)
    torch.cuda.synchronize()
    assert rel_close(y.cpu().numpy(), g["spmv_full"])


def test_matrix_validation_errors(gpu):
    bad = abi.Crs(np.array([0, 1, 2]), np.array([0, 0], np.int32), np.array([1.0, 2.0]))   # row 1 lacks its diagonal
    with pytest.raises(gpu.DgError) as e:
        gpu.DeviceMatrix(bad, gpu.DG_STORE_LOWER_DIAG_LAST)
    assert e.value.code == 7
    bad2 = abi.Crs(np.array([0, 1, 2]), np.array([0, 5], np.int32), np.array([1.0, 2.0]))  # column out of range
    with pytest.raises(gpu.DgError):
        gpu.DeviceMatrix(bad2)


def test_matrix_create_rejects_device_arrays(gpu):
    """The host-array entry reads row[n] on the host: device arrays get DG_ERR_ARG, not a crash."""
    torch = pytest.importorskip("torch")
    g, low, full = sml_inputs()
    dev = [torch.from_numpy(a).cuda() for a in (full.row, full.col, full.val)]
    lib = gpu.load()
    h = C.c_void_p()
    rc = lib.dg_matrix_create(full.n, C.cast(dev[0].data_ptr(), C.POINTER(C.c_long)), C.cast(dev[1].data_ptr(), C.POINTER(C.c_int)),
                              C.cast(dev[2].data_ptr(), C.POINTER(C.c_double)), gpu.DG_STORE_FULL, gpu.DG_VALUES_F64, C.byref(h))
    assert rc == 1 and not h.value
    assert b"dg_matrix_create_device" in lib.dg_last_error()


@pytest.mark.parametrize("name,sym,slow", [("lanczos_sym", True, False), ("lanczos_slow_sym", True, True),
                                           ("lanczos", False, False), ("lanczos_slow", False, True)])
def test_lanczos_golden(gpu, name, sym, slow):
    g, low, full = sml_inputs()
    m = gpu.DeviceMatrix(low if sym else full, gpu.DG_STORE_LOWER_DIAG_LAST if sym else gpu.DG_STORE_FULL)
    p = gpu.default_params(lanczos_slow=int(slow))
    v, info = gpu.ground_state(m, p, guess=g["guess"], lanczos_only=True)
    E = float(g[name + "_E"])
    assert info.converged
    assert abs(info.eig_val - E) <= 1e-12 * abs(E)
    assert abs(info.lanczos_steps - int(g[name + "_steps"])) <= 3
    assert abs(abs(v @ g[name + "_vec"]) - 1) < 1e-9


def test_ground_state_golden(gpu):
    g, low, full = sml_inputs()
    m = gpu.DeviceMatrix(low, gpu.DG_STORE_LOWER_DIAG_LAST)
    v, info = gpu.ground_state(m, gpu.default_params(), guess=g["guess"])
    assert info.ii_converged and info.error < 1e-9
    assert abs(abs(v @ g["ii_sym_vec"]) - 1) < 1e-12
    assert info.ii_steps == int(g["ii_sym_iters"])


def test_lanczos_restart_matches_oracle(gpu, oracle):
    g, low, full = sml_inputs()
    m = gpu.DeviceMatrix(low, gpu.DG_STORE_LOWER_DIAG_LAST)
    p = gpu.default_params(lanczos_block_step=30)
    v, info = gpu.ground_state(m, p, guess=g["guess"], lanczos_only=True)
    rc, out, vo = oracle.lanczos(low, True, guess=g["guess"], max_block_step=30)
    assert out.converged and info.converged
    assert abs(info.eig_val - out.eig_val) < 1e-12 * abs(out.eig_val)
    assert abs(abs(v @ vo) - 1) < 1e-9


def test_lanczos_tight(gpu, oracle):
    g, low, full = sml_inputs()
    m = gpu.DeviceMatrix(low, gpu.DG_STORE_LOWER_DIAG_LAST)
    v, info = gpu.ground_state(m, gpu.default_params(lanczos_tight=1, lanczos_acc=1e-10), guess=g["guess"],
                               lanczos_only=True)
    rc, out, vo = oracle.lanczos(low, True, guess=g["guess"], tight=True, acc=1e-10)
    assert abs(info.eig_val - out.eig_val) < 1e-12 * abs(out.eig_val)
    assert abs(info.lanczos_steps - out.steps) <= 2


def test_seeded_start_matches_oracle(gpu, oracle):
    """Guess "No": GPU and oracle draw the same seeded start vector."""
    g, low, full = sml_inputs()
    m = gpu.DeviceMatrix(full)
    v, info = gpu.ground_state(m, gpu.default_params(seed=77), lanczos_only=True)
    rc, out, vo = oracle.lanczos(full, False, seed=77)
    assert abs(info.eig_val - out.eig_val) < 1e-12 * abs(out.eig_val)
    assert abs(info.lanczos_steps - out.steps) <= 2
    assert abs(abs(v @ vo) - 1) < 1e-9


def test_lanczos_nonconvergence_status(gpu):
    g, low, full = sml_inputs()
    m = gpu.DeviceMatrix(low, gpu.DG_STORE_LOWER_DIAG_LAST)
    with pytest.raises(gpu.DgError) as e:
        gpu.ground_state(m, gpu.default_params(lanczos_max_step=5), guess=g["guess"], lanczos_only=True)
    assert e.value.code == 4


def test_dense_path(gpu):
    A = sp.random(300, 300, density=0.05, random_state=7)
    A = (A + A.T).tocsr()
    m = gpu.DeviceMatrix(abi.lower_diag_last(A), gpu.DG_STORE_LOWER_DIAG_LAST)
    v, info = gpu.ground_state(m, gpu.default_params(), lanczos_only=True)
    w, Z = np.linalg.eigh(A.toarray())
    assert info.dense and abs(info.eig_val - w[0]) < 1e-12 * max(1.0, abs(w[0]))
    assert abs(abs(v @ Z[:, 0]) - 1) < 1e-9


def test_cg_minres_golden(gpu):
    g = golden("sml_random1500.npz")
    B = abi.Crs(g["B_row"], g["B_col"], g["B_val"])
    m = gpu.DeviceMatrix(B, gpu.DG_STORE_LOWER_DIAG_LAST)
    x = g["x0"].copy()
    rc, it = gpu.linear_solve(m, g["b"], x, acc=1e-10, max_step=1000)
    assert rc == 0 and abs(it - int(g["cg_iters"])) <= 1
    np.testing.assert_allclose(x, g["cg_x"], rtol=0, atol=1e-8)
    x = g["x0"].copy()
    rc, it = gpu.linear_solve(m, g["b"], x, acc=1e-6, max_step=1000, minres=True)
    assert rc == 0 and abs(it - int(g["mr_iters"])) <= 1
    np.testing.assert_allclose(x, g["mr_x"], rtol=0, atol=1e-6)


def test_cg_iteration_limit(gpu):
    g = golden("sml_random1500.npz")
    m = gpu.DeviceMatrix(abi.Crs(g["B_row"], g["B_col"], g["B_val"]), gpu.DG_STORE_LOWER_DIAG_LAST)
    x = g["x0"].copy()
    rc, it = gpu.linear_solve(m, g["b"], x, acc=1e-30, max_step=7)
    assert rc == 4 and it == 7


def test_residual_golden(gpu):
    g, low, full = sml_inputs()
    E = float(g["lanczos_sym_E"])
    m = gpu.DeviceMatrix(low, gpu.DG_STORE_LOWER_DIAG_LAST)
    assert gpu.residual_l1(m, g["lanczos_sym_vec"], E) == pytest.approx(float(g["conv_sym"]), rel=1e-6)


def test_heisenberg16_energy(gpu, oracle):
    g = golden("xxz16.npz")
    basis, row, col, val = oracle.ed_build(ed_models.xxz_chain(16))
    m = gpu.DeviceMatrix(abi.Crs(row, col, val))
    v, info = gpu.ground_state(m, gpu.default_params(), guess=g["guess"])
    assert abs(info.eig_val - float(g["E"])) < 1e-12 * abs(float(g["E"]))
    assert info.ii_converged


# ---- drop-in entry points (reference names, reference structs) ------------------------------

def test_dropin_lanczos_sym_and_ii(gpu, in_tmp):
    lib = gpu.load()
    g, low, full = sml_inputs()
    vec = g["guess"].copy()
    val = np.zeros(1)
    box = abi.BOX_LAN(M=low.ref, Eig_Vec=abi.ptr(vec, C.c_double), eig_val=abi.ptr(val, C.c_double), acc=1e-14,
                      min_step=1, max_step=800, max_block_step=800, p_threads=4, Guess=b"Yes", Type=b"Normal")
    lib.LANCZOS_SYM(C.byref(box))
    assert abs(val[0] - float(g["lanczos_sym_E"])) < 1e-12 * abs(val[0])
    steps = int((in_tmp / "SML_out" / "LANCZOS_SYM_Step.txt").read_text().split()[-1])
    assert abs(steps - int(g["lanczos_sym_steps"])) <= 3
    before = low.val.copy()
    ev = val.copy()
    ii = abi.BOX_II(M=low.ref, ii_acc=1e-9, ii_diag_add=1e-11, ii_max_step=3, cg_acc=1e-7, cg_max_step=1000,
                    Eig_Vec=abi.ptr(vec, C.c_double), Eig_Val=abi.ptr(ev, C.c_double), p_threads=4, Type=b"CG")
    lib.INVERSE_ITERATION_SYM(C.byref(ii))
    assert ii.error < 1e-9
    assert np.array_equal(before, low.val)          # the caller's matrix is untouched
    assert (in_tmp / "SML_out" / "Inv_iter_step.txt").exists()
    assert abs(abs(vec @ g["ii_sym_vec"]) - 1) < 1e-12


def test_dropin_diagonalize_superblock(gpu, in_tmp):
    lib = gpu.load()
    g, low, full = sml_inputs()
    par = abi.DMRG_PARAMETER()
    par.Diag_Method, par.Lan_Con, par.II_Type = b"Lanczos", b"Normal", b"CG"
    par.diag_acc, par.diag_min_step, par.diag_max_step = 1e-14, 1, 800
    par.cg_acc, par.cg_max_step = 1e-7, 1000
    par.inv_iter_acc, par.inv_iter_diag_add, par.inv_iter_max_step = 1e-9, 1e-11, 3
    gs = np.zeros(low.n)
    st = abi.DMRG_STATUS()
    st.GS_Vec = abi.ptr(gs, C.c_double)
    tm = abi.DMRG_TIME()
    lib.DMRG_DIAGONALIZE_SUPERBLOCK_SYM(low.ref, C.byref(tm), C.byref(par), C.byref(st), 8)
    assert abs(st.gs_val - float(g["lanczos_sym_E"])) < 1e-12 * abs(st.gs_val)
    assert st.gs_error < 1e-9 and tm.diag > 0 and tm.inv_iter > 0
    assert abs(abs(gs @ g["ii_sym_vec"]) - 1) < 1e-9


def test_dropin_cg_minres_converge(gpu, in_tmp):
    lib = gpu.load()
    g = golden("sml_random1500.npz")
    B = abi.Crs(g["B_row"], g["B_col"], g["B_val"])
    b = g["b"].copy()
    for minres, key in ((False, "cg"), (True, "mr")):
        x = g["x0"].copy()
        box = abi.BOX_CG(M=B.ref, acc=1e-10 if not minres else 1e-6, Vec=abi.ptr(b, C.c_double),
                         Out_Vec=abi.ptr(x, C.c_double), max_step=1000, p_threads=2)
        (lib.MINIMUM_RESIDUAL_SYM if minres else lib.CONJUGATE_GRADIENT_SYM)(C.byref(box))
        np.testing.assert_allclose(x, g[key + "_x"], rtol=0, atol=1e-6 if minres else 1e-8)
    g2, low, full = sml_inputs()
    r = lib.CONVERGE_CHECK(full.ref, abi.ptr(g2["lanczos_sym_vec"].copy(), C.c_double), float(g2["lanczos_sym_E"]), 1)
    assert r == pytest.approx(float(g2["conv_full"]), rel=1e-6)
    y = np.zeros(full.n)
    lib.MATRIX_VECTOR_PRODUCT(full.ref, abi.ptr(g2["x"].copy(), C.c_double), abi.ptr(y, C.c_double), 1)
    assert rel_close(y, g2["spmv_full"])


def test_dropin_exact_diagonalize(gpu, oracle, in_tmp):
    lib = gpu.load()
    g = golden("xxz16.npz")
    basis, row, col, val = oracle.ed_build(ed_models.xxz_chain(16))
    H = abi.Crs(row, col, val)
    vec = np.zeros(len(basis))
    value, error = np.zeros(1), np.zeros(1)
    vecs = (C.POINTER(C.c_double) * 1)(abi.ptr(vec, C.c_double))
    info = abi.EXACT_HAM_INFO(dim=0, diag_num=1, Vector=C.cast(vecs, C.POINTER(C.POINTER(C.c_double))),
                              Value=abi.ptr(value, C.c_double), Error=abi.ptr(error, C.c_double), Ham=H.ref)
    par = abi.EXACT_PARAMETER(diag_num=1, Diag_Method=b"Lanczos_Slow", diag_acc=1e-14, diag_min_step=1,
                              diag_max_step=800, cg_acc=1e-7, cg_max_step=1000, inv_iter_acc=1e-9,
                              inv_iter_diag_add=1e-11, inv_iter_max_step=3)
    lib.EXACT_DIAGONALIZE_HAMILTONIAN(C.byref(info), C.byref(par), C.byref(abi.EXACT_TIME()), 4)
    assert abs(value[0] - float(g["E"])) < 1e-12 * abs(value[0])
    assert error[0] < 1e-8 and info.dim == len(basis)


def test_dropin_fatal_error_exits(gpu, tmp_path):
    """Reference behaviour: an invalid Guess string prints, logs to SML_out/error.txt and exits(1)."""
    code = textwrap.dedent(f"""
        import sys, ctypes as C, numpy as np
        sys.path.insert(0, {str(ROOT)!r})
        from dmrg_c_gb300 import abi, lib
        L = lib.load()
        crs = abi.Crs(np.array([0, 1, 2]), np.array([0, 1], np.int32), np.array([1.0, 2.0]))
        v = np.ones(2); e = np.zeros(1)
        box = abi.BOX_LAN(M=crs.ref, Eig_Vec=abi.ptr(v, C.c_double), eig_val=abi.ptr(e, C.c_double), acc=1e-14,
                          min_step=1, max_step=10, max_block_step=10, p_threads=1, Guess=b"Maybe", Type=b"Normal")
        L.LANCZOS_SYM(C.byref(box))
        print("not reached")
    """)
    r = subprocess.run([sys.executable, "-c", code], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 1
    assert "Error in LANCZOS_SYM" in r.stdout and "not reached" not in r.stdout
    assert "Box->Guess=Maybe is error" in (tmp_path / "SML_out" / "error.txt").read_text()


def _sell_cases(oracle, rng):
    cases = []
    A = sp.random(5000, 5000, density=0.002, random_state=3, format="csr")
    A = A.tolil()
    A[17, :4000] = rng.standard_normal(4000)          # one dense row
    A = A.tocsr()
    A.eliminate_zeros()
    cases.append(("dense_row", abi.Crs.from_scipy(A), A))
    B = sp.random(3001, 3001, density=0.001, random_state=4, format="csr")   # many empty rows
    cases.append(("empty_rows", abi.Crs.from_scipy(B), B))
    basis, row, col, val = oracle.ed_build(ed_models.hubbard_chain(8, U=4.0))
    H = sp.csr_matrix((val, col, row), shape=(len(basis), len(basis)))
    cases.append(("hubbard8", abi.Crs(row, col, val), H))
    return cases


def test_sell_matches_csr_and_oracle(gpu, oracle, rng):
    for name, crs, A in _sell_cases(oracle, rng):
        m = gpu.DeviceMatrix(crs)
        fmt, stored = m.format()
        assert fmt == gpu.DG_FORMAT_SELL and stored >= crs.nnz
        x = rng.standard_normal(crs.n)
        y_sell = m.spmv(x)
        assert np.array_equal(y_sell, m.spmv(x)), name          # deterministic
        m.set_format(gpu.DG_FORMAT_CSR)
        y_csr = m.spmv(x)
        ref = A @ x
        assert rel_close(y_sell, ref), name
        assert rel_close(y_csr, ref), name
        m.set_format(gpu.DG_FORMAT_SELL)
        assert rel_close(m.spmv(x, sigma=-0.5), ref - 0.5 * x), name


def test_sell_solver_parity(gpu):
    """Lanczos + inverse iteration give the same eigenpair in both layouts."""
    g, low, full = sml_inputs()
    m = gpu.DeviceMatrix(low, gpu.DG_STORE_LOWER_DIAG_LAST)
    v1, i1 = gpu.ground_state(m, gpu.default_params(), guess=g["guess"])
    m.set_format(gpu.DG_FORMAT_CSR)
    v2, i2 = gpu.ground_state(m, gpu.default_params(), guess=g["guess"])
    assert abs(i1.eig_val - i2.eig_val) < 1e-12 * abs(i1.eig_val)
    assert abs(abs(v1 @ v2) - 1) < 1e-12


@pytest.mark.parametrize("ws", [1, 2, 4, 8])
def test_sell_warps_per_slice(gpu, oracle, rng, ws):
    for name, crs, A in _sell_cases(oracle, rng):
        m = gpu.DeviceMatrix(crs)
        x = rng.standard_normal(crs.n)
        for variant in range(4):
            m.set_sell_shape(ws, 53)
            m.set_sell_variant(variant)
            y = m.spmv(x)
            assert np.array_equal(y, m.spmv(x)), (name, variant)
            assert rel_close(y, A @ x), (name, variant)


def test_autotune_keeps_results(gpu, oracle, rng):
    for name, crs, A in _sell_cases(oracle, rng):
        m = gpu.DeviceMatrix(crs)
        r = m.autotune(iters=2)
        assert r.candidates >= 40 and r.ms > 0
        x = rng.standard_normal(crs.n)
        assert rel_close(m.spmv(x), A @ x), name
