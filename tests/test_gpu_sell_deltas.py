"""The 16-bit column-delta stream of the sliced-ELL layout (variants 5 and 6).

Each row's columns are stored as deltas from the previous column, restarted from a 32-bit
checkpoint every 32 elements; a gap of 65,536 columns or more is bridged by zero-valued elements.
With one warp per slice the delta variants add the same elements in the same order as the
register form with 8-element groups (variant 1) on the same layout, so products and solves are
bitwise the same; with several warps per slice each warp takes whole 32-element chunks, and the
products are checked against an exact product.  Matrices with unsorted rows get no delta stream,
and the delta variants are refused on them."""
import functools

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import GOLDEN
from dmrg_c_gb300 import abi, workloads

pytestmark = pytest.mark.gpu

V_U8, V_D8, V_TMA16 = 1, 5, 6


@functools.lru_cache(maxsize=1)
def _bridged(n=100_000, half=32, far=66_000, seed=5):
    """Rows of 2*half clustered columns around the diagonal plus one column `far` further on
    (mod n, never inside the cluster): for r < n - far the gap to the far column is >= 65,536
    and needs one bridge."""
    rng = np.random.default_rng(seed)
    r = np.arange(n)
    c = r[:, None] + np.arange(-half, half)[None, :]
    c = np.concatenate([c, ((r + far) % n)[:, None]], axis=1)
    rows = np.broadcast_to(r[:, None], c.shape)
    keep = (c >= 0) & (c < n)
    rows, cols = rows[keep], c[keep]
    A = sp.csr_matrix((rng.standard_normal(rows.size), (rows, cols)), shape=(n, n))
    A.sort_indices()
    return A


def _expected_bridges(A):
    d = np.diff(A.indices.astype(np.int64))
    first = np.zeros(A.nnz, bool)
    first[A.indptr[:-1][np.diff(A.indptr) > 0]] = True
    g = d[~first[1:]]
    return int(np.sum(np.maximum(0, (g - 1) // 65535)))


def _cases(oracle, rng):
    """(name, CRS, lower-triangle storage?)"""
    cases = []
    A = sp.random(5000, 5000, density=0.002, random_state=3, format="csr").tolil()
    A[17, :4000] = rng.standard_normal(4000)          # one dense row: 125 chunks in one slice
    A = A.tocsr()
    A.eliminate_zeros()
    A.sort_indices()
    cases.append(("dense_row", abi.Crs.from_scipy(A), False))
    B = sp.random(3001, 3001, density=0.001, random_state=4, format="csr")   # many empty rows
    B.sort_indices()
    cases.append(("empty_rows", abi.Crs.from_scipy(B), False))
    cases.append(("bridged", abi.Crs.from_scipy(_bridged()), False))
    cases.append(("xxz_superblock_m64", workloads.xxz_superblock_m64(0).explicit_lower(), True))
    return cases


def _matrix(gpu, crs, lower):
    return gpu.DeviceMatrix(crs, gpu.DG_STORE_LOWER_DIAG_LAST if lower else gpu.DG_STORE_FULL, gpu.DG_VALUES_BOTH)


@pytest.mark.parametrize("grid", [1, 7, 600])
def test_delta_product_is_bitwise_the_register_form(gpu, oracle, rng, monkeypatch, grid):
    monkeypatch.setenv("DG_SELL_DELTAS", "1")          # build the stream at every size
    for name, crs, lower in _cases(oracle, rng):
        m = _matrix(gpu, crs, lower)
        present, _ = m.sell_deltas()
        assert present, name
        x = rng.standard_normal(crs.n)
        x32 = x.astype(np.float32)
        out = {}
        for var in (V_U8, V_D8, V_TMA16):
            m.set_sell_shape(1, grid)
            m.set_sell_variant(var)
            out[var] = (m.spmv(x), m.spmv(x, sigma=-0.75), m.spmv_mixed(x32))
        for var in (V_D8, V_TMA16):
            for a, b in zip(out[V_U8], out[var]):
                assert np.array_equal(a, b), (name, var)
        assert m.sell_error() == 0


def test_bridges_counted_and_exact(gpu, rng, monkeypatch):
    """The bridged matrix: the bridge count is the one the gaps call for, and the product on
    the delta stream matches an exact (long double) product."""
    monkeypatch.setenv("DG_SELL_DELTAS", "1")
    A = _bridged()
    want = _expected_bridges(A)
    assert want > 10_000
    m = gpu.DeviceMatrix(abi.Crs.from_scipy(A), gpu.DG_STORE_FULL, gpu.DG_VALUES_BOTH)
    present, bridges = m.sell_deltas()
    assert present and bridges == want
    x = rng.standard_normal(A.shape[0])
    exact = (A.astype(np.longdouble) @ x.astype(np.longdouble)).astype(np.float64)
    for ws in (1, 2, 4, 8):
        m.set_sell_shape(ws, 300)
        m.set_sell_variant(V_D8)
        y = m.spmv(x)
        assert np.max(np.abs(y - exact)) <= 1e-13 * np.max(np.abs(exact))


@pytest.mark.parametrize("ws", [2, 4, 8])
def test_delta_product_several_warps(gpu, oracle, rng, monkeypatch, ws):
    """Warps of a slice take whole chunks: FP64 products against an exact product, FP32 ones
    against the FP64 product at FP32 accuracy, on every case (the dense row has 125 chunks)."""
    monkeypatch.setenv("DG_SELL_DELTAS", "1")
    for name, crs, lower in _cases(oracle, rng):
        m = _matrix(gpu, crs, lower)
        A = sp.csr_matrix((crs.val, crs.col, crs.row), shape=(crs.n, crs.n))
        if lower:
            A = A + sp.tril(A, -1).T
        x = rng.standard_normal(crs.n)
        exact = (A.astype(np.longdouble) @ x.astype(np.longdouble)).astype(np.float64)
        scale = max(1.0, np.max(np.abs(exact)))
        for var in (V_D8, V_TMA16):                   # with several warps variant 6 runs 5
            m.set_sell_shape(ws, 97)
            m.set_sell_variant(var)
            y = m.spmv(x)
            assert np.max(np.abs(y - exact)) <= 1e-13 * scale, (name, var)
            y32 = m.spmv_mixed(x.astype(np.float32))
            ref32 = A @ x.astype(np.float32).astype(np.float64)
            assert np.max(np.abs(y32 - ref32)) <= 1e-5 * max(1.0, np.max(np.abs(ref32))), (name, var)


def test_unsorted_rows_have_no_delta_stream(gpu, rng, monkeypatch):
    monkeypatch.setenv("DG_SELL_DELTAS", "1")
    A = sp.random(2000, 2000, density=0.01, random_state=9, format="csr")
    A.sort_indices()
    col = A.indices.copy()
    r = 5
    seg = slice(A.indptr[r], A.indptr[r + 1])
    assert seg.stop - seg.start >= 2
    col[seg] = col[seg][::-1]                          # one row in decreasing column order
    crs = abi.Crs(A.indptr.astype(np.int64), col.astype(np.int32), A.data.copy(), n=2000)
    m = gpu.DeviceMatrix(crs, gpu.DG_STORE_FULL, gpu.DG_VALUES_BOTH)
    assert m.sell_deltas() == (False, 0)
    with pytest.raises(gpu.DgError):
        m.set_sell_variant(V_D8)
    with pytest.raises(gpu.DgError):
        m.set_sell_mixed(1, V_TMA16)
    x = rng.standard_normal(2000)
    A2 = sp.csr_matrix((crs.val, crs.col, crs.row), shape=(2000, 2000))
    assert np.allclose(m.spmv(x), A2 @ x, rtol=0, atol=1e-12)


def test_small_matrices_skip_the_stream_by_default(gpu, monkeypatch):
    monkeypatch.delenv("DG_SELL_DELTAS", raising=False)
    m = _matrix(gpu, workloads.xxz_superblock_m64(0).explicit_lower(), True)
    assert m.sell_deltas() == (False, 0)


@pytest.mark.parametrize("mixed", [0, 2], ids=["fp64", "mixed2"])
def test_delta_solve_is_bitwise_the_register_form(gpu, mixed):
    """Lanczos + inverse iteration / refinement on the Hubbard m=512 superblock (L=64, U=4, 4th sweep) of the reference's own
    Hubbard run (n = 238,462, 236 elements a row; the stream is built by default at this size):
    with one warp per slice the same energy and vector bit for bit as variant 1."""
    from dmrg_c_gb300 import sb_models
    path = GOLDEN / "dmrg_hubbard_vf_sweep4.npz"
    if not path.exists():
        pytest.skip("no Hubbard m=512 superblock fixture")
    sb = sb_models.load_dmrg_superblock(path)
    s = gpu.SuperblockCRS(sb.model)
    res = {}
    for var in (V_U8, V_D8, V_TMA16):
        m = s.matrix(gpu.DG_VALUES_BOTH)
        present, bridges = m.sell_deltas()
        if var == V_U8:   # the device layout against its restatement on the matrix it holds
            from test_sell_layout import row_bridges, sell_stored
            row, col, _ = m.download()
            br = row_bridges(row, col)
            assert present and bridges == int(br.sum()) > 0
            assert m.format()[1] == sell_stored(np.diff(row) + br)
        m.set_sell_shape(1, 1216)
        m.set_sell_variant(var)
        p = gpu.default_params(mixed=mixed, seed=7, lanczos_acc=1e-14, cg_acc=1e-7, cg_max_step=2000)
        v, info = gpu.ground_state(m, p)
        res[var] = (info.eig_val, info.lanczos_steps, info.cg_steps, v)
        assert m.sell_error() == 0
    for var in (V_D8, V_TMA16):
        assert res[V_U8][:3] == res[var][:3]
        assert np.array_equal(res[V_U8][3], res[var][3])
    assert abs(res[V_D8][0] - sb.gs_val) <= 1e-10 * abs(sb.gs_val)
