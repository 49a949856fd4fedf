"""Block operators on superblock vectors and expectation values on the GPU
(DMRG_V_M_{LL,LR,RR,RL}_Q0..Q4, DMRG_EXPECTATION_ONSITE / _INTERSITE_Q0 and the dg_sb_vm /
dg_sb_expect device API) against the reference-made fixture and the oracle.

Products are compared bit for bit; expectation values within 1e-12 of sum_i |w_i||(Ov)_i|
(only the order of the final dot-product sums differs from the reference's)."""
import numpy as np
import pytest

from conftest import golden
from dmrg_c_gb300 import sb_models

pytestmark = pytest.mark.gpu

NAMES = ("LL", "LR", "RR", "RL")


def _bits(a):
    return np.asarray(a, np.float64).view(np.int64)


def _problem():
    g = golden("sb_obs.npz")
    return sb_models.ObservableProblem.from_arrays(g), g


def test_vm_dropins_vs_reference_golden(gpu, oracle):
    p, g = _problem()
    lib = gpu.load()
    v = g["v"]
    st, inv0 = p.sectors[p.target], p.inv_sector(p.target)
    for pos, op in ((0, p.ops["LL"][0]), (1, p.ops["On"]), (2, p.ops["RR"][1]), (3, p.ops["On"])):
        y = oracle.call_vm_q0(lib, st, inv0, p.dim_LL, p.dim_RR, p.d, op, pos, v)
        assert np.array_equal(_bits(y), _bits(g[f"q0_{NAMES[pos]}"])), pos
    q_out = p.target - 1001
    shift = {0: p.ops["CdLL"][0], 1: p.ops["CdOn"], 2: p.ops["CdRR"][0], 3: p.ops["CdOn"]}
    n = 0
    for k in (1, 2, 3, 4):
        wb = p.whole_basis(k)
        for pos, op in shift.items():
            for sign in (0, 1):
                key = f"q{k}_{NAMES[pos]}_{sign}"
                if key not in g:
                    continue
                y = oracle.call_vm_whole(lib, wb, p.index(q_out, k), op, pos, v, ele=p.ele, sign=bool(sign))
                assert np.array_equal(_bits(y), _bits(g[key])), key
                n += 1
    assert n == 25


def test_expectation_dropins_vs_reference_golden(gpu, oracle):
    p, g = _problem()
    lib = gpu.load()
    v = g["v"]
    st, inv0 = p.sectors[p.target], p.inv_sector(p.target)
    LLs, RRs, On = p.ops["LL"], p.ops["RR"], p.ops["On"]
    tol = 1e-12 * float(np.dot(np.abs(v), np.abs(v))) * 10
    out, temp = oracle.call_expectation_onsite(lib, st, inv0, p.dim_LL, p.dim_RR, p.d, LLs, On, RRs, v)
    assert np.allclose(out, g["onsite"], rtol=0, atol=tol)
    assert np.array_equal(_bits(temp), _bits(g["onsite_temp"]))
    for origin in (0, 1, len(LLs)):
        cf = p.ops["CF"][origin:] if origin < len(LLs) else p.ops["CF"][:1]
        out, t1, t2 = oracle.call_expectation_intersite_q0(lib, st, inv0, p.dim_LL, p.dim_RR, p.d, cf, LLs, On, RRs, origin, v)
        ref = g[f"inter{origin}"]
        m = ~np.isnan(ref)
        assert np.array_equal(np.isnan(out), ~m), origin          # the same entries written
        assert np.allclose(out[m], ref[m], rtol=0, atol=tol), origin
        assert np.array_equal(_bits(t1), _bits(g[f"inter{origin}_t1"]))
        assert np.array_equal(_bits(t2), _bits(g[f"inter{origin}_t2"]))
    # an origin past the LR site returns without writing
    out, t1, t2 = oracle.call_expectation_intersite_q0(lib, st, inv0, p.dim_LL, p.dim_RR, p.d, p.ops["CF"], LLs, On, RRs,
                                                       len(LLs) + 1, v)
    assert np.isnan(out).all() and np.isnan(t1).all() and np.isnan(t2).all()


@pytest.fixture(scope="module")
def big():
    """A larger problem (blocks of 72 / 64 states) for the device API."""
    return sb_models.random_observable_problem(dim_LL=72, dim_RR=64, n_LL=4, n_RR=4, per_row=9, seed=9, n_sites=7)


def _device_objects(gpu, p, q_out):
    out_b = gpu.superblock_states(p.sectors[q_out], p.dim_LL, p.dim_RR, p.d)
    inv_b = gpu.superblock_states(p.sectors[p.target], p.dim_LL, p.dim_RR, p.d, inv=p.inv)
    ops = [*p.ops["LL"], *p.ops["RR"], p.ops["On"], p.ops["CdLL"][0], p.ops["CdRR"][0], p.ops["CdOn"]]
    rows = [p.dim_LL] * len(p.ops["LL"]) + [p.dim_RR] * len(p.ops["RR"]) + [p.d, p.dim_LL, p.dim_RR, p.d]
    return out_b, inv_b, gpu.BlockOperators(ops, rows), ops


def test_device_vm_vs_oracle(gpu, oracle, big):
    import torch
    p = big
    rng = np.random.default_rng(3)
    nL = len(p.ops["LL"])
    nR = len(p.ops["RR"])
    # in-sector observables (Q0) and the sector-changing operator with the sign, host and device vectors
    for q_out, cases in ((p.target, [(0, 0), (2, nL), (1, nL + nR), (3, nL + nR)]),
                         (p.target - 1001, [(0, nL + nR + 1), (1, nL + nR + 3), (2, nL + nR + 2), (3, nL + nR + 3)])):
        out_b, inv_b, ops, host_ops = _device_objects(gpu, p, q_out)
        v = rng.standard_normal(len(p.sectors[p.target][0]))
        for pos, k in cases:
            for sign in (False, True):
                ele = p.ele if sign else None
                want = oracle.sb_vm(p.sectors[q_out], p.inv, p.dim_RR, p.d, host_ops[k], pos, v, ele=ele)
                got = gpu.sb_vm(out_b, inv_b, ops, k, pos, v, sign=sign, ele=p.ele)
                assert np.array_equal(_bits(got), _bits(want)), (q_out, pos, sign)
                vd = torch.from_numpy(v).cuda()
                yd = torch.empty(out_b.n, dtype=torch.float64, device="cuda")
                gpu.sb_vm(out_b, inv_b, ops, k, pos, vd, out=yd, sign=sign, ele=p.ele)
                assert np.array_equal(_bits(yd.cpu().numpy()), _bits(want))


def test_device_expect_vs_oracle(gpu, oracle, big):
    p = big
    rng = np.random.default_rng(4)
    out_b, inv_b, ops, host_ops = _device_objects(gpu, p, p.target)
    v = rng.standard_normal(out_b.n)
    v /= np.linalg.norm(v)
    w1 = rng.standard_normal(out_b.n)
    nL, nR = len(p.ops["LL"]), len(p.ops["RR"])
    terms = ([(0, k, 0, 0) for k in range(nL)] + [(1, nL + nR, 0, 1), (3, nL + nR, 0, 0)]
             + [(2, nL + k, 1, 1) for k in range(nR)])
    got = gpu.sb_expect(out_b, inv_b, ops, terms, v, v, w1, ele=p.ele)
    want = []
    for pos, k, sign, w in terms:
        y = oracle.sb_vm(p.sectors[p.target], p.inv, p.dim_RR, p.d, host_ops[k], pos, v, ele=p.ele if sign else None)
        want.append(np.dot((v, w1)[w], y))
        tol = 1e-12 * float(np.dot(np.abs((v, w1)[w]), np.abs(y))) + 1e-300
        assert abs(got[len(want) - 1] - want[-1]) <= tol, (pos, k, sign, w)
    # fixed-order sums: bitwise the same on every call
    again = gpu.sb_expect(out_b, inv_b, ops, terms, v, v, w1, ele=p.ele)
    assert np.array_equal(_bits(got), _bits(again))


def test_device_basis_feeds_observables(gpu, oracle, big):
    """A basis built on the device (dg_sb_basis_build) serves as both the states and the Inv table."""
    p = big
    b = gpu.SuperblockBasis(p.dim_LL, p.dim_RR, p.d, p.q_LL, p.q_RR, p.q_site, p.target)
    LL, LR, RR, RL, inv = b.download()
    assert np.array_equal(np.stack([LL, LR, RR, RL]), np.stack(p.sectors[p.target]))
    ops = gpu.BlockOperators([p.ops["LL"][1]], [p.dim_LL])
    v = np.random.default_rng(5).standard_normal(b.n)
    got = gpu.sb_vm(b, b, ops, 0, 0, v)
    want = oracle.sb_vm(p.sectors[p.target], p.inv_sector(p.target), p.dim_RR, p.d, p.ops["LL"][1], 0, v)
    assert np.array_equal(_bits(got), _bits(want))


def test_device_api_rejects_bad_input(gpu, big):
    p = big
    out_b, inv_b, ops, _ = _device_objects(gpu, p, p.target)
    v = np.zeros(out_b.n)
    with pytest.raises(gpu.DgError):
        gpu.sb_vm(out_b, inv_b, ops, 0, 0, v[:10])                 # Inv entries past the input vector
    with pytest.raises(gpu.DgError):
        gpu.sb_vm(out_b, inv_b, ops, 0, 2, v)                      # an LL operator on the RR position
    with pytest.raises(gpu.DgError):
        gpu.sb_vm(out_b, out_b, ops, 0, 0, v)                      # the states carry no Inv table
    with pytest.raises(gpu.DgError):
        gpu.sb_vm(out_b, inv_b, ops, len(p.ops["LL"]) + len(p.ops["RR"]), 3, v, sign=True, ele=None)   # sign without ele
    with pytest.raises(gpu.DgError):
        gpu.superblock_states([np.array([p.dim_LL], np.int16)] + [np.zeros(1, np.int16)] * 3, p.dim_LL, p.dim_RR, p.d)
    # an empty output sector is a no-op
    e = gpu.superblock_states([np.zeros(0, np.int16)] * 4, p.dim_LL, p.dim_RR, p.d)
    assert gpu.sb_vm(e, inv_b, ops, 0, 0, v).shape == (0,)
    assert np.array_equal(gpu.sb_expect(e, inv_b, ops, [(0, 0, 0, 0)], v, np.zeros(0)), [0.0])


def test_density_matrix_form_vs_oracle(gpu, oracle, big, monkeypatch):
    """One sector with its own Inv table: the expectation values go through the reduced density
    matrices of the LL+LR and RR+RL halves (a trace per term).  They agree with the oracle's
    product-then-dot within 1e-12, and with the per-state gather form."""
    p = big
    st, inv0 = p.sectors[p.target], p.inv_sector(p.target)
    b = gpu.superblock_states(st, p.dim_LL, p.dim_RR, p.d, inv=inv0)
    nL, nR = len(p.ops["LL"]), len(p.ops["RR"])
    ops_l = [*p.ops["LL"], *p.ops["RR"], p.ops["On"], *p.ops["CF"]]
    rows = [p.dim_LL] * nL + [p.dim_RR] * nR + [p.d] + [p.dim_LL] * len(p.ops["CF"])
    ops = gpu.BlockOperators(ops_l, rows)
    rng = np.random.default_rng(8)
    v = rng.standard_normal(b.n)
    v /= np.linalg.norm(v)
    w1 = oracle.sb_vm(st, inv0, p.dim_RR, p.d, p.ops["LL"][0], 0, v)
    terms = ([(0, k, 0, 0) for k in range(nL)] + [(1, nL + nR, 0, 0), (3, nL + nR, 0, 1)]
             + [(2, nL + k, 0, k % 2) for k in range(nR)] + [(0, nL + nR + 1 + k, 0, 1) for k in range(len(p.ops["CF"]))])
    got = gpu.sb_expect(b, b, ops, terms, v, v, w1)
    monkeypatch.setenv("DG_SB_EXPECT_TRACE", "0")
    gathered = gpu.sb_expect(b, b, ops, terms, v, v, w1)
    monkeypatch.delenv("DG_SB_EXPECT_TRACE")
    assert not np.array_equal(_bits(got), _bits(gathered))      # the two forms really ran
    for k, (pos, op, sign, w) in enumerate(terms):
        y = oracle.sb_vm(st, inv0, p.dim_RR, p.d, ops_l[op], pos, v)
        ww = (v, w1)[w]
        want = np.dot(ww, y)
        tol = 1e-12 * float(np.dot(np.abs(ww), np.abs(y))) + 1e-300
        assert abs(got[k] - want) <= tol, (k, pos, got[k], want)
        assert abs(gathered[k] - want) <= tol, (k, pos)
    assert np.array_equal(_bits(got), _bits(gpu.sb_expect(b, b, ops, terms, v, v, w1)))   # reproducible


def test_density_matrix_form_on_device_built_basis(gpu, oracle, big):
    """The basis built on the device carries its block structure: the same values as above."""
    p = big
    b = gpu.SuperblockBasis(p.dim_LL, p.dim_RR, p.d, p.q_LL, p.q_RR, p.q_site, p.target)
    st, inv0 = p.sectors[p.target], p.inv_sector(p.target)
    ops_l = [p.ops["LL"][2], p.ops["RR"][3], p.ops["On"]]
    ops = gpu.BlockOperators(ops_l, [p.dim_LL, p.dim_RR, p.d])
    v = np.random.default_rng(9).standard_normal(b.n)
    terms = [(0, 0, 0, 0), (2, 1, 0, 0), (1, 2, 0, 0), (3, 2, 0, 0)]
    got = gpu.sb_expect(b, b, ops, terms, v, v)
    for k, (pos, op, _, _) in enumerate(terms):
        y = oracle.sb_vm(st, inv0, p.dim_RR, p.d, ops_l[op], pos, v)
        assert abs(got[k] - np.dot(v, y)) <= 1e-12 * float(np.dot(np.abs(v), np.abs(y))), k


def test_density_matrix_form_skips_unordered_states(gpu, oracle, big):
    """States not in the reference's order (here: reversed) have no block structure; the values
    still come out right (per-state form)."""
    p = big
    st = tuple(a[::-1].copy() for a in p.sectors[p.target])
    inv = -np.ones_like(p.inv)
    inv[p.sup(st)] = np.arange(len(st[0]), dtype=np.int32)
    b = gpu.superblock_states(st, p.dim_LL, p.dim_RR, p.d, inv=inv)
    ops = gpu.BlockOperators([p.ops["LL"][0], p.ops["RR"][0]], [p.dim_LL, p.dim_RR])
    v = np.random.default_rng(10).standard_normal(b.n)
    got = gpu.sb_expect(b, b, ops, [(0, 0, 0, 0), (2, 1, 0, 0)], v, v)
    for k, (op, pos) in enumerate(((p.ops["LL"][0], 0), (p.ops["RR"][0], 2))):
        y = oracle.sb_vm(st, inv, p.dim_RR, p.d, op, pos, v)
        assert abs(got[k] - np.dot(v, y)) <= 1e-12 * float(np.dot(np.abs(v), np.abs(y))), k


def test_expectation_dropin_takes_density_matrix_form(gpu, oracle, monkeypatch):
    """DMRG_EXPECTATION_ONSITE on a reference-ordered basis goes through the density matrices
    (its sums differ in the last bits from the per-state form; both match the reference)."""
    p, g = _problem()
    lib = gpu.load()
    v = g["v"]
    st, inv0 = p.sectors[p.target], p.inv_sector(p.target)
    a, _ = oracle.call_expectation_onsite(lib, st, inv0, p.dim_LL, p.dim_RR, p.d, p.ops["LL"], p.ops["On"], p.ops["RR"], v)
    monkeypatch.setenv("DG_SB_EXPECT_TRACE", "0")
    b, _ = oracle.call_expectation_onsite(lib, st, inv0, p.dim_LL, p.dim_RR, p.d, p.ops["LL"], p.ops["On"], p.ops["RR"], v)
    assert not np.array_equal(_bits(a), _bits(b))
    tol = 1e-12 * float(np.dot(np.abs(v), np.abs(v))) * 10
    assert np.allclose(a, g["onsite"], rtol=0, atol=tol) and np.allclose(b, g["onsite"], rtol=0, atol=tol)


def _libc_free():
    import ctypes as C
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    return libc.free


def test_density_matrix_dropin_vs_reference_golden(gpu, oracle):
    p, g = _problem()
    st, inv0 = p.sectors[p.target], p.inv_sector(p.target)
    lllr = oracle.lllr_list(p.q_LL, p.q_site, st)
    blocks = oracle.call_density_matrix(gpu.load(), st, inv0, p.dim_LL, p.dim_RR, p.d, g["v"], lllr, _libc_free())
    got = np.concatenate([b.ravel() for b in blocks])
    assert np.array_equal(_bits(got), _bits(g["dm_blocks"]))


def test_density_matrix_device_api_vs_oracle(gpu, oracle, big):
    """dg_sb_density_matrix: every block of the pairs holding states, bitwise the oracle's."""
    import ctypes as C
    import torch
    p = big
    st, inv0 = p.sectors[p.target], p.inv_sector(p.target)
    v = np.random.default_rng(12).standard_normal(len(st[0]))
    lllr = oracle.lllr_list(p.q_LL, p.q_site, st)
    want = oracle.density_matrix_blocks(st, inv0, p.d, p.dim_RR, v, lllr)
    # the oracle's blocks restricted to pairs with states, in order
    LLl, LRl, sums = lllr[0], lllr[1], lllr[2]
    keep, b0 = [], 0
    for M, dim in zip(want, lllr[4]):
        live = np.flatnonzero(sums[b0:b0 + dim] > 0)
        if len(live):
            keep.append(M[np.ix_(live, live)])
        b0 += dim
    for b in (gpu.superblock_states(st, p.dim_LL, p.dim_RR, p.d, inv=inv0),
              gpu.SuperblockBasis(p.dim_LL, p.dim_RR, p.d, p.q_LL, p.q_RR, p.q_site, p.target)):
        nb, npair, ne = C.c_int(), C.c_int(), C.c_long()
        gpu.check(gpu.load().dg_sb_density_info(b.h, C.byref(nb), C.byref(npair), C.byref(ne)))
        assert nb.value == len(keep) and ne.value == sum(k.size for k in keep)
        pll, plr, bs = np.empty(npair.value, np.int32), np.empty(npair.value, np.int32), np.empty(nb.value + 1, np.int32)
        gpu.check(gpu.load().dg_sb_density_layout(b.h, pll.ctypes.data_as(C.POINTER(C.c_int)),
                                                  plr.ctypes.data_as(C.POINTER(C.c_int)), bs.ctypes.data_as(C.POINTER(C.c_int))))
        live = sums > 0
        assert np.array_equal(pll, LLl[live]) and np.array_equal(plr, LRl[live])
        rho = np.empty(ne.value)
        gpu.check(gpu.load().dg_sb_density_matrix(b.h, C.c_void_p(v.ctypes.data), C.c_void_p(rho.ctypes.data)))
        assert np.array_equal(_bits(rho), _bits(np.concatenate([k.ravel() for k in keep])))
        vd = torch.from_numpy(v).cuda()
        rd = torch.empty(ne.value, dtype=torch.float64, device="cuda")
        gpu.check(gpu.load().dg_sb_density_matrix(b.h, C.c_void_p(vd.data_ptr()), C.c_void_p(rd.data_ptr())))
        assert np.array_equal(_bits(rd.cpu().numpy()), _bits(rho))


def test_ed_expectation_dropins_vs_reference_golden(gpu, oracle):
    """EXACT_EXPECTATION_ONSITE / _INTERSITE_Q0 (every site in one device pass) against the
    reference: values within 1e-12 of |v|^2, work vectors bit for bit, nothing written for an
    empty site range."""
    from dmrg_c_gb300 import abi
    g = golden("ed_obs_hubbard6.npz")
    basis, vec = g["basis"], g["vec"]
    dens = abi.Crs(np.arange(5), np.arange(4, dtype=np.int32), np.array([0.0, 1.0, 1.0, 2.0]))
    nup = abi.Crs(np.arange(5), np.arange(4, dtype=np.int32), np.array([0.0, 1.0, 0.0, 1.0]))
    lib = gpu.load()
    tol = 1e-12 * float(vec @ vec) * 4
    out, t, _ = oracle.call_exact_expectation(lib, None, dens, 0, 6, basis, vec, 4)
    assert np.allclose(out, g["onsite"], rtol=0, atol=tol)
    assert np.array_equal(_bits(t), _bits(g["onsite_t"]))
    for start, end in ((0, 6), (2, 5), (3, 3)):
        out, t1, t2 = oracle.call_exact_expectation(lib, nup, dens, start, end, basis, vec, 4)
        assert np.allclose(out, g[f"inter_{start}_{end}"], rtol=0, atol=tol)
        assert np.array_equal(_bits(t1), _bits(g[f"inter_{start}_{end}_t1"]))
        ref_t2 = g[f"inter_{start}_{end}_t2"]
        assert np.array_equal(np.isnan(t2), np.isnan(ref_t2))
        assert np.array_equal(_bits(t2[~np.isnan(t2)]), _bits(ref_t2[~np.isnan(ref_t2)]))
