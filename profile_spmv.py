"""Measurement harness (beside bench.py, not part of the package): SpMV rate survey of the library's operator kernels on the named superblock and ED matrices.

    python profile_spmv.py                      # heuristic and autotuned rates
    python profile_spmv.py --sweep              # every SELL shape / variant / window
    python profile_spmv.py --case hubbard_m512 --format sell --launches 3
                                                             # a few launches, for an ncu capture
    python profile_spmv.py --case hubbard_m512 --mixed --launches 3
                                                             # the mixed-precision product
    python profile_spmv.py --case dmrg_hubbard_m512 --mixed --launches 3 --ws 2 --variant 5
                                                             # a given shape and kernel variant
    python profile_spmv.py --sweep --cases xxz_ed22 hubbard_ed12
                                                             # the ED Hamiltonians
    python profile_spmv.py --build ed_hubbard12 # device ED build (basis + CRS)
    python profile_spmv.py --obc klm_m128       # matrix-free OBC vs explicit Lanczos
    python profile_spmv.py --vm                 # EXACT_V_M_Q0 on the Hubbard L=12 basis
    python profile_spmv.py --solvers klm_m128   # CG / MINRES / mixed solve times
    python profile_spmv.py --build sb_m512      # device superblock CRS build

Rates are CUDA-event timed on the library stream (dg_profile_spmv): "cold" rewrites a
256 MiB buffer before every launch so the matrix is not L2-resident, "warm" does not.
Bytes per launch are the algorithmic CRS footprint nnz_full*12 + (n+1)*4 + 2*n*8.
"""
from __future__ import annotations

import argparse
import json
import sys

from dmrg_c_gb300 import ed_models
from dmrg_c_gb300 import lib as L
from dmrg_c_gb300 import workloads

CASES = {
    "xxz_m64": workloads.xxz_superblock_m64,
    "klm_m128": workloads.klm_superblock_m128,
    "hubbard_m512": workloads.hubbard_superblock_m512,
}
# ED Hamiltonians (full storage, built on the device): the largest batched-XXZ and served-Hubbard sizes
ED_CASES = {
    "xxz_ed22": lambda: ed_models.xxz_chain(22, Jz=1.3, hz=0.4),
    "hubbard_ed12": lambda: ed_models.hubbard_chain(12, U=4.0, hz=0.2),
}


# superblocks of the reference's own DMRG runs (tests/golden), built on the device from their term lists
DMRG_CASES = {
    "dmrg_hubbard_m512": "dmrg_hubbard_vf_sweep4.npz",
    "dmrg_klm_m128": "dmrg_klm_vf_sweep4.npz",
    "dmrg_xxz_m64": "dmrg_xxz_vf_sweep4.npz",
}


def _matrix(name, values=None):
    """Device matrix of a named case (synthetic superblock: host lower CRS uploaded; ED and recorded
    DMRG superblocks: built on the device)."""
    values = L.DG_VALUES_F64 if values is None else values
    if name in DMRG_CASES:
        from pathlib import Path
        from dmrg_c_gb300 import sb_models
        sb = sb_models.load_dmrg_superblock(Path(__file__).resolve().parent / "tests" / "golden" / DMRG_CASES[name])
        s = L.SuperblockCRS(sb.model)
        m = s.matrix(values)
        s.close()
        return m
    if name in ED_CASES:
        ed = L.EDSystem(ED_CASES[name]())
        m = ed.matrix(values)
        ed.close()
        return m
    return L.DeviceMatrix(CASES[name](0).explicit_lower(), L.DG_STORE_LOWER_DIAG_LAST, values)
FLUSH = 256 << 20


def algorithmic_bytes(n, nnz_full, s_val=8, s_vec=8):
    return nnz_full * (s_val + 4) + (n + 1) * 4 + 2 * n * s_vec


def _sell_grid(n, ws, sms):
    slices = (n + 31) // 32
    per_block = 8 // ws            # slices one 256-thread block covers per trip
    return max(1, min(sms * 16, (slices + per_block - 1) // per_block))


def _csr_grid(n, lanes, sms):
    return max(1, min(sms * 16, (n * lanes + 255) // 256))


def _rate(m, x, y, iters):
    prof = m.profile_spmv_mixed if x.dtype != y.dtype else m.profile_spmv
    cold = prof(x, y, iters=iters, flush_bytes=FLUSH)
    warm = prof(x, y, iters=iters)
    return cold, warm


def survey(names, sweep, iters, out, mixed=False):
    """Heuristic, swept and autotuned rates; with `mixed` the FP32-value product (FP32 x, FP64 y).
    The sweep sets the FP64 and the FP32 variant together; the autotuner tunes the FP64 product."""
    import torch
    rows = []
    for name in names:
        m = _matrix(name, L.DG_VALUES_BOTH if mixed else L.DG_VALUES_F64)
        n, nnz = m.n, m.nnz
        B = algorithmic_bytes(n, nnz, 4, 4) if mixed else algorithmic_bytes(n, nnz)
        x = torch.randn(n, dtype=torch.float32 if mixed else torch.float64, device="cuda")
        y = torch.empty(n, dtype=torch.float64, device="cuda")
        sms = torch.cuda.get_device_properties(x.device).multi_processor_count
        c, w = _rate(m, x, y, iters)
        print(f"## {name}: n={n} nnz_full={nnz} bytes={B / 1e6:.1f} MB", flush=True)
        print(f"   heuristic: cold {c * 1e3:7.1f} us ({B / c / 1e6:5.0f} GB/s)  warm {w * 1e3:7.1f} us "
              f"({B / w / 1e6:5.0f} GB/s)", flush=True)
        rows.append(dict(case=name, kind="heuristic", n=n, nnz_full=nnz, bytes=B, cold_us=c * 1e3, warm_us=w * 1e3))
        if sweep:
            for window in (2048, 32):
                m.set_sell_window(window)
                for ws in (1, 2, 4, 8):
                    for var in range(7):
                        if (var in (5, 6) and not m.sell_deltas()[0]) or (var in (4, 6) and ws > 1):
                            continue   # no delta stream / the streamed forms run one warp a slice
                        m.set_sell_shape(ws, _sell_grid(n, ws, sms))
                        m.set_sell_variant(var)
                        c, w = _rate(m, x, y, iters)
                        print(f"   sell win={window:4d} ws={ws} var={var}: cold {c * 1e3:7.1f} us "
                              f"({B / c / 1e6:5.0f} GB/s)  warm {w * 1e3:7.1f} us ({B / w / 1e6:5.0f} GB/s)", flush=True)
                        rows.append(dict(case=name, kind="sell", window=window, ws=ws, variant=var, bytes=B,
                                         cold_us=c * 1e3, warm_us=w * 1e3))
            for lanes in (2, 4, 8, 16, 32):
                m.set_shape(lanes, _csr_grid(n, lanes, sms))
                c, w = _rate(m, x, y, iters)
                print(f"   csr lanes={lanes:2d}: cold {c * 1e3:7.1f} us ({B / c / 1e6:5.0f} GB/s)  warm "
                      f"{w * 1e3:7.1f} us ({B / w / 1e6:5.0f} GB/s)", flush=True)
                rows.append(dict(case=name, kind="csr", lanes=lanes, bytes=B, cold_us=c * 1e3, warm_us=w * 1e3))
        r = m.autotune(iters=5)
        c, w = _rate(m, x, y, iters)
        print(f"   autotuned (format={r.format} shape={r.shape} variant={r.variant} window={r.window} grid={r.grid}): "
              f"cold {c * 1e3:7.1f} us ({B / c / 1e6:5.0f} GB/s)  warm {w * 1e3:7.1f} us ({B / w / 1e6:5.0f} GB/s)",
              flush=True)
        rows.append(dict(case=name, kind="autotuned", format=r.format, shape=r.shape, variant=r.variant,
                         window=r.window, grid=r.grid, bytes=B, cold_us=c * 1e3, warm_us=w * 1e3))
        del m
    if out:
        with open(out, "w") as f:
            json.dump(rows, f, indent=1)


def launches(name, fmt, count, mixed=False, ws=None, grid=None, variant=None, window=None):
    """`count` launches of one kernel on one matrix (nothing else on the device after setup);
    ws / grid / variant / window override the sliced-ELL shape the library chose."""
    import torch
    m = _matrix(name, L.DG_VALUES_BOTH if mixed else L.DG_VALUES_F64)
    x = torch.randn(m.n, dtype=torch.float64, device="cuda")
    if fmt == "csr":
        m.set_shape(8, _csr_grid(m.n, 8, torch.cuda.get_device_properties(x.device).multi_processor_count))
    else:
        if window is not None:
            m.set_sell_window(window)
        if ws is not None or grid is not None:
            sms = torch.cuda.get_device_properties(x.device).multi_processor_count
            w = ws if ws is not None else 1
            m.set_sell_shape(w, grid if grid is not None else _sell_grid(m.n, w, sms))
        if variant is not None:
            m.set_sell_variant(variant)
    y = torch.empty_like(x)
    if mixed:
        t = m.profile_spmv_mixed(x.float(), y, iters=count)
        B = algorithmic_bytes(m.n, m.nnz, 4, 4)
    else:
        t = m.profile_spmv(x, y, iters=count)
        B = algorithmic_bytes(m.n, m.nnz)
    print(f"{name} {fmt}{' mixed' if mixed else ''}: {t * 1e3:.1f} us per launch ({B / t / 1e6:.0f} GB/s), "
          f"n={m.n} nnz_full={m.nnz}")


def obc_solve(name, repeats=3):
    """Matrix-free superblock operator against the explicit CRS on the same superblock: the drop-in
    DMRG_LANCZOS_SLOW_OBC (block operators and basis tables uploaded, the product gathers through
    Inv_LLLRRRRL) and LANCZOS_SLOW_SYM on the explicit lower triangle (uploaded and expanded), same
    start vector and accuracy; wall time per call including the uploads."""
    import ctypes as C
    import os
    import tempfile
    import time
    import numpy as np
    from dmrg_c_gb300 import abi
    sb = CASES[name](0)
    lib = L.load()
    guess = np.random.default_rng(3).standard_normal(sb.n)
    low = sb.explicit_lower()
    old = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        try:
            for form in ("obc", "explicit"):
                for k in range(repeats):
                    vec, val = guess.copy(), np.zeros(1)
                    if form == "obc":
                        box = abi.DMRG_BOX_LAN(Eig_Vec=abi.ptr(vec, C.c_double), eig_val=abi.ptr(val, C.c_double), acc=1e-14,
                                               min_step=1, max_step=800, p_threads=1, Guess=b"Yes", Type=b"Normal",
                                               M_LLLR=sb.M_LLLR.ref, M_LRRL=sb.M_LRRL.ref, M_LRRL_Sign=sb.M_LRRL_Sign.ref,
                                               M_RRRL=sb.M_RRRL.ref, Ele_RR=abi.ptr(sb.ele_rr, C.c_int),
                                               Dmrg_Basis=C.pointer(sb.basis))
                        t0 = time.perf_counter()
                        lib.DMRG_LANCZOS_SLOW_OBC(C.byref(box))
                    else:
                        box = abi.BOX_LAN(M=low.ref, Eig_Vec=abi.ptr(vec, C.c_double), eig_val=abi.ptr(val, C.c_double),
                                          acc=1e-14, min_step=1, max_step=800, max_block_step=800, p_threads=1,
                                          Guess=b"Yes", Type=b"Normal")
                        t0 = time.perf_counter()
                        lib.LANCZOS_SLOW_SYM(C.byref(box))
                    t = time.perf_counter() - t0
                    print(f"{name} {form}: {t * 1e3:.2f} ms per Lanczos solve (E = {val[0]:.15f})", flush=True)
        finally:
            os.chdir(old)


def vm(repeats=10):
    """EXACT_V_M_Q0 (a site operator applied to a vector on an ED basis) on the Hubbard L=12 basis
    (n = 853,776), from pinned host arrays: wall time per drop-in call (basis, vector and operator
    uploaded, one binary-searched gather per stored operator element, result downloaded), at the
    first and the last site."""
    import ctypes as C
    import time
    import numpy as np
    import torch
    from dmrg_c_gb300 import abi
    ed = L.EDSystem(ed_models.hubbard_chain(12, U=4.0, hz=0.2))
    basis = ed.download()[0]
    ed.close()
    n = len(basis)
    b_t = torch.from_numpy(basis).pin_memory()
    v_t = torch.randn(n, dtype=torch.float64).pin_memory()
    o_t = torch.zeros(n, dtype=torch.float64).pin_memory()
    info = abi.EXACT_BASIS_INFO(dim=n, Basis=abi.ptr(b_t.numpy(), C.c_long), tot_sz=0, tot_ele=0, tot_parity=0)
    op = abi.Crs(np.array([0, 1, 2, 3, 4]), np.array([0, 1, 2, 3], np.int32), np.array([0.0, 1.0, 1.0, 2.0]), n=4)
    lib = L.load()
    v, o = abi.ptr(v_t.numpy(), C.c_double), abi.ptr(o_t.numpy(), C.c_double)
    for site in (0, 11):
        lib.EXACT_V_M_Q0(op.ref, v, o, 4, site, 1, C.byref(info))   # warm
        t0 = time.perf_counter()
        for _ in range(repeats):
            lib.EXACT_V_M_Q0(op.ref, v, o, 4, site, 1, C.byref(info))
        t = (time.perf_counter() - t0) / repeats
        print(f"EXACT_V_M_Q0 hubbard L=12 (n={n}) site {site}: {t * 1e3:.3f} ms per call "
              f"({3 * n * 8 / t / 1e9:.1f} GB/s of host<->device vectors+basis)", flush=True)


def observables(repeats=5, per_row=16):
    """Site expectation values <psi|O_site|psi> over all 64 sites of the Hubbard L=64, m=512
    superblock (half filling, 2Sz = 0): 31 block operators on each of LL and RR (conserving the
    block labels, per_row elements a row) and one site operator on LR and RL.  Times the device
    API (dg_sb_expect, every site in one launch, vector resident) and the drop-in
    DMRG_EXPECTATION_ONSITE from host arrays (basis, Inv table, operators and vector uploaded,
    Temp_V downloaded)."""
    import ctypes as C
    import time
    import numpy as np
    import scipy.sparse as sp
    import torch
    from dmrg_c_gb300 import abi, sb_models, workloads
    qb = workloads._block_labels(512, 31, 31.0, 1.25, 0.9, 0)
    qs = workloads.hubbard_site_labels()
    b = L.SuperblockBasis(512, 512, 4, qb, qb, qs, 64 * workloads.QN_SCALE)
    LL, LR, RR, RL, inv = b.download()
    n = b.n
    rng = np.random.default_rng(7)
    n_block = 31
    ops_LL = [sb_models._crs(sb_models._random_sym_op(qb, per_row, rng)) for _ in range(n_block)]
    ops_RR = [sb_models._crs(sb_models._random_sym_op(qb, per_row, rng)) for _ in range(n_block)]
    on = sb_models._crs(sp.csr_matrix(np.diag([0.0, 1.0, 1.0, 2.0])))
    nnz_rows = np.mean([o.nnz / 512 for o in ops_LL])
    v = rng.standard_normal(n)
    v /= np.linalg.norm(v)
    ops = L.BlockOperators(ops_LL + ops_RR + [on], [512] * (2 * n_block) + [4])
    terms = ([(0, k, 0, 0) for k in range(n_block)] + [(1, 2 * n_block, 0, 0), (3, 2 * n_block, 0, 0)]
             + [(2, n_block + k, 0, 0) for k in range(n_block - 1, -1, -1)])
    vd = torch.from_numpy(v).cuda()
    L.sb_expect(b, b, ops, terms, vd, vd)   # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(repeats):
        e_dev = L.sb_expect(b, b, ops, terms, vd, vd)
    t_dev = (time.perf_counter() - t0) / repeats
    import os
    os.environ["DG_SB_EXPECT_TRACE"] = "0"
    e_gat = L.sb_expect(b, b, ops, terms, vd, vd)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(repeats):
        e_gat = L.sb_expect(b, b, ops, terms, vd, vd)
    t_gat = (time.perf_counter() - t0) / repeats
    del os.environ["DG_SB_EXPECT_TRACE"]
    print(f"observables hubbard m=512: n = {n}, {len(terms)} sites, ~{nnz_rows:.1f} elements per block-operator row", flush=True)
    print(f"  dg_sb_expect, density-matrix form (Gram blocks + one trace launch): {t_dev * 1e3:.3f} ms per call "
          f"({t_dev * 1e6 / len(terms):.1f} us per site)", flush=True)
    print(f"  dg_sb_expect, per-state gather form (one launch + sum): {t_gat * 1e3:.3f} ms per call "
          f"({t_gat * 1e6 / len(terms):.1f} us per site); max |difference| {np.abs(e_dev - e_gat).max():.2e}", flush=True)
    # drop-in from host arrays
    st = [np.ascontiguousarray(a) for a in (LL, LR, RR, RL)]
    B = abi.DMRG_BASIS(LL_LLLRRRRL=abi.ptr(st[0], C.c_short), LR_LLLRRRRL=abi.ptr(st[1], C.c_short),
                       RR_LLLRRRRL=abi.ptr(st[2], C.c_short), RL_LLLRRRRL=abi.ptr(st[3], C.c_short),
                       Inv_LLLRRRRL=abi.ptr(inv, C.c_int), dim_LLLRRRRL=n, dim_LL=512, dim_RR=512, dim_onsite=4)
    S = abi.DMRG_STATUS(LL_site=n_block - 1, RR_site=n_block - 1, dim_LLLRRRRL=n)
    arr = lambda ops_: (C.POINTER(abi.CRS1) * len(ops_))(*[o.ref for o in ops_])   # noqa: E731
    out = np.zeros(len(terms))
    temp = np.zeros(n)
    lib = L.load()
    args = (arr(ops_LL), on.ref, arr(ops_RR), abi.ptr(out, C.c_double), abi.ptr(v, C.c_double), abi.ptr(temp, C.c_double), 1,
            C.byref(B), C.byref(S))
    lib.DMRG_EXPECTATION_ONSITE(*args)
    t0 = time.perf_counter()
    for _ in range(repeats):
        lib.DMRG_EXPECTATION_ONSITE(*args)
    t_drop = (time.perf_counter() - t0) / repeats
    print(f"  DMRG_EXPECTATION_ONSITE (host arrays, {inv.nbytes / 2**20:.0f} MiB Inv table uploaded): {t_drop * 1e3:.3f} ms per call",
          flush=True)
    print(f"  max |device - drop-in| = {np.abs(e_dev - out).max():.2e}", flush=True)


def truncation(repeats=3):
    """DMRG_GET_SYSTEM_INFO_Q2 (density matrices, their eigen-decompositions, the cut and the
    transformation matrix) on the largest superblocks of the Kondo-lattice m=128 and Hubbard m=512
    runs, keeping m states: wall time per drop-in call from host arrays."""
    import ctypes as C
    import time
    import numpy as np
    import os
    from dmrg_c_gb300 import abi, sb_models, workloads
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    lib = L.load()
    cases = (("klm m=128", workloads._block_labels(128, 11, 5.0, 0.95, 0.85, 0), workloads.klm_site_labels(), 12, 128),
             ("hubbard m=512", workloads._block_labels(512, 31, 31.0, 1.25, 0.9, 0), workloads.hubbard_site_labels(), 64, 512))
    for name, qb, qs, ne, m in cases:
        d, dim = len(qs), len(qb)
        st = sb_models.sector_states(qb, qb, qs, ne * workloads.QN_SCALE)
        n = len(st[0])
        inv = -np.ones(dim * d * dim * d, np.int32)
        inv[((st[0].astype(np.int64) * d + st[1]) * dim + st[2]) * d + st[3]] = np.arange(n, dtype=np.int32)
        # the LLLR list in the reference's order and its blocks
        LL, LR = (x.ravel() for x in np.meshgrid(np.arange(dim), np.arange(d), indexing="ij"))
        lab = np.asarray(qb, np.int64)[LL] + np.asarray(qs, np.int64)[LR]
        o = np.lexsort((LR, LL, lab))
        LL, LR, lab = LL[o].astype(np.int16), LR[o].astype(np.int16), lab[o]
        cnt = np.zeros(dim * d, np.int64)
        np.add.at(cnt, st[0].astype(np.int64) * d + st[1], 1)
        sums = np.ascontiguousarray(cnt[LL.astype(np.int64) * d + LR], np.int32)
        N = np.ascontiguousarray(np.rint(lab / workloads.QN_SCALE), np.int32)
        sz = np.ascontiguousarray(lab - N * workloads.QN_SCALE, np.int32)
        v = np.random.default_rng(5).standard_normal(n)
        v /= np.linalg.norm(v)
        sts = [np.ascontiguousarray(a) for a in st]
        B = abi.DMRG_BASIS(LL_LLLRRRRL=abi.ptr(sts[0], C.c_short), LR_LLLRRRRL=abi.ptr(sts[1], C.c_short),
                           RR_LLLRRRRL=abi.ptr(sts[2], C.c_short), RL_LLLRRRRL=abi.ptr(sts[3], C.c_short),
                           Inv_LLLRRRRL=abi.ptr(inv, C.c_int), dim_LLLRRRRL=n, dim_LL=dim, dim_RR=dim, dim_onsite=d,
                           LL_LLLR=abi.ptr(LL, C.c_short), LR_LLLR=abi.ptr(LR, C.c_short), dim_LLLR=dim * d,
                           Sum_LLLR=abi.ptr(sums, C.c_int))
        T = abi.DMRG_TIME()
        blocks = np.unique(lab, return_counts=True)[1]
        times = []
        os.environ["DG_SB_TRUNC_TIMES"] = "1"
        for it in range(repeats + 1):
            t0 = time.perf_counter()
            S = lib.DMRG_GET_SYSTEM_INFO_Q2(abi.ptr(N, C.c_int), abi.ptr(sz, C.c_int), C.byref(B), abi.ptr(v, C.c_double), m, 1,
                                            C.byref(T)).contents
            times.append(time.perf_counter() - t0)
            kept, tr = S.dim_renorm, S.tr_error
            for mat in (S.Trans_Matrix.contents, S.Trans_Matrix_Dagger.contents):
                for a in (mat.Val, mat.Row, mat.Col):
                    libc.free(C.cast(a, C.c_void_p))
            for a in (S.Trans_Matrix, S.Trans_Matrix_Dagger, S.Val_DM_Dist, S.Q_Number1, S.Q_Number2, S.Q_Number3):
                libc.free(C.cast(a, C.c_void_p))
            libc.free(C.cast(C.pointer(S), C.c_void_p))
        print(f"DMRG_GET_SYSTEM_INFO_Q2 {name}: n = {n}, {len(blocks)} density blocks (largest {blocks.max()}), kept {kept}, "
              f"truncation error {tr:.3e}: {min(times[1:]) * 1e3:.2f} ms per call", flush=True)


def renorm_operands(r3, c3, nblk, per_row, seed=0):
    """T^dagger, O, T of one renormalisation: T (r3 x c3) with each column on one of nblk row blocks,
    O conserving the blocks with per_row elements a row (the shape TRANSFORM_MATRIX sees)."""
    import numpy as np
    import scipy.sparse as sp
    from dmrg_c_gb300 import abi
    rng = np.random.default_rng(seed)
    blocks = np.sort(rng.integers(0, nblk, r3))
    rows_t, cols_t = [], []
    for j in range(c3):
        r = np.flatnonzero(blocks == j % nblk)
        rows_t.append(r)
        cols_t.append(np.full(len(r), j))
    rt, ct = np.concatenate(rows_t), np.concatenate(cols_t)
    T = sp.csc_matrix((rng.standard_normal(len(rt)), (rt, ct)), shape=(r3, c3))
    ro, co = [], []
    for b in range(nblk):
        idx = np.flatnonzero(blocks == b)
        if len(idx) == 0:
            continue
        k = min(per_row, len(idx))
        for i in idx:
            ro.append(np.full(k, i))
            co.append(rng.choice(idx, size=k, replace=False))
    ro, co = np.concatenate(ro), np.concatenate(co)
    O = sp.csr_matrix((rng.standard_normal(len(ro)), (ro, co)), shape=(r3, r3))
    return abi.Crs.from_scipy(T.T.tocsr()), abi.Crs.from_scipy(O), abi.Ccs.from_scipy(T)


def renorm(repeats=5):
    """CRS_CRS_CCS_PRODUCT (T^dagger O T) with the shapes of the KLM m=128 (LLLR 1024 -> 128) and
    Hubbard m=512 (LLLR 2048 -> 512) renormalisations: wall time per drop-in call from host arrays."""
    import ctypes as C
    import time
    import numpy as np
    from dmrg_c_gb300 import abi
    lib = L.load()
    for name, r3, c3, nblk, per_row in (("klm m=128", 1024, 128, 47, 16), ("hubbard m=512", 2048, 512, 57, 24)):
        M1, M2, M3 = renorm_operands(r3, c3, nblk, per_row)
        work = abi.Ccs.empty(c3, r3 * c3)
        out = abi.Crs(np.zeros(c3 + 1, np.int64), np.zeros(c3 * c3, np.int32), np.zeros(c3 * c3), n=c3)
        wv = np.zeros(r3)
        args = (M1.ref, M2.ref, M3.ref, out.ref, work.ref, abi.ptr(wv, C.c_double))
        lib.CRS_CRS_CCS_PRODUCT(*args)
        t0 = time.perf_counter()
        for _ in range(repeats):
            lib.CRS_CRS_CCS_PRODUCT(*args)
        t = (time.perf_counter() - t0) / repeats
        print(f"CRS_CRS_CCS_PRODUCT {name}: T {r3} x {c3} ({M3.col[-1]} stored), O {M2.nnz} stored -> W {int(work.col[c3])}, "
              f"Out {int(out.row[c3])} stored: {t * 1e3:.2f} ms per call", flush=True)


def solvers(name, repeats=5):
    """Whole ground-state solves on one device-resident matrix with the solver forms side by side:
    Lanczos + inverse iteration with CG or with MINRES inner solves (FP64), and the two
    mixed-precision forms; ms per solve (device resident, library timers), steps and energy."""
    import numpy as np
    m = _matrix(name, L.DG_VALUES_BOTH)
    guess = np.random.default_rng(3).standard_normal(m.n)
    forms = (("FP64, II with CG", dict()), ("FP64, II with MINRES", dict(ii_minres=1)),
             ("mixed=1", dict(mixed=1)), ("mixed=2", dict(mixed=2)))
    for label, kw in forms:
        ms, info = [], None
        for k in range(repeats + 1):
            v, info = L.ground_state(m, L.default_params(**kw), guess=guess)
            if k:
                ms.append(info.ms_lanczos + info.ms_ii)
        print(f"{name} {label}: {np.median(ms):.3f} ms per solve (Lanczos {info.lanczos_steps} steps, inner "
              f"{info.cg_steps} steps, E = {info.eig_val:.15f})", flush=True)


BUILDS = ("ed_hubbard12", "ed_xxz22", "sb_m512", "sb_basis_m512")


def build(which, repeats=3):
    """Device builds: ED basis + Hamiltonian, the superblock CRS from host basis arrays, or the
    superblock basis and then the CRS on it (wall time per build)."""
    import time
    from dmrg_c_gb300 import ed_models
    if which.startswith("ed_"):
        model = ed_models.hubbard_chain(12, U=4.0, hz=0.2) if which == "ed_hubbard12" else ed_models.xxz_chain(22, Jz=1.3)
        make = lambda: L.EDSystem(model)  # noqa: E731
    elif which == "sb_basis_m512":
        # the m=512 superblock basis (227,652 states, 16.8 M-entry Inv table), then its CRS on it
        qb = workloads._block_labels(512, 31, 31.0, 1.25, 0.9, 0)
        site = workloads.hubbard_site_labels()
        model = workloads.hubbard_sb_model_m512(0)

        class _Both:
            def __init__(self):
                t0 = time.perf_counter()
                self.b = L.SuperblockBasis(512, 512, 4, qb, qb, site, 64 * workloads.QN_SCALE)
                self.t_basis = time.perf_counter() - t0
                self.s = L.SuperblockCRS(model, basis=self.b)
                self.n, self.nnz = self.s.n, self.s.nnz
                print(f"  basis {self.t_basis * 1e3:.2f} ms", flush=True)

            def close(self):
                self.s.close()
                self.b.close()
        make = _Both
    else:
        model = workloads.hubbard_sb_model_m512(0)
        make = lambda: L.SuperblockCRS(model)  # noqa: E731
    for k in range(repeats):
        t0 = time.perf_counter()
        s = make()
        dt = time.perf_counter() - t0
        print(f"{which}: {dt * 1e3:.1f} ms (n={getattr(s, 'dim', getattr(s, 'n', 0))}, nnz={s.nnz})", flush=True)
        s.close()


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--cases", nargs="*", default=list(CASES), choices=list(CASES) + list(ED_CASES) + list(DMRG_CASES))
    ap.add_argument("--sweep", action="store_true")
    ap.add_argument("--iters", type=int, default=10)
    ap.add_argument("--json", default=None)
    ap.add_argument("--case", choices=list(CASES) + list(ED_CASES) + list(DMRG_CASES), default=None)
    ap.add_argument("--format", choices=["sell", "csr"], default="sell")
    ap.add_argument("--launches", type=int, default=3)
    ap.add_argument("--mixed", action="store_true")
    ap.add_argument("--ws", type=int, default=None, help="warps per slice (with --case)")
    ap.add_argument("--grid", type=int, default=None, help="blocks (with --case)")
    ap.add_argument("--variant", type=int, default=None, help="sliced-ELL kernel variant (with --case)")
    ap.add_argument("--window", type=int, default=None, help="row-sorting window (with --case)")
    ap.add_argument("--build", choices=BUILDS, default=None)
    ap.add_argument("--obc", choices=list(CASES), default=None, help="matrix-free vs explicit Lanczos on a superblock")
    ap.add_argument("--vm", action="store_true", help="EXACT_V_M_Q0 on the Hubbard L=12 basis")
    ap.add_argument("--obs", action="store_true", help="site expectation values on the Hubbard m=512 superblock")
    ap.add_argument("--trunc", action="store_true", help="DMRG_GET_SYSTEM_INFO_Q2 on the KLM m=128 and Hubbard m=512 superblocks")
    ap.add_argument("--renorm", action="store_true", help="CRS_CRS_CCS_PRODUCT with the KLM m=128 and Hubbard m=512 shapes")
    ap.add_argument("--solvers", choices=list(CASES) + list(ED_CASES) + list(DMRG_CASES), default=None,
                    help="solve times of the solver forms on one matrix")
    a = ap.parse_args(argv)
    if a.solvers:
        solvers(a.solvers)
    elif a.vm:
        vm()
    elif a.obs:
        observables()
    elif a.trunc:
        truncation()
    elif a.renorm:
        renorm()
    elif a.obc:
        obc_solve(a.obc)
    elif a.build:
        build(a.build)
    elif a.case:
        launches(a.case, a.format, a.launches, a.mixed, a.ws, a.grid, a.variant, a.window)
    else:
        survey(a.cases, a.sweep, a.iters, a.json, a.mixed)
    return 0


if __name__ == "__main__":
    sys.exit(main())
