"""Loader and typed bindings of libdmrg_gb300.so (the C-ABI in include/dmrg_gb300.h).

The library is built in-tree (``python -m dmrg_c_gb300.build``).  There is no fallback:
importing the bindings raises if the shared library is missing, and every native call
that fails raises :class:`DgError` with the library's own message.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import abi
from .abi import (BOX_CG, BOX_II, BOX_LAN, CRS1, DMRG_BASIS, DMRG_BOX_CG, DMRG_BOX_II, DMRG_BOX_LAN, DMRG_PARAMETER,
                  DMRG_STATUS, DMRG_TIME, EXACT_BASIS_INFO, EXACT_HAM_INFO, EXACT_PARAMETER, EXACT_TIME,
                  EXACT_WHOLE_BASIS_Q1, EXACT_WHOLE_BASIS_Q2, EXACT_WHOLE_BASIS_Q3, dg_ed_model, dg_solve_info,
                  dg_solver_params)

LIB_PATH = Path(__file__).resolve().parent / "libdmrg_gb300.so"

DG_STATUS = {0: "DG_OK", 1: "DG_ERR_ARG", 2: "DG_ERR_CUDA", 3: "DG_ERR_NOMEM", 4: "DG_ERR_NOCONV", 5: "DG_ERR_TIMEOUT",
             6: "DG_ERR_NODEVICE", 7: "DG_ERR_MATRIX"}


class DgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{DG_STATUS.get(code, code)}: {msg}")
        self.code = code


P = C.POINTER
vp = C.c_void_p
dp = P(C.c_double)
ip = P(C.c_int)
lp = P(C.c_long)
fp = P(C.c_float)

# name -> (restype, argtypes); every declaration of include/dmrg_gb300.h
SIGNATURES = {
    # drop-in (reference names)
    "MATRIX_VECTOR_PRODUCT": (None, [P(CRS1), dp, dp, C.c_int]),
    "MATRIX_VECTOR_PRODUCT_SYM": (None, [P(CRS1), dp, dp, P(dp), C.c_int]),
    "LANCZOS": (None, [P(BOX_LAN)]),
    "LANCZOS_SYM": (None, [P(BOX_LAN)]),
    "LANCZOS_SLOW": (None, [P(BOX_LAN)]),
    "LANCZOS_SLOW_SYM": (None, [P(BOX_LAN)]),
    "INVERSE_ITERATION": (None, [P(BOX_II)]),
    "INVERSE_ITERATION_SYM": (None, [P(BOX_II)]),
    "CONJUGATE_GRADIENT": (None, [P(BOX_CG)]),
    "CONJUGATE_GRADIENT_SYM": (None, [P(BOX_CG)]),
    "MINIMUM_RESIDUAL": (None, [P(BOX_CG)]),
    "MINIMUM_RESIDUAL_SYM": (None, [P(BOX_CG)]),
    "CONVERGE_CHECK": (C.c_double, [P(CRS1), dp, C.c_double, C.c_int]),
    "CONVERGE_CHECK_SYM": (C.c_double, [P(CRS1), dp, C.c_double, C.c_int]),
    "DMRG_DIAGONALIZE_SUPERBLOCK": (None, [P(CRS1), P(DMRG_TIME), P(DMRG_PARAMETER), P(DMRG_STATUS), C.c_int]),
    "DMRG_DIAGONALIZE_SUPERBLOCK_SYM": (None, [P(CRS1), P(DMRG_TIME), P(DMRG_PARAMETER), P(DMRG_STATUS), C.c_int]),
    "DMRG_MATRIX_VECTOR_PRODUCT_OBC": (None, [P(CRS1), P(CRS1), P(CRS1), P(CRS1), dp, dp, ip, C.c_int, P(DMRG_BASIS)]),
    "DMRG_LANCZOS_SLOW_OBC": (None, [P(DMRG_BOX_LAN)]),
    "DMRG_V_M_LL_Q0": (None, [P(CRS1), dp, dp, C.c_int, C.c_int, P(DMRG_BASIS)]),
    "DMRG_V_M_LR_Q0": (None, [P(CRS1), dp, dp, C.c_int, C.c_int, P(DMRG_BASIS)]),
    "DMRG_V_M_RR_Q0": (None, [P(CRS1), dp, dp, C.c_int, C.c_int, P(DMRG_BASIS)]),
    "DMRG_V_M_RL_Q0": (None, [P(CRS1), dp, dp, C.c_int, C.c_int, P(DMRG_BASIS)]),
    "DMRG_V_M_LL_Q1": (None, [P(CRS1), C.c_int, dp, dp, C.c_int, P(abi.DMRG_WHOLE_BASIS_Q1)]),
    "DMRG_V_M_LR_Q1": (None, [P(CRS1), C.c_int, dp, ip, C.c_char_p, dp, C.c_int, P(abi.DMRG_WHOLE_BASIS_Q1)]),
    "DMRG_V_M_RR_Q1": (None, [P(CRS1), C.c_int, dp, ip, ip, C.c_char_p, dp, C.c_int, P(abi.DMRG_WHOLE_BASIS_Q1)]),
    "DMRG_V_M_RL_Q1": (None, [P(CRS1), C.c_int, dp, ip, ip, ip, C.c_char_p, dp, C.c_int, P(abi.DMRG_WHOLE_BASIS_Q1)]),
    "DMRG_V_M_LL_Q2": (None, [P(CRS1), C.c_int, C.c_int, dp, dp, C.c_int, P(abi.DMRG_WHOLE_BASIS_Q2)]),
    "DMRG_V_M_LR_Q2": (None, [P(CRS1), C.c_int, C.c_int, dp, ip, C.c_char_p, dp, C.c_int, P(abi.DMRG_WHOLE_BASIS_Q2)]),
    "DMRG_V_M_RR_Q2": (None, [P(CRS1), C.c_int, C.c_int, dp, ip, ip, C.c_char_p, dp, C.c_int, P(abi.DMRG_WHOLE_BASIS_Q2)]),
    "DMRG_V_M_RL_Q2": (None, [P(CRS1), C.c_int, C.c_int, dp, ip, ip, ip, C.c_char_p, dp, C.c_int, P(abi.DMRG_WHOLE_BASIS_Q2)]),
    "DMRG_V_M_LL_Q3": (None, [P(CRS1), C.c_int, C.c_int, C.c_int, dp, dp, C.c_int, P(abi.DMRG_WHOLE_BASIS_Q3)]),
    "DMRG_V_M_LR_Q3": (None, [P(CRS1), C.c_int, C.c_int, C.c_int, dp, ip, C.c_char_p, dp, C.c_int, P(abi.DMRG_WHOLE_BASIS_Q3)]),
    "DMRG_V_M_RR_Q3": (None, [P(CRS1), C.c_int, C.c_int, C.c_int, dp, ip, ip, C.c_char_p, dp, C.c_int, P(abi.DMRG_WHOLE_BASIS_Q3)]),
    "DMRG_V_M_RL_Q3": (None, [P(CRS1), C.c_int, C.c_int, C.c_int, dp, ip, ip, ip, C.c_char_p, dp, C.c_int, P(abi.DMRG_WHOLE_BASIS_Q3)]),
    "DMRG_V_M_RR_Q4": (None, [P(CRS1), C.c_int, C.c_int, C.c_int, C.c_int, dp, ip, ip, C.c_char_p, dp, C.c_int, P(abi.DMRG_WHOLE_BASIS_Q4)]),
    "DMRG_V_M_RL_Q4": (None, [P(CRS1), C.c_int, C.c_int, C.c_int, C.c_int, dp, ip, ip, ip, C.c_char_p, dp, C.c_int, P(abi.DMRG_WHOLE_BASIS_Q4)]),
    "DMRG_EXPECTATION_ONSITE": (None, [P(P(CRS1)), P(CRS1), P(P(CRS1)), dp, dp, dp, C.c_int, P(DMRG_BASIS), P(DMRG_STATUS)]),
    "DMRG_EXPECTATION_INTERSITE_Q0": (None, [P(P(CRS1)), P(P(CRS1)), P(CRS1), P(P(CRS1)), dp, C.c_int, dp, dp, dp, C.c_int,
                                              P(DMRG_BASIS), P(DMRG_STATUS)]),
    "DMRG_CONJUGATE_GRADIENT_OBC": (None, [P(DMRG_BOX_CG)]),
    "DMRG_INVERSE_ITERATION_OBC": (None, [P(DMRG_BOX_II)]),
    "DMRG_CONVERGE_CHECK_OBC": (C.c_double, [C.c_double, P(CRS1), P(CRS1), P(CRS1), P(CRS1), dp, dp, ip, C.c_int,
                                            P(DMRG_BASIS)]),
    "EXACT_DIAGONALIZE_HAMILTONIAN": (None, [P(EXACT_HAM_INFO), P(EXACT_PARAMETER), P(EXACT_TIME), C.c_int]),
    "EXACT_V_M_Q0": (None, [P(CRS1), dp, dp, C.c_int, C.c_int, C.c_int, P(EXACT_BASIS_INFO)]),
    "EXACT_V_M_Q1": (None, [P(CRS1), C.c_int, dp, C.c_int, dp, C.c_int, C.c_int, C.c_int, P(EXACT_WHOLE_BASIS_Q1)]),
    "EXACT_V_M_Q2": (None, [P(CRS1), C.c_int, C.c_int, dp, C.c_int, C.c_int, dp, C.c_char_p, ip, C.c_int, C.c_int,
                            C.c_int, P(EXACT_WHOLE_BASIS_Q2)]),
    "EXACT_V_M_Q3": (None, [P(CRS1), C.c_int, C.c_int, C.c_int, dp, C.c_int, C.c_int, C.c_int, dp, C.c_char_p, ip,
                            C.c_int, C.c_int, C.c_int, P(EXACT_WHOLE_BASIS_Q3)]),
    # native API
    "dg_last_error": (C.c_char_p, []),
    "dg_device_count": (C.c_int, []),
    "dg_version": (C.c_char_p, []),
    "dg_kernel_launches": (C.c_long, []),
    "dg_release_pool": (C.c_int, []),
    "dg_profile_spmv": (C.c_int, [vp, vp, vp, C.c_int, C.c_size_t, P(C.c_float)]),
    "dg_profile_spmv_mixed": (C.c_int, [vp, vp, vp, C.c_int, C.c_size_t, P(C.c_float)]),
    "dg_matrix_create": (C.c_int, [C.c_int, lp, ip, dp, C.c_int, C.c_int, P(vp)]),
    "dg_matrix_create_device": (C.c_int, [C.c_int, C.c_long, vp, vp, vp, C.c_int, C.c_int, P(vp)]),
    "dg_matrix_free": (None, [vp]),
    "dg_matrix_info": (C.c_int, [vp, ip, lp, ip, ip]),
    "dg_matrix_set_shape": (C.c_int, [vp, C.c_int, C.c_int]),
    "dg_matrix_set_format": (C.c_int, [vp, C.c_int]),
    "dg_matrix_set_sell_shape": (C.c_int, [vp, C.c_int, C.c_int]),
    "dg_matrix_set_sell_variant": (C.c_int, [vp, C.c_int]),
    "dg_matrix_sell_error": (C.c_int, [vp, C.POINTER(C.c_int)]),
    "dg_matrix_set_sell_mixed": (C.c_int, [vp, C.c_int, C.c_int]),
    "dg_shape_cache_apply": (C.c_int, [vp, C.c_int, C.c_int, ip]),
    "dg_shape_cache_clear": (C.c_int, []),
    "dg_shape_cache_size": (C.c_int, [ip]),
    "dg_matrix_sell_deltas": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_long), C.POINTER(C.c_long)]),
    "dg_matrix_sell_config": (C.c_int, [vp, ip, ip, ip, ip, ip]),
    "dg_matrix_set_sell_window": (C.c_int, [vp, C.c_int]),
    "dg_matrix_autotune": (C.c_int, [vp, C.c_int, P(abi.dg_tune_result)]),
    "dg_matrix_format": (C.c_int, [vp, ip, lp]),
    "dg_matrix_download": (C.c_int, [vp, lp, ip, dp]),
    "dg_spmv": (C.c_int, [vp, vp, vp, C.c_double]),
    "dg_spmv_f32": (C.c_int, [vp, vp, vp]),
    "dg_spmv_mixed": (C.c_int, [vp, vp, vp]),
    "dg_solver_params_default": (None, [P(dg_solver_params)]),
    "dg_lanczos": (C.c_int, [vp, P(dg_solver_params), vp, vp, P(dg_solve_info)]),
    "dg_inverse_iteration": (C.c_int, [vp, P(dg_solver_params), C.c_double, vp, P(dg_solve_info)]),
    "dg_ground_state": (C.c_int, [vp, P(dg_solver_params), vp, vp, P(dg_solve_info)]),
    "dg_batch_ground_state": (C.c_int, [C.c_int, P(vp), P(dg_solver_params), P(vp), P(dg_solve_info), P(C.c_int)]),
    "dg_linear_solve": (C.c_int, [vp, C.c_double, vp, vp, C.c_double, C.c_int, C.c_int, ip]),
    "dg_residual_l1": (C.c_int, [vp, vp, C.c_double, dp]),
    "dg_cg_noalloc": (C.c_int, [C.c_int, vp, vp, vp, C.c_double, vp, vp, C.c_double, C.c_int, ip]),
    "FIND_DIM": (C.c_int, [P(abi.MODEL_1DKLM_VF), P(EXACT_TIME)]),
    "GET_BASIS": (lp, [P(abi.MODEL_1DKLM_VF), P(EXACT_TIME), C.c_int]),
    "GET_HAM": (P(CRS1), [P(abi.MODEL_1DKLM_VF), P(EXACT_BASIS_INFO), P(EXACT_PARAMETER), P(EXACT_TIME)]),
    "dg_ed_dim": (C.c_int, [P(abi.dg_ed_model), lp]),
    "dg_ed_build": (C.c_int, [P(abi.dg_ed_model), P(vp)]),
    "dg_ed_free": (None, [vp]),
    "dg_ed_info": (C.c_int, [vp, lp, lp]),
    "dg_ed_download": (C.c_int, [vp, lp, lp, ip, dp]),
    "dg_ed_matrix": (C.c_int, [vp, C.c_int, P(vp)]),
    "dg_sb_basis_upload": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, P(C.c_short), P(C.c_short), P(C.c_short),
                                     P(C.c_short), ip, P(vp)]),
    "dg_sb_ops_create": (C.c_int, [C.c_int, P(P(CRS1)), ip, P(vp)]),
    "EXACT_EXPECTATION_ONSITE": (None, [P(CRS1), dp, dp, dp, C.c_int, C.c_int, C.c_int, P(abi.EXACT_BASIS_INFO)]),
    "EXACT_EXPECTATION_INTERSITE_Q0": (None, [P(CRS1), P(CRS1), C.c_int, C.c_int, dp, dp, dp, dp, C.c_int, C.c_int,
                                              P(abi.EXACT_BASIS_INFO)]),
    "dg_sb_density_info": (C.c_int, [vp, ip, ip, lp]),
    "dg_sb_density_layout": (C.c_int, [vp, ip, ip, ip]),
    "dg_sb_density_matrix": (C.c_int, [vp, vp, vp]),
    "DMRG_GET_DENSITY_MATRIX": (P(dp), [C.c_int, ip, P(DMRG_BASIS), dp, C.c_int]),
    "CRS_CRS_CCS_PRODUCT": (None, [P(CRS1), P(CRS1), P(abi.CCS1), P(CRS1), P(abi.CCS1), dp]),
    "DMRG_GET_SYSTEM_INFO_Q1": (P(abi.DMRG_SYSTEM_INFO), [ip, P(DMRG_BASIS), dp, C.c_int, C.c_int, P(DMRG_TIME)]),
    "DMRG_GET_SYSTEM_INFO_Q2": (P(abi.DMRG_SYSTEM_INFO), [ip, ip, P(DMRG_BASIS), dp, C.c_int, C.c_int, P(DMRG_TIME)]),
    "DMRG_GET_SYSTEM_INFO_Q3": (P(abi.DMRG_SYSTEM_INFO), [ip, ip, ip, P(DMRG_BASIS), dp, C.c_int, C.c_int, P(DMRG_TIME)]),
    "dg_sb_ops_free": (None, [vp]),
    "dg_sb_vm": (C.c_int, [vp, vp, vp, C.c_int, C.c_int, C.c_int, ip, ip, ip, vp, C.c_long, vp]),
    "dg_sb_expect": (C.c_int, [vp, vp, vp, C.c_int, P(abi.dg_sb_expect_term), ip, ip, ip, vp, C.c_long, vp, vp, dp]),
    "dg_sb_build": (C.c_int, [P(abi.dg_sb_model), P(vp)]),
    "dg_sb_info": (C.c_int, [vp, ip, lp]),
    "dg_sb_download": (C.c_int, [vp, lp, ip, dp]),
    "dg_sb_matrix": (C.c_int, [vp, C.c_int, P(vp)]),
    "dg_sb_free": (None, [vp]),
    "dg_sb_basis_build": (C.c_int, [P(abi.dg_sb_basis_spec), P(vp)]),
    "dg_sb_basis_info": (C.c_int, [vp, ip]),
    "dg_sb_basis_download": (C.c_int, [vp, P(C.c_short), P(C.c_short), P(C.c_short), P(C.c_short), ip]),
    "dg_sb_basis_free": (None, [vp]),
    "dg_sb_build_with_basis": (C.c_int, [P(abi.dg_sb_model), vp, P(vp)]),
    "dg_engine_create": (C.c_int, [P(abi.dg_engine_config), P(vp)]),
    "dg_engine_submit_ed": (C.c_int, [vp, P(abi.dg_ed_model), P(dg_solver_params), C.c_long, vp]),
    "dg_engine_poll": (C.c_int, [vp, P(abi.dg_job_result), C.c_int, ip, C.c_int]),
    "dg_engine_pending": (C.c_int, [vp, ip, ip, P(C.c_size_t)]),
    "dg_engine_clock_ms": (C.c_double, [vp]),
    "dg_engine_destroy": (None, [vp]),
}

DG_STORE_FULL, DG_STORE_LOWER_DIAG_LAST = 0, 1
DG_VALUES_F64, DG_VALUES_F32, DG_VALUES_BOTH = 1, 2, 3
DG_FORMAT_CSR, DG_FORMAT_SELL = 0, 1

_lib = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Load (once) and type the library.  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else Path(os.environ.get("DG_LIB", LIB_PATH))
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build the CUDA library first (python -m dmrg_c_gb300.build)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != 0:
        raise DgError(rc, load().dg_last_error().decode(errors="replace"))


def kernel_launches() -> int:
    return int(load().dg_kernel_launches())


def device_count() -> int:
    return int(load().dg_device_count())


def as_ptr(a):
    """ctypes void* for a numpy array or a torch tensor (host or device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return C.c_void_p(a.ctypes.data)
    return C.c_void_p(a.data_ptr())          # torch tensor


class DeviceMatrix:
    """A device-resident CRS operator (dg_matrix)."""

    def __init__(self, crs: abi.Crs | None, storage: int = DG_STORE_FULL, values: int = DG_VALUES_F64, handle=None):
        lib = load()
        if handle is not None:
            h = handle
        else:
            h = C.c_void_p()
            check(lib.dg_matrix_create(crs.n, abi.ptr(crs.row, C.c_long), abi.ptr(crs.col, C.c_int),
                                       abi.ptr(crs.val, C.c_double), storage, values, C.byref(h)))
        self.h = h
        n, nnz, lanes, grid = C.c_int(), C.c_long(), C.c_int(), C.c_int()
        check(lib.dg_matrix_info(h, C.byref(n), C.byref(nnz), C.byref(lanes), C.byref(grid)))
        self.n, self.nnz, self.lanes, self.grid = n.value, nnz.value, lanes.value, grid.value

    def close(self):
        if self.h:
            load().dg_matrix_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_shape(self, lanes: int, grid: int):
        """Use the CSR kernel with this many lanes per row and blocks."""
        check(load().dg_matrix_set_shape(self.h, lanes, grid))
        self.lanes, self.grid = lanes, grid

    def set_sell_shape(self, warps_per_slice: int, grid: int):
        check(load().dg_matrix_set_sell_shape(self.h, warps_per_slice, grid))

    def set_sell_variant(self, variant: int):
        check(load().dg_matrix_set_sell_variant(self.h, variant))

    def set_sell_mixed(self, warps_per_slice: int, variant: int):
        """Warps per slice and variant of the FP32 (mixed-precision) product alone."""
        check(load().dg_matrix_set_sell_mixed(self.h, warps_per_slice, variant))

    def sell_deltas(self) -> tuple[bool, int]:
        """(whether the 16-bit column-delta stream exists, its zero bridge elements)."""
        present, bridges = C.c_int(0), C.c_long(0)
        check(load().dg_matrix_sell_deltas(self.h, C.byref(present), C.byref(bridges), None))
        return bool(present.value), bridges.value

    def sell_checkpoints(self) -> int:
        """32-bit column checkpoints of the delta stream (0 without one)."""
        k = C.c_long(0)
        check(load().dg_matrix_sell_deltas(self.h, None, None, C.byref(k)))
        return k.value

    def sell_config(self) -> dict:
        """The sliced-ELL launch configuration in use (FP64 and FP32 products)."""
        v = [C.c_int(0) for _ in range(5)]
        check(load().dg_matrix_sell_config(self.h, *(C.byref(a) for a in v)))
        return dict(ws=v[0].value, grid=v[1].value, variant=v[2].value, ws32=v[3].value, variant32=v[4].value)

    def shape_cache_apply(self, tune: bool = True, iters: int = 3) -> int:
        """Take the tuned sliced-ELL shape of this matrix's size class (1), tune and record it
        (2), or keep the current shape (0)."""
        how = C.c_int(0)
        check(load().dg_shape_cache_apply(self.h, int(tune), iters, C.byref(how)))
        return how.value

    def sell_error(self) -> int:
        e = C.c_int(0)
        check(load().dg_matrix_sell_error(self.h, C.byref(e)))
        return e.value

    def set_sell_window(self, window: int):
        check(load().dg_matrix_set_sell_window(self.h, window))

    def autotune(self, iters: int = 3) -> abi.dg_tune_result:
        r = abi.dg_tune_result()
        check(load().dg_matrix_autotune(self.h, iters, C.byref(r)))
        return r

    def set_format(self, fmt: int):
        check(load().dg_matrix_set_format(self.h, fmt))

    def format(self):
        f, stored = C.c_int(), C.c_long()
        check(load().dg_matrix_format(self.h, C.byref(f), C.byref(stored)))
        return f.value, stored.value

    def download(self):
        row = np.empty(self.n + 1, np.int64)
        col = np.empty(self.nnz, np.int32)
        val = np.empty(self.nnz, np.float64)
        check(load().dg_matrix_download(self.h, abi.ptr(row, C.c_long), abi.ptr(col, C.c_int), abi.ptr(val, C.c_double)))
        return row, col, val

    def spmv(self, x, y=None, sigma: float = 0.0):
        if y is None:
            y = np.empty(self.n, np.float64)
        check(load().dg_spmv(self.h, as_ptr(x), as_ptr(y), sigma))
        return y

    def profile_spmv(self, x_dev, y_dev, iters=20, flush_bytes=0) -> float:
        """Average ms per launch of the fused product kernel (CUDA events on the library stream)."""
        ms = C.c_float()
        check(load().dg_profile_spmv(self.h, as_ptr(x_dev), as_ptr(y_dev), iters, flush_bytes, C.byref(ms)))
        return ms.value

    def spmv_mixed(self, x, y=None):
        """FP32 values and FP32 x, compensated accumulation, FP64 result."""
        if y is None:
            y = np.empty(self.n, np.float64)
        check(load().dg_spmv_mixed(self.h, as_ptr(x), as_ptr(y)))
        return y

    def profile_spmv_mixed(self, x32_dev, y_dev, iters=20, flush_bytes=0) -> float:
        """Average ms per launch of the mixed-precision product kernel."""
        ms = C.c_float()
        check(load().dg_profile_spmv_mixed(self.h, as_ptr(x32_dev), as_ptr(y_dev), iters, flush_bytes, C.byref(ms)))
        return ms.value

    def spmv_f32(self, x, y=None):
        if y is None:
            y = np.empty(self.n, np.float32)
        check(load().dg_spmv_f32(self.h, as_ptr(x), as_ptr(y)))
        return y


class EDSystem:
    """Basis and Hamiltonian of one ED model, enumerated and assembled on the device (dg_ed)."""

    def __init__(self, model):
        self.model = model            # keeps the dg_ed_model storage alive
        h = C.c_void_p()
        check(load().dg_ed_build(C.byref(model.struct), C.byref(h)))
        self.h = h
        dim, nnz = C.c_long(), C.c_long()
        check(load().dg_ed_info(h, C.byref(dim), C.byref(nnz)))
        self.dim, self.nnz = dim.value, nnz.value

    def close(self):
        if self.h:
            load().dg_ed_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def download(self):
        """(basis, row, col, val) as numpy arrays."""
        basis = np.empty(self.dim, np.int64)
        row = np.empty(self.dim + 1, np.int64)
        col = np.empty(self.nnz, np.int32)
        val = np.empty(self.nnz, np.float64)
        check(load().dg_ed_download(self.h, abi.ptr(basis, C.c_long), abi.ptr(row, C.c_long), abi.ptr(col, C.c_int),
                                    abi.ptr(val, C.c_double)))
        return basis, row, col, val

    def matrix(self, values: int = DG_VALUES_F64) -> DeviceMatrix:
        h = C.c_void_p()
        check(load().dg_ed_matrix(self.h, values, C.byref(h)))
        return DeviceMatrix(None, handle=h)


class SuperblockBasis:
    """Superblock basis built on the device (dg_sb_basis): the states (LL, LR, RR, RL) whose
    quantum numbers sum to the targets in the reference's order, and Inv_LLLRRRRL.

    qn1 / qn2: per-state quantum numbers of the left block, the right block and a site (qn2 may
    be None for one conserved quantity; with two, qn1 is the primary key)."""

    def __init__(self, dim_LL, dim_RR, d, qn1_LL, qn1_RR, qn1_site, target1, qn2_LL=None, qn2_RR=None, qn2_site=None,
                 target2=0):
        two = qn2_LL is not None
        arr = lambda a: np.ascontiguousarray(a, np.int32)   # noqa: E731
        self._keep = [arr(a) for a in (qn1_LL, qn1_RR, qn1_site)] + ([arr(a) for a in (qn2_LL, qn2_RR, qn2_site)] if two else [])
        k = self._keep
        ptrs = [abi.ptr(a, C.c_int) for a in k] + ([None] * 3 if not two else [])
        spec = abi.dg_sb_basis_spec(dim_LL=dim_LL, dim_RR=dim_RR, dim_onsite=d, n_qn=2 if two else 1,
                                    qn1_LL=ptrs[0], qn1_RR=ptrs[1], qn1_site=ptrs[2], qn2_LL=ptrs[3], qn2_RR=ptrs[4],
                                    qn2_site=ptrs[5], target1=target1, target2=target2)
        h = C.c_void_p()
        check(load().dg_sb_basis_build(C.byref(spec), C.byref(h)))
        self.h = h
        n = C.c_int()
        check(load().dg_sb_basis_info(h, C.byref(n)))
        self.n, self.dim_LL, self.dim_RR, self.d = n.value, dim_LL, dim_RR, d

    def close(self):
        if self.h:
            load().dg_sb_basis_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def download(self):
        """(LL, LR, RR, RL, inv) as numpy arrays."""
        st = [np.empty(self.n, np.int16) for _ in range(4)]
        inv = np.empty(self.dim_LL * self.d * self.dim_RR * self.d, np.int32)
        check(load().dg_sb_basis_download(self.h, *(abi.ptr(a, C.c_short) for a in st), abi.ptr(inv, C.c_int)))
        return (*st, inv)


def superblock_states(states, dim_LL, dim_RR, d, inv=None) -> "SuperblockBasis":
    """A SuperblockBasis from host arrays (dg_sb_basis_upload): one sector's (LL, LR, RR, RL) and,
    optionally, an Inv_LLLRRRRL table (a whole basis's table may index other sectors)."""
    st = [np.ascontiguousarray(a, np.int16) for a in states]
    inv_a = np.ascontiguousarray(inv, np.int32) if inv is not None else None
    h = C.c_void_p()
    check(load().dg_sb_basis_upload(len(st[0]), dim_LL, dim_RR, d, *(abi.ptr(a, C.c_short) for a in st),
                                    abi.ptr(inv_a, C.c_int) if inv_a is not None else None, C.byref(h)))
    b = SuperblockBasis.__new__(SuperblockBasis)
    b.h, b.n, b.dim_LL, b.dim_RR, b.d = h, len(st[0]), dim_LL, dim_RR, d
    return b


class BlockOperators:
    """Device copies of square block operators (dg_sb_ops): ops[k] (abi.Crs) acts on a position
    with rows[k] states."""

    def __init__(self, ops, rows):
        self._ops = list(ops)
        arr = (P(CRS1) * len(self._ops))(*[o.ref for o in self._ops])
        r = np.ascontiguousarray(rows, np.int32)
        h = C.c_void_p()
        check(load().dg_sb_ops_create(len(self._ops), arr, abi.ptr(r, C.c_int), C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            load().dg_sb_ops_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _eles(ele):
    if ele is None:
        return [None, None, None], []
    keep = [np.ascontiguousarray(a, np.int32) if a is not None else None for a in ele]
    return [abi.ptr(a, C.c_int) if a is not None else None for a in keep], keep


def _vec_ptr(x):
    """(pointer, length, keep-alive) for a numpy array or a CUDA torch tensor."""
    if hasattr(x, "data_ptr"):
        return C.c_void_p(x.data_ptr()), int(x.numel()), x
    a = np.ascontiguousarray(x, np.float64)
    return C.c_void_p(a.ctypes.data), len(a), a


def sb_vm(out_states: "SuperblockBasis", inv_table: "SuperblockBasis", ops: BlockOperators, op: int, pos: int, v, out=None,
          sign=False, ele=None):
    """O_op v over out_states' states (dg_sb_vm): DMRG_V_M_<pos> on device-resident data.
    v / out may be numpy arrays or CUDA tensors; returns out."""
    if out is None:
        out = np.empty(out_states.n)
    pv, nv, kv = _vec_ptr(v)
    po_, _, ko = _vec_ptr(out)
    ep, ke = _eles(ele)
    check(load().dg_sb_vm(out_states.h, inv_table.h, ops.h, op, pos, int(sign), *ep, pv, nv, po_))
    return out


def sb_expect(out_states: "SuperblockBasis", inv_table: "SuperblockBasis", ops: BlockOperators, terms, v, w0, w1=None,
              ele=None):
    """[sum_i w_t[i] (O_t v)[i] for each term] (dg_sb_expect); terms = (pos, op, sign, weight)."""
    tt = (abi.dg_sb_expect_term * max(len(terms), 1))(*[abi.dg_sb_expect_term(*t) for t in terms])
    out = np.empty(len(terms))
    pv, nv, kv = _vec_ptr(v)
    p0, _, k0 = _vec_ptr(w0)
    p1, k1 = (None, None) if w1 is None else _vec_ptr(w1)[::2]
    ep, ke = _eles(ele)
    check(load().dg_sb_expect(out_states.h, inv_table.h, ops.h, len(terms), tt, *ep, pv, nv, p0, p1,
                              out.ctypes.data_as(dp)))
    return out


class SuperblockCRS:
    """Superblock Hamiltonian (lower triangle, diagonal last) built on the device from a
    dmrg_c_gb300.sb_models.SBModel term list (dg_sb); with a SuperblockBasis the states and the
    Inv table come from the device basis instead of the model's host arrays."""

    def __init__(self, model, basis: "SuperblockBasis | None" = None):
        self.model = model
        h = C.c_void_p()
        if basis is None:
            check(load().dg_sb_build(C.byref(model.struct), C.byref(h)))
        else:
            check(load().dg_sb_build_with_basis(C.byref(model.struct), basis.h, C.byref(h)))
        self.h = h
        n, nnz = C.c_int(), C.c_long()
        check(load().dg_sb_info(h, C.byref(n), C.byref(nnz)))
        self.n, self.nnz = n.value, nnz.value

    def close(self):
        if self.h:
            load().dg_sb_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def download(self):
        row = np.empty(self.n + 1, np.int64)
        col = np.empty(self.nnz, np.int32)
        val = np.empty(self.nnz, np.float64)
        check(load().dg_sb_download(self.h, abi.ptr(row, C.c_long), abi.ptr(col, C.c_int), abi.ptr(val, C.c_double)))
        return row, col, val

    def matrix(self, values: int = DG_VALUES_F64) -> DeviceMatrix:
        h = C.c_void_p()
        check(load().dg_sb_matrix(self.h, values, C.byref(h)))
        return DeviceMatrix(None, handle=h)


def shape_cache_clear():
    """Forget every tuned size class (dg_shape_cache_clear)."""
    check(load().dg_shape_cache_clear())


def shape_cache_size() -> int:
    k = C.c_int(0)
    check(load().dg_shape_cache_size(C.byref(k)))
    return k.value


class Engine:
    """Concurrent ED ground-state engine (dg_engine): submit models, poll results."""

    def __init__(self, workers: int = 0, hbm_budget: int = 0, lanczos_batch: bool = False, tune_shapes: bool = False):
        cfg = abi.dg_engine_config(workers=workers, hbm_budget=hbm_budget, lanczos_batch=int(lanczos_batch),
                                   tune_shapes=int(tune_shapes))
        h = C.c_void_p()
        check(load().dg_engine_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self._keep = {}

    def submit(self, model, params: dg_solver_params, job_id: int, want_vector: bool = False):
        vec = None
        if want_vector:
            vec = np.empty(ed_dim(model), np.float64)
        self._keep[job_id] = vec
        check(load().dg_engine_submit_ed(self.h, C.byref(model.struct), C.byref(params), job_id,
                                         as_ptr(vec) if vec is not None else None))

    def poll(self, max_results: int = 256, wait_ms: int = 0):
        """Finished results as a list of (dg_job_result, eigenvector or None)."""
        buf = (abi.dg_job_result * max_results)()
        n = C.c_int()
        check(load().dg_engine_poll(self.h, buf, max_results, C.byref(n), wait_ms))
        return [(buf[i], self._keep.pop(buf[i].id, None)) for i in range(n.value)]

    def pending(self):
        q, r, b = C.c_int(), C.c_int(), C.c_size_t()
        check(load().dg_engine_pending(self.h, C.byref(q), C.byref(r), C.byref(b)))
        return q.value, r.value, b.value

    def clock_ms(self) -> float:
        return float(load().dg_engine_clock_ms(self.h))

    def close(self):
        if self.h:
            load().dg_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ed_dim(model) -> int:
    dim = C.c_long()
    check(load().dg_ed_dim(C.byref(model.struct), C.byref(dim)))
    return dim.value


def default_params(**kw) -> dg_solver_params:
    p = dg_solver_params()
    load().dg_solver_params_default(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def ground_state(m: DeviceMatrix, params: dg_solver_params | None = None, guess=None, out=None, lanczos_only=False):
    """Lanczos (+ inverse iteration) on the device; returns (eigvec, dg_solve_info)."""
    p = params or default_params()
    if out is None:
        out = np.empty(m.n, np.float64)
    info = dg_solve_info()
    fn = load().dg_lanczos if lanczos_only else load().dg_ground_state
    check(fn(m.h, C.byref(p), as_ptr(guess), as_ptr(out), C.byref(info)))
    return out, info


def batch_ground_state(mats, params: dg_solver_params | None = None, want_vectors=True):
    """Ground states of several DeviceMatrix solved together (dg_batch_ground_state); returns
    ([eigvec or None], [dg_solve_info]).  Raises DgError if any instance failed."""
    p = params or default_params()
    k = len(mats)
    handles = (vp * max(k, 1))(*[m.h for m in mats])
    outs = [np.empty(m.n, np.float64) for m in mats] if want_vectors else []
    vecs = (vp * max(k, 1))(*[as_ptr(o) for o in outs]) if want_vectors else None
    infos = (dg_solve_info * max(k, 1))()
    st = (C.c_int * max(k, 1))()
    check(load().dg_batch_ground_state(k, handles, C.byref(p), vecs, infos, st))
    for i in range(k):
        check(st[i])
    return (outs if want_vectors else [None] * k), [infos[i] for i in range(k)]


def linear_solve(m: DeviceMatrix, b, x, sigma=0.0, acc=1e-7, max_step=1000, minres=False):
    it = C.c_int()
    rc = load().dg_linear_solve(m.h, sigma, as_ptr(b), as_ptr(x), acc, max_step, int(minres), C.byref(it))
    return rc, it.value


def residual_l1(m: DeviceMatrix, x, lam: float) -> float:
    out = C.c_double()
    check(load().dg_residual_l1(m.h, as_ptr(x), lam, C.byref(out)))
    return out.value
