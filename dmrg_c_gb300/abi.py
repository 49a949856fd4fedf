"""ctypes mirrors of the C-ABI structures (include/dmrg_gb300_types.h, dmrg_gb300_ed.h,
dmrg_gb300.h) and helpers that wrap numpy arrays into them.

The layouts are those of the reference's include/SML.h, include/dmrg.h and include/exact.h,
so a structure built here can be handed to libdmrg_gb300 or to any library compiled against
the reference headers.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

c_double_p = C.POINTER(C.c_double)
c_int_p = C.POINTER(C.c_int)
c_long_p = C.POINTER(C.c_long)
c_short_p = C.POINTER(C.c_short)


class CRS1(C.Structure):
    """include/SML.h:17-28"""
    _fields_ = [("max_val", C.c_long), ("max_row", C.c_int), ("row_dim", C.c_int), ("col_dim", C.c_int),
                ("Col", c_int_p), ("Row", c_long_p), ("Val", c_double_p)]


class BOX_CG(C.Structure):
    """include/SML.h:56-65"""
    _fields_ = [("M", C.POINTER(CRS1)), ("acc", C.c_double), ("Vec", c_double_p), ("Out_Vec", c_double_p),
                ("max_step", C.c_int), ("p_threads", C.c_int)]


class BOX_II(C.Structure):
    """include/SML.h:67-86"""
    _fields_ = [("M", C.POINTER(CRS1)), ("ii_acc", C.c_double), ("ii_diag_add", C.c_double), ("ii_max_step", C.c_int),
                ("cg_acc", C.c_double), ("cg_max_step", C.c_int), ("error", C.c_double), ("Eig_Vec", c_double_p),
                ("Eig_Val", c_double_p), ("p_threads", C.c_int), ("Type", C.c_char * 100)]


class BOX_LAN(C.Structure):
    """include/SML.h:122-135"""
    _fields_ = [("M", C.POINTER(CRS1)), ("Eig_Vec", c_double_p), ("eig_val", c_double_p), ("acc", C.c_double),
                ("min_step", C.c_int), ("max_step", C.c_int), ("max_block_step", C.c_int), ("p_threads", C.c_int),
                ("Guess", C.c_char * 100), ("Type", C.c_char * 100)]


class DMRG_PARAMETER(C.Structure):
    """include/dmrg.h:6-38"""
    _fields_ = [("Initial_Guess", C.c_char * 1000), ("Enviro_Copy", C.c_char * 1000), ("II_Type", C.c_char * 1000),
                ("Lan_Con", C.c_char * 1000), ("max_dim_system", C.c_int), ("sweep", C.c_int),
                ("Diag_Method", C.c_char * 1000), ("diag_acc", C.c_double), ("diag_min_step", C.c_int),
                ("diag_max_step", C.c_int), ("cg_acc", C.c_double), ("cg_max_step", C.c_int),
                ("inv_iter_acc", C.c_double), ("inv_iter_diag_add", C.c_double), ("inv_iter_max_step", C.c_int),
                ("sp_LL", C.c_double), ("param_iter", C.c_int), ("param_iter_now", C.c_int),
                ("dim_LLLRRRRL_limit", C.c_int)]


class DMRG_TIME(C.Structure):
    """include/dmrg.h:40-51"""
    _fields_ = [(n, C.c_double) for n in ("diag", "inv_iter", "make_ham", "make_basis", "make_dens_mat", "trans_main",
                                          "trans_exp", "total")]


class DMRG_BASIS(C.Structure):
    """include/dmrg.h:54-99"""
    _fields_ = [("LL_LLLRRRRL", c_short_p), ("LR_LLLRRRRL", c_short_p), ("RL_LLLRRRRL", c_short_p),
                ("RR_LLLRRRRL", c_short_p), ("Inv_LLLRRRRL", c_int_p), ("dim_LLLRRRRL", C.c_int), ("dim_LL", C.c_int),
                ("dim_RR", C.c_int), ("dim_onsite", C.c_int), ("tot_sz_LLLRRRRL", C.c_int),
                ("tot_ele_LLLRRRRL", C.c_int), ("tot_ele_1_LLLRRRRL", C.c_int), ("tot_ele_2_LLLRRRRL", C.c_int),
                ("tot_parity_LLLRRRRL", C.c_int), ("LL_LLLR", c_short_p), ("LR_LLLR", c_short_p),
                ("Inv_LLLR", C.POINTER(c_int_p)), ("dim_LLLR", C.c_int), ("LR_LRRL", c_short_p), ("RL_LRRL", c_short_p),
                ("Inv_LRRL", C.POINTER(c_int_p)), ("dim_LRRL", C.c_int), ("RR_RRRL", c_short_p), ("RL_RRRL", c_short_p),
                ("Inv_RRRL", C.POINTER(c_int_p)), ("dim_RRRL", C.c_int), ("Sum_LLLR", c_int_p), ("Tot_Sz_LLLR", c_int_p),
                ("Tot_Ele_LLLR", c_int_p), ("Tot_Ele_1_LLLR", c_int_p), ("Tot_Ele_2_LLLR", c_int_p),
                ("Tot_Parity_LLLR", c_int_p)]


def _whole_basis_type(depth: int, lines: str):
    sp = c_short_p
    ip = c_int_p
    for _ in range(depth):
        sp = C.POINTER(sp)
    for _ in range(depth - 1):
        ip = C.POINTER(ip)
    return type(f"DMRG_WHOLE_BASIS_Q{depth}", (C.Structure,), {
        "__doc__": lines,
        "_fields_": [("LL_LLLRRRRL", sp), ("LR_LLLRRRRL", sp), ("RL_LLLRRRRL", sp), ("RR_LLLRRRRL", sp),
                     ("Inv_LLLRRRRL", c_int_p), ("Dim", ip), ("max_dim", C.c_int), ("dim_RR", C.c_int),
                     ("dim_onsite", C.c_int)]})


DMRG_WHOLE_BASIS_Q1 = _whole_basis_type(1, "include/dmrg.h:140-152")
DMRG_WHOLE_BASIS_Q2 = _whole_basis_type(2, "include/dmrg.h:155-167")
DMRG_WHOLE_BASIS_Q3 = _whole_basis_type(3, "include/dmrg.h:169-181")
DMRG_WHOLE_BASIS_Q4 = _whole_basis_type(4, "include/dmrg.h:183-195")
WHOLE_BASIS = {1: DMRG_WHOLE_BASIS_Q1, 2: DMRG_WHOLE_BASIS_Q2, 3: DMRG_WHOLE_BASIS_Q3, 4: DMRG_WHOLE_BASIS_Q4}


class WholeBasis:
    """A DMRG_WHOLE_BASIS_Qk over numpy arrays.  ``sectors`` maps a k-tuple of non-negative
    quantum-number indices to the sector's (LL, LR, RR, RL) state arrays; ``shape`` gives the
    extent of each index (absent sectors have dimension 0); ``inv`` is the shared Inv_LLLRRRRL
    table.  ``.struct`` / ``.ref`` view it; the arrays are kept alive by this object."""

    def __init__(self, sectors: dict, shape: tuple, inv, dim_RR: int, dim_onsite: int):
        k = len(shape)
        self.keep = []
        self.inv = np.ascontiguousarray(inv, np.int32)
        dummy = np.zeros(1, np.int16)
        self.keep.append(dummy)

        def build(prefix, leaf, leaf_type):
            # value of type leaf_type at depth k, POINTER(type at depth + 1) above it
            depth = len(prefix)
            if depth == k:
                return leaf(prefix)
            elem_t = leaf_type
            for _ in range(k - depth - 1):
                elem_t = C.POINTER(elem_t)
            arr = (elem_t * shape[depth])(*[build(prefix + (i,), leaf, leaf_type) for i in range(shape[depth])])
            self.keep.append(arr)
            return C.cast(arr, C.POINTER(elem_t))

        def states(idx):
            def leaf(prefix):
                st = sectors.get(prefix)
                a = np.ascontiguousarray(st[idx], np.int16) if st is not None and len(st[0]) else dummy
                self.keep.append(a)
                return a.ctypes.data_as(c_short_p)
            return build((), leaf, c_short_p)

        dim = build((), lambda prefix: len(sectors[prefix][0]) if prefix in sectors else 0, C.c_int)
        dims = [len(v[0]) for v in sectors.values()]
        T = WHOLE_BASIS[k]
        self.struct = T(LL_LLLRRRRL=states(0), LR_LLLRRRRL=states(1), RR_LLLRRRRL=states(2), RL_LLLRRRRL=states(3),
                        Inv_LLLRRRRL=self.inv.ctypes.data_as(c_int_p), Dim=dim, max_dim=max(dims) if dims else 0,
                        dim_RR=dim_RR, dim_onsite=dim_onsite)
        self.ref = C.pointer(self.struct)


class CCS1(C.Structure):
    """include/SML.h:43-54"""
    _fields_ = [("max_val", C.c_long), ("max_col", C.c_int), ("row_dim", C.c_int), ("col_dim", C.c_int),
                ("Col", c_long_p), ("Row", c_int_p), ("Val", c_double_p)]


class DMRG_SYSTEM_INFO(C.Structure):
    """include/dmrg.h:220-234"""
    _fields_ = [("Trans_Matrix", C.POINTER(CCS1)), ("Trans_Matrix_Dagger", C.POINTER(CRS1)), ("tr_error", C.c_double),
                ("Val_DM_Dist", c_double_p), ("sum_val_dm", C.c_double), ("dim_LLLR", C.c_int), ("dim_renorm", C.c_int),
                ("Q_Number1", c_int_p), ("Q_Number2", c_int_p), ("Q_Number3", c_int_p)]


class DMRG_STATUS(C.Structure):
    """include/dmrg.h:236-267"""
    _fields_ = [("BC", C.c_char * 1000), ("Enviro_Copy", C.c_char * 100), ("LL_site", C.c_int), ("RR_site", C.c_int),
                ("max_dim_system", C.c_int), ("dim_LLLRRRRL", C.c_int), ("dim_LL", C.c_int), ("dim_onsite", C.c_int),
                ("dim_RR", C.c_int), ("spin", C.c_int), ("tot_sz", C.c_int), ("tot_ele", C.c_int), ("tot_ele_1", C.c_int),
                ("tot_ele_2", C.c_int), ("tot_parity", C.c_int), ("GS_Vec", c_double_p), ("gs_val", C.c_double),
                ("gs_error", C.c_double), ("percent_LL", C.c_double), ("sweep_now", C.c_int),
                ("param_iter_now", C.c_int), ("tot_iter_now", C.c_int), ("sweep", C.c_int), ("param_iter", C.c_int),
                ("tot_iter", C.c_int)]


class DMRG_BOX_LAN(C.Structure):
    """include/dmrg.h:269-286"""
    _fields_ = [("Eig_Vec", c_double_p), ("eig_val", c_double_p), ("acc", C.c_double), ("min_step", C.c_int),
                ("max_step", C.c_int), ("p_threads", C.c_int), ("Guess", C.c_char * 100), ("Type", C.c_char * 100),
                ("M_LLLR", C.POINTER(CRS1)), ("M_LRRL", C.POINTER(CRS1)), ("M_LRRL_Sign", C.POINTER(CRS1)),
                ("M_RRRL", C.POINTER(CRS1)), ("Ele_RR", c_int_p), ("Dmrg_Basis", C.POINTER(DMRG_BASIS))]


class DMRG_BOX_CG(C.Structure):
    """include/dmrg.h:288-303"""
    _fields_ = [("acc", C.c_double), ("diag_val", C.c_double), ("Vec", c_double_p), ("Out_Vec", c_double_p),
                ("max_step", C.c_int), ("p_threads", C.c_int), ("M_LLLR", C.POINTER(CRS1)),
                ("M_LRRL", C.POINTER(CRS1)), ("M_LRRL_Sign", C.POINTER(CRS1)), ("M_RRRL", C.POINTER(CRS1)),
                ("Ele_RR", c_int_p), ("Dmrg_Basis", C.POINTER(DMRG_BASIS))]


class DMRG_BOX_II(C.Structure):
    """include/dmrg.h:305-328"""
    _fields_ = [("ii_acc", C.c_double), ("ii_diag_add", C.c_double), ("ii_max_step", C.c_int), ("cg_acc", C.c_double),
                ("cg_max_step", C.c_int), ("Eig_Vec", c_double_p), ("eig_val", c_double_p), ("error", C.c_double),
                ("p_threads", C.c_int), ("M_LLLR", C.POINTER(CRS1)), ("M_LRRL", C.POINTER(CRS1)),
                ("M_LRRL_Sign", C.POINTER(CRS1)), ("M_RRRL", C.POINTER(CRS1)), ("Ele_RR", c_int_p),
                ("Dmrg_Basis", C.POINTER(DMRG_BASIS))]


class EXACT_PARAMETER(C.Structure):
    """include/exact.h:14-37"""
    _fields_ = [("diag_num", C.c_int), ("est_max_row_elem_num", C.c_int), ("Diag_Method", C.c_char * 1000),
                ("diag_acc", C.c_double), ("diag_min_step", C.c_int), ("diag_max_step", C.c_int), ("cg_acc", C.c_double),
                ("cg_max_step", C.c_int), ("inv_iter_acc", C.c_double), ("inv_iter_diag_add", C.c_double),
                ("inv_iter_max_step", C.c_int), ("param_iter", C.c_int), ("param_iter_now", C.c_int)]


class EXACT_TIME(C.Structure):
    """include/exact.h:39-51"""
    _fields_ = [(n, C.c_double) for n in ("diag", "inv_iter", "make_ham", "find_dim", "make_basis", "exp_values", "cf",
                                          "sc", "total")]


class EXACT_HAM_INFO(C.Structure):
    """include/exact.h:54-64"""
    _fields_ = [("dim", C.c_int), ("diag_num", C.c_int), ("Vector", C.POINTER(c_double_p)), ("Value", c_double_p),
                ("Error", c_double_p), ("mem_ham", C.c_double), ("Ham", C.POINTER(CRS1))]


class EXACT_BASIS_INFO(C.Structure):
    """include/exact.h:66-74"""
    _fields_ = [("dim", C.c_int), ("Basis", c_long_p), ("tot_sz", C.c_int), ("tot_ele", C.c_int),
                ("tot_parity", C.c_int)]


class EXACT_WHOLE_BASIS_Q1(C.Structure):
    """include/exact.h:89-95"""
    _fields_ = [("Dim", c_int_p), ("Basis", C.POINTER(c_long_p)), ("max_dim", C.c_int)]


class EXACT_WHOLE_BASIS_Q2(C.Structure):
    """include/exact.h:97-103"""
    _fields_ = [("Dim", C.POINTER(c_int_p)), ("Basis", C.POINTER(C.POINTER(c_long_p))), ("max_dim", C.c_int)]


class EXACT_WHOLE_BASIS_Q3(C.Structure):
    """include/exact.h:105-111"""
    _fields_ = [("Dim", C.POINTER(C.POINTER(c_int_p))), ("Basis", C.POINTER(C.POINTER(C.POINTER(c_long_p)))),
                ("max_dim", C.c_int)]


class ExactWholeBasis:
    """An EXACT_WHOLE_BASIS_Q1 / _Q2 / _Q3 over numpy arrays (include/exact.h:89-111): ``sectors``
    maps a k-tuple of non-negative quantum-number indices to that sector's ascending int64 code
    table, ``shape`` gives the extent of each index (absent sectors have dimension 0).  With
    ``pad`` each table is followed by one sentinel larger than any code (the reference's binary
    search may read one element past the table, exact/EXACT_V_M_Q1.c:29).  ``.ref`` points at the
    struct; the arrays are kept alive by this object."""

    def __init__(self, sectors: dict, shape: tuple, pad: bool = False):
        k = len(shape)
        assert 1 <= k <= 3
        self.keep = []
        empty = np.full(1, np.iinfo(np.int64).max, np.int64)
        self.keep.append(empty)

        def build(prefix, leaf, leaf_type):
            depth = len(prefix)
            if depth == k:
                return leaf(prefix)
            elem_t = leaf_type
            for _ in range(k - depth - 1):
                elem_t = C.POINTER(elem_t)
            arr = (elem_t * shape[depth])(*[build(prefix + (i,), leaf, leaf_type) for i in range(shape[depth])])
            self.keep.append(arr)
            return C.cast(arr, C.POINTER(elem_t))

        def table(prefix):
            b = sectors.get(prefix)
            if b is None or len(b) == 0:
                return empty.ctypes.data_as(c_long_p)
            a = np.ascontiguousarray(b, np.int64)
            if pad:
                a = np.concatenate([a, [np.iinfo(np.int64).max]])
            self.keep.append(a)
            return a.ctypes.data_as(c_long_p)

        dim = build((), lambda prefix: len(sectors[prefix]) if prefix in sectors else 0, C.c_int)
        basis = build((), table, c_long_p)
        T = {1: EXACT_WHOLE_BASIS_Q1, 2: EXACT_WHOLE_BASIS_Q2, 3: EXACT_WHOLE_BASIS_Q3}[k]
        self.struct = T(Dim=dim, Basis=basis, max_dim=max((len(v) for v in sectors.values()), default=0))
        self.ref = C.pointer(self.struct)


class MODEL_1DKLM_VF(C.Structure):
    """include/model.h:23-45"""
    _fields_ = [("BC", C.c_char * 1000), ("p_threads", C.c_int), ("spin_loc", C.c_int), ("tot_site", C.c_int),
                ("tot_sz", C.c_int), ("tot_ele", C.c_int), ("dim_onsite", C.c_int), ("dim_lspin", C.c_int),
                ("dim_charge", C.c_int), ("cf_origin", C.c_int), ("avg_range", C.c_double), ("t", C.c_double),
                ("J", C.c_double), ("D_z", C.c_double), ("I_xy", C.c_double), ("I_z", C.c_double), ("h_z", C.c_double),
                ("mu", C.c_double)]


class dg_solver_params(C.Structure):
    """include/dmrg_gb300.h: dg_solver_params"""
    _fields_ = [("lanczos_acc", C.c_double), ("lanczos_min_step", C.c_int), ("lanczos_max_step", C.c_int),
                ("lanczos_block_step", C.c_int), ("lanczos_tight", C.c_int), ("lanczos_slow", C.c_int),
                ("dense_below", C.c_int), ("ii_acc", C.c_double), ("ii_diag_add", C.c_double), ("ii_max_step", C.c_int),
                ("cg_acc", C.c_double), ("cg_max_step", C.c_int), ("ii_minres", C.c_int), ("mixed", C.c_int),
                ("seed", C.c_uint64), ("lookahead", C.c_int)]


class dg_solve_info(C.Structure):
    """include/dmrg_gb300.h: dg_solve_info"""
    _fields_ = [("eig_val", C.c_double), ("error", C.c_double), ("lanczos_steps", C.c_int), ("ii_steps", C.c_int),
                ("cg_steps", C.c_int), ("spmv_count", C.c_int), ("converged", C.c_int), ("ii_converged", C.c_int),
                ("dense", C.c_int), ("ms_lanczos", C.c_double), ("ms_ii", C.c_double), ("eig_lanczos", C.c_double)]


class dg_tune_result(C.Structure):
    """include/dmrg_gb300.h: dg_tune_result"""
    _fields_ = [("format", C.c_int), ("shape", C.c_int), ("variant", C.c_int), ("grid", C.c_int), ("ms", C.c_float),
                ("candidates", C.c_int), ("window", C.c_int)]


class dg_sb_term(C.Structure):
    """include/dmrg_gb300_sb.h: dg_sb_term"""
    _fields_ = [("pos1", C.c_int), ("pos2", C.c_int), ("op1", C.c_int), ("op2", C.c_int), ("coef", C.c_double),
                ("sign_mask", C.c_int), ("sign_even", C.c_int)]


class dg_sb_model(C.Structure):
    """include/dmrg_gb300_sb.h: dg_sb_model"""
    _fields_ = [("n", C.c_int), ("dim_LL", C.c_int), ("dim_RR", C.c_int), ("dim_onsite", C.c_int),
                ("LL", C.POINTER(C.c_short)), ("LR", C.POINTER(C.c_short)), ("RR", C.POINTER(C.c_short)),
                ("RL", C.POINTER(C.c_short)), ("inv", C.POINTER(C.c_int)), ("n_ops", C.c_int), ("ops", C.POINTER(CRS1)),
                ("n_terms", C.c_int), ("terms", C.POINTER(dg_sb_term)), ("ele", C.POINTER(C.c_int) * 4)]


class dg_sb_expect_term(C.Structure):
    """include/dmrg_gb300_sb.h"""
    _fields_ = [("pos", C.c_int), ("op", C.c_int), ("sign", C.c_int), ("weight", C.c_int)]


class dg_sb_basis_spec(C.Structure):
    """include/dmrg_gb300_sb.h: dg_sb_basis_spec"""
    _fields_ = [("dim_LL", C.c_int), ("dim_RR", C.c_int), ("dim_onsite", C.c_int), ("n_qn", C.c_int),
                ("qn1_LL", C.POINTER(C.c_int)), ("qn1_RR", C.POINTER(C.c_int)), ("qn1_site", C.POINTER(C.c_int)),
                ("qn2_LL", C.POINTER(C.c_int)), ("qn2_RR", C.POINTER(C.c_int)), ("qn2_site", C.POINTER(C.c_int)),
                ("target1", C.c_int), ("target2", C.c_int)]


class dg_engine_config(C.Structure):
    """include/dmrg_gb300_ed.h: dg_engine_config"""
    _fields_ = [("workers", C.c_int), ("hbm_budget", C.c_size_t), ("lanczos_batch", C.c_int), ("tune_shapes", C.c_int)]


class dg_job_result(C.Structure):
    """include/dmrg_gb300_ed.h: dg_job_result"""
    _fields_ = [("id", C.c_long), ("status", C.c_int), ("converged", C.c_int), ("eig_val", C.c_double),
                ("error", C.c_double), ("lanczos_steps", C.c_int), ("cg_steps", C.c_int), ("dim", C.c_long),
                ("nnz", C.c_long), ("t_submit_ms", C.c_double), ("t_start_ms", C.c_double), ("t_built_ms", C.c_double),
                ("t_done_ms", C.c_double)]


class dg_ed_term(C.Structure):
    """include/dmrg_gb300_ed.h"""
    _fields_ = [("kind", C.c_int), ("site1", C.c_int), ("site2", C.c_int), ("op1", C.c_int), ("op2", C.c_int),
                ("coef", C.c_double), ("sign_mode", C.c_int)]


class dg_ed_model(C.Structure):
    """include/dmrg_gb300_ed.h"""
    _fields_ = [("n_sites", C.c_int), ("dim_onsite", C.c_int), ("qn1", c_int_p), ("qn2", c_int_p), ("use_qn1", C.c_int),
                ("use_qn2", C.c_int), ("target_qn1", C.c_int), ("target_qn2", C.c_int), ("n_ops", C.c_int),
                ("ops", C.POINTER(CRS1)), ("n_terms", C.c_int), ("terms", C.POINTER(dg_ed_term)), ("n_ele", c_int_p)]


# ---------------------------------------------------------------------------------------
# numpy <-> struct helpers
# ---------------------------------------------------------------------------------------
def ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class Crs:
    """A CRS1 structure viewing numpy arrays (row int64, col int32, val float64).

    The arrays are kept alive by this object; ``.struct`` is the CRS1 and ``.ref`` a
    pointer to it."""

    def __init__(self, row, col, val, n=None, ncol=None):
        self.row = np.ascontiguousarray(row, dtype=np.int64)
        self.col = np.ascontiguousarray(col, dtype=np.int32)
        self.val = np.ascontiguousarray(val, dtype=np.float64)
        n = len(self.row) - 1 if n is None else n
        if len(self.col) == 0:          # keep valid pointers for empty matrices
            self.col = np.zeros(1, np.int32)
            self.val = np.zeros(1, np.float64)
        self.struct = CRS1(max_val=max(len(self.val), 1), max_row=n + 1, row_dim=n, col_dim=n if ncol is None else ncol,
                           Col=ptr(self.col, C.c_int), Row=ptr(self.row, C.c_long), Val=ptr(self.val, C.c_double))
        self.ref = C.pointer(self.struct)

    @property
    def n(self) -> int:
        return self.struct.row_dim

    @property
    def nnz(self) -> int:
        return int(self.row[self.n])

    @classmethod
    def from_scipy(cls, A):
        A = A.tocsr()
        A.sort_indices()
        return cls(A.indptr, A.indices, A.data, n=A.shape[0], ncol=A.shape[1])


class Ccs:
    """A CCS1 structure viewing numpy arrays (col offsets int64, row int32, val float64), kept alive
    by this object; ``.ref`` points to it."""

    def __init__(self, col, row, val, n_rows, n_cols, max_val=None):
        self.col = np.ascontiguousarray(col, dtype=np.int64)
        self.row = np.ascontiguousarray(row if len(row) else np.zeros(1), dtype=np.int32)
        self.val = np.ascontiguousarray(val if len(val) else np.zeros(1), dtype=np.float64)
        self.struct = CCS1(max_val=max_val if max_val is not None else max(len(val), 1), max_col=n_cols + 1, row_dim=n_rows,
                           col_dim=n_cols, Col=ptr(self.col, C.c_long), Row=ptr(self.row, C.c_int), Val=ptr(self.val, C.c_double))
        self.ref = C.pointer(self.struct)

    @classmethod
    def from_scipy(cls, A):
        A = A.tocsc()
        A.sort_indices()
        return cls(A.indptr, A.indices, A.data, A.shape[0], A.shape[1])

    @classmethod
    def empty(cls, n_cols, max_val):
        """An output CCS as GET_CCS1(n_cols, max_val) allocates it."""
        c = cls(np.zeros(n_cols + 1, np.int64), np.zeros(max(max_val, 1), np.int32), np.zeros(max(max_val, 1)), 0, 0, max_val)
        c.struct.max_col = n_cols + 1
        return c


def lower_diag_last(A) -> Crs:
    """Symmetric matrix -> the *_SYM layout: lower triangle, columns ascending, diagonal
    stored last in every row (explicitly, even when zero)."""
    import scipy.sparse as sp
    A = sp.csr_matrix(A)
    n = A.shape[0]
    L = sp.tril(A, k=-1).tocsr()
    L.sort_indices()
    d = A.diagonal()
    rows, cols, vals = [0], [], []
    for i in range(n):
        b, e = L.indptr[i], L.indptr[i + 1]
        cols.extend(L.indices[b:e].tolist())
        vals.extend(L.data[b:e].tolist())
        cols.append(i)
        vals.append(d[i])
        rows.append(len(cols))
    return Crs(np.array(rows), np.array(cols), np.array(vals), n=n)


def full_from_lower(c: Crs):
    """Full scipy CSR from a lower-triangle-diagonal-last Crs."""
    import scipy.sparse as sp
    n = c.n
    L = sp.csr_matrix((c.val[:c.nnz], c.col[:c.nnz], c.row), shape=(n, n))
    D = sp.diags(L.diagonal())
    return (L + L.T - D).tocsr()


def cstr(s: str) -> bytes:
    return s.encode()
