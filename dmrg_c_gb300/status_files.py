"""The DMRG drivers' result files, written from the DMRG_STATUS / DMRG_TIME the drop-in solve fills.

A driver that calls DMRG_DIAGONALIZE_SUPERBLOCK_SYM reports every step in three files; their
line formats are the reference's, so the files of a run on this library read like the
reference's own:

* ``result/log.txt`` (and stdout): the status line of PRINT_STATUS
  (main/dmrg/<model>/src/status/PRINT_STATUS.c:16-40; three variants of one format);
* ``result/SystemInfo/Energy_<sweep>.txt``: one line per step with the superblock and system
  sizes, the step counter, E, E/N and the solve's error (OUTPUT_T_ERROR.c:99-120), after a
  model-specific two-line header on the first step of a sweep;
* ``result/[<LL+1>_1_1_<RR+1>]_<sweep>/AverageValues/energy.txt``: the model parameters with E
  and E/N (OUTPUT_ENERGY.c:11-41 of xxz_vf, klm_vf and hubbard_vf).

The formats are C printf conversions; Python's ``%`` operator rounds them identically.
"""
from __future__ import annotations

import os
from pathlib import Path


def status_line(model: str, st, tm, elapsed_s: float) -> str:
    """PRINT_STATUS's line (without the newline) of driver ``model`` (xxz_vf, klm_vf, hubbard_vf;
    main/dmrg/<model>/src/status/PRINT_STATUS.c) for a DMRG_STATUS ``st`` and DMRG_TIME ``tm``;
    ``elapsed_s`` is the step's wall time (the driver's omp_get_wtime() - Dmrg_Time->total)."""
    bc = st.BC.decode() if isinstance(st.BC, bytes) else str(st.BC)
    N = st.LL_site + st.RR_site + 4
    first = ("OBC", "SSD") if model == "xxz_vf" else ("OBC", "SSD", "PBC_LL_LR_RL_RR")
    if bc in first:
        sites = "(%-3d,1,1,%3d)" % (st.LL_site + 1, st.RR_site + 1)
        dims = "(%-4d,%-2d,%2d,%4d)" % (st.dim_LL, st.dim_onsite, st.dim_onsite, st.dim_RR)
    else:
        sites = "(%-3d,1,%3d,1)" % (st.LL_site + 1, st.RR_site + 1)
        dims = "(%-4d,%-2d,%4d,%2d)" % (st.dim_LL, st.dim_onsite, st.dim_RR, st.dim_onsite)
    head = "[%s]E/N=%.15f(%.1e),N=%-3d%s,dim=%-7d%s," % (bc, st.gs_val / N, st.gs_error, N, sites, st.dim_LLLRRRRL, dims)
    fill = st.tot_ele / N
    if model == "xxz_vf":
        mid = "Spin=%.1f, Sz=%.1f, T:" % (st.spin / 2.0, st.tot_sz / 2.0)
        tr = tm.trans_main + tm.trans_exp
    elif model == "klm_vf":
        mid = "Spin=%.1f, Sz=%-4.1f, fill=%.3f, T:" % (st.spin / 2.0, st.tot_sz / 2.0, fill)
        tr = tm.trans_main
    elif model == "hubbard_vf":
        mid = "Sz=%-4.1f,fill=%.3f,T:" % (st.tot_sz / 2.0, fill)
        tr = tm.trans_main
    else:
        raise ValueError(f"unknown model {model}")
    times = "%-6.1f(D:%-6.1f,II:%-6.1f,Ham:%-5.1f,Tr:%-4.1f)," % (elapsed_s, tm.diag, tm.inv_iter, tm.make_ham, tr)
    pct = "LL:%4.1f%%," % (st.percent_LL * 100) if (model == "xxz_vf" or bc in first) else "LL:%4.1f," % (st.percent_LL * 100)
    tail = "%3d/%3d, %2d/%d" % (st.tot_iter_now, st.tot_iter, st.param_iter_now + 1, st.param_iter)
    return head + mid + times + pct + tail + (" " if model == "xxz_vf" else "")


def energy_sweep_line(LL_site: int, RR_site: int, tot_iter_now: int, gs_val: float, gs_error: float) -> str:
    """One step's line of SystemInfo/Energy_<sweep>.txt."""
    n = LL_site + RR_site + 4
    return "%-3d  %-3d  %-3d  %+.15f  %+.15f  %.1e" % (n, LL_site + 2, tot_iter_now, gs_val, gs_val / n, gs_error)


def energy_txt_line(model: str, p: dict, gs_val: float, LL_site: int, RR_site: int) -> str:
    """The model's AverageValues/energy.txt line; ``p`` holds the MODEL_* fields it prints."""
    n = LL_site + RR_site + 4
    if model == "xxz_vf":
        return "%1.1f  %1.1f  %.4f  %.4f  %.4f  %.4f  %+.15f  %+.15f  %d  %d" % (
            p["spin"] / 2.0, p["tot_sz"] / 2.0, p["J_xy"], p["J_z"], p["D_z"], p["h_z"], gs_val, gs_val / n, 0, n - 1)
    if model == "klm_vf":
        return "%1.1f  %1.1f  %.4f  %.4f  %.4f  %.4f  %.4f  %.4f  %.4f  %+.15f  %+.15f" % (
            p["spin_loc"] / 2.0, p["tot_sz"] / 2.0, p["t"], p["J"], p["I_xy"], p["I_z"], p["D_z"], p["h_z"], p["mu"], gs_val,
            gs_val / n)
    if model == "hubbard_vf":
        return "%1.1f  %.4f  %.4f  %.4f  %.4f  %.4f  %.4f  %+.15f  %+.15f" % (
            p["tot_sz"] / 2.0, p["t1"], p["t2"], p["U"], p["V"], p["h_z"], p["mu"], gs_val, gs_val / n)
    raise ValueError(f"unknown model {model}")


def energy_txt_path(LL_site: int, RR_site: int, sweep_now: int) -> Path:
    return Path("result") / f"[{LL_site + 1}_1_1_{RR_site + 1}]_{sweep_now}" / "AverageValues" / "energy.txt"


def append(path, line: str, root=".") -> Path:
    """Appends ``line`` to ``root/path`` (creating the folders), as the drivers' "a+" files."""
    p = Path(root) / path
    os.makedirs(p.parent, exist_ok=True)
    with open(p, "a") as f:
        f.write(line + "\n")
    return p
