"""The drivers' result-file lines written by dmrg_c_gb300.status_files, against the files of the
reference's own DMRG runs (tests/golden/dmrg_<model>_steps.npz): SystemInfo/Energy_<sweep>.txt
(OUTPUT_T_ERROR.c:99-120) and AverageValues/energy.txt (OUTPUT_ENERGY.c) byte for byte from each
step's recorded gs_val / gs_error, and the PRINT_STATUS line of result/log.txt with its timing
fields masked."""
import json
import re

import numpy as np
import pytest

from conftest import GOLDEN
from dmrg_c_gb300 import abi, status_files

MODELS = [m for m in ("xxz_vf", "klm_vf", "hubbard_vf") if (GOLDEN / f"dmrg_{m}_steps.npz").exists()]
TIMES = re.compile(r"T:[^)]*\)")


def _steps(model):
    return np.load(GOLDEN / f"dmrg_{model}_steps.npz")


@pytest.mark.parametrize("model", MODELS)
def test_energy_sweep_lines_are_the_references(model):
    z = _steps(model)
    ref = {}
    for entry in z["energy_sweep_txt"]:
        k, line = str(entry).split("\t", 1)
        if line and not line.startswith("###"):
            ref.setdefault(int(k), []).append(line)
    mine = {}
    for i in range(len(z["gs_val"])):
        line = status_files.energy_sweep_line(int(z["LL_site"][i]), int(z["RR_site"][i]), i + 1, float(z["gs_val"][i]),
                                              float(z["gs_error"][i]))
        mine.setdefault(int(z["sweep"][i]), []).append(line)
    assert mine == ref


@pytest.mark.parametrize("model", MODELS)
def test_energy_txt_lines_are_the_references(model):
    z = _steps(model)
    params = json.loads(str(z["model_params"]))
    lines = [str(e) for e in z["energy_txt"]]
    for entry in lines:
        folder, line = entry.split("\t", 1)
        m = re.match(r"\[(\d+)_1_1_(\d+)\]_(\d+)", folder)
        LL, RR, sweep = int(m.group(1)) - 1, int(m.group(2)) - 1, int(m.group(3))
        i = np.flatnonzero((z["sweep"] == sweep) & (z["LL_site"] == LL) & (z["RR_site"] == RR))[-1]
        assert status_files.energy_txt_line(model, params, float(z["gs_val"][i]), LL, RR) == line
        assert str(status_files.energy_txt_path(LL, RR, sweep)).startswith(f"result/{folder}/")


@pytest.mark.parametrize("model", MODELS)
def test_status_lines_are_the_references(model):
    """The driver's bookkeeping fields (block dimensions, LL percentage, counters) are read from the
    reference line; E/N, the error, sizes and the superblock dimension come from the step log."""
    z = _steps(model)
    lines = [str(s) for s in z["log_txt"] if str(s).startswith("[")]
    assert len(lines) == len(z["gs_val"])
    pat = re.compile(r"dim=\s*\d+\s*\((\d+)\s*,(\d+)\s*,\s*\d+,\s*(\d+)\),(?:Spin=([\d.]+), )?Sz=([-\d.]+)\s*,(?: ?fill=([\d.]+),)?"
                     r".*LL:\s*([\d.]+)%,\s*(\d+)/\s*(\d+),\s*(\d+)/(\d+)")
    params = json.loads(str(z["model_params"]))
    for i, ref_line in enumerate(lines):
        g = pat.search(ref_line).groups()
        st = abi.DMRG_STATUS()
        st.BC = b"OBC"
        st.LL_site, st.RR_site = int(z["LL_site"][i]), int(z["RR_site"][i])
        st.dim_LLLRRRRL = int(z["n"][i])
        st.dim_LL, st.dim_onsite, st.dim_RR = int(g[0]), int(g[1]), int(g[2])
        st.spin = int(round(float(g[3]) * 2)) if g[3] else params.get("spin_loc", params.get("spin", 0))
        st.tot_sz = int(round(float(g[4]) * 2))
        N = st.LL_site + st.RR_site + 4
        st.tot_ele = int(round(float(g[5]) * N)) if g[5] else 0      # the electrons of the current chain
        st.percent_LL = float(g[6]) / 100.0
        st.tot_iter_now, st.tot_iter = int(g[7]), int(g[8])
        st.param_iter_now, st.param_iter = int(g[9]) - 1, int(g[10])
        st.gs_val, st.gs_error = float(z["gs_val"][i]), float(z["gs_error"][i])
        line = status_files.status_line(model, st, abi.DMRG_TIME(), 0.0)
        assert TIMES.sub("T:()", line) == TIMES.sub("T:()", ref_line)
