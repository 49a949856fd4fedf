#!/usr/bin/env python3
"""Benchmark: DMRG superblock ground-state solves on GB300 (one JSON line on stdout).

Workloads are superblocks of the reference's own DMRG runs (tests/golden/dmrg_<model>_sweep<k>.npz,
recorded from main/dmrg/<model> at the configurations below; the term list is built into the
superblock CRS on the device, bitwise the reference's GET_HAM_LLLRRRRL):

  hubbard_m512 (default)  Hubbard DMRG (hubbard_vf), OBC, L=64, t=1, U=4, N_e=64, 2Sz=0, m=512:
                          the largest superblock of the 4th finite sweep
  klm_m128                Kondo lattice DMRG (klm_vf), OBC, L=24, J=1, h_z=0.1, N_e=12, 2Sz=0, m=128
  xxz_m64                 XXZ DMRG (xxz_vf), OBC, L=32, Jxy=Jz=1, 2Sz=0, m=64

One step = one ground-state solve as DMRG_DIAGONALIZE_SUPERBLOCK_SYM does it: Lanczos (acc 1e-14,
"Normal"; Lanczos_Slow for xxz_vf) then inverse iteration with CG (the driver's cg_acc), FP64.

* ``value``: solves/s with the matrix resident on the device; the device time of each solve
  (CUDA events on the library stream) summed over K steps.  Inputs larger than L2 (hubbard_m512:
  0.69 GB of CRS) or L2 flushed (256 MiB rewrite) before every step (the smaller workloads).
* ``e2e``: solves/s through the drop-in entry point DMRG_DIAGONALIZE_SUPERBLOCK_SYM from pinned
  host arrays (lower-triangle CRS upload, device expansion, solve, eigenvector download), every
  step timed on its own.
* ``mixed`` / ``mixed_fp32_spmv``: the mixed-precision forms on the same superblock, with their
  energy error against the reference's gs_val and the FP64 result.
* ``sweeps``: every recorded sweep superblock of klm_vf and hubbard_vf solved FP64 and in both
  mixed forms: |dE|/|E| against the reference's gs_val per sweep.
* ``roofline``: the fused FP64 product kernel on the workload, CUDA-event timed, algorithmic bytes
  nnz_full*12 + (n+1)*4 + 2*n*8 per launch; ``roofline_mixed`` the FP32-value product, with the
  bytes of the layout it reads (the 16-bit column-delta stream when the matrix has one) and the
  CRS-equivalent rate beside them.
* ``cpu_baseline``: the oracle's OpenMP restatement of the same solve on all host cores.

``--impl reference`` times the CPU path (the oracle port of the reference's LANCZOS_SYM +
INVERSE_ITERATION_SYM; the reference itself cannot be built on the benchmark host) on the same
superblock.  Multi-GPU runs (torchrun) are independent replicas.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "ground-state solves/s and SpMV GB/s, mixed vs FP64 at |dE|<1e-10; p50/p99 ms"
FLUSH_BYTES = 256 << 20
L2_BYTES = 129 << 20
GOLDEN = ROOT / "tests" / "golden"

WORKLOADS = {
    "hubbard_m512": ("dmrg_hubbard_vf_sweep4.npz",
                     "hubbard_vf DMRG superblock (reference run, 4th sweep's largest): L=64 t=1 U=4 N_e=64 2Sz=0 m=512, "
                     "FP64 Lanczos + inverse iteration"),
    "klm_m128": ("dmrg_klm_vf_sweep4.npz",
                 "klm_vf DMRG superblock (reference run, 4th sweep's largest): L=24 J=1 h_z=0.1 N_e=12 2Sz=0 m=128, "
                 "FP64 Lanczos + inverse iteration"),
    "xxz_m64": ("dmrg_xxz_vf_sweep4.npz",
                "xxz_vf DMRG superblock (reference run, 4th sweep's largest): L=32 Jxy=Jz=1 2Sz=0 m=64, "
                "FP64 Lanczos_Slow + inverse iteration"),
}


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    return ws, int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0"))


def replica_barrier(ws):
    """Line all replicas up before and after the timed region (no-op for one process)."""
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def replica_time(total_ms, ws, device="cuda"):
    """Max over replicas of the timed region (ms): every replica solves the same workload
    independently, so the job's throughput is ws * steps over the slowest replica's time."""
    if ws <= 1:
        return float(total_ms)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(steps, ws, max_ms):
    """Whole-job solves/s over all replicas."""
    return ws * steps / (max_ms * 1e-3)


def load_workload(name):
    from dmrg_c_gb300 import sb_models
    return sb_models.load_dmrg_superblock(GOLDEN / WORKLOADS[name][0])


def solver_settings(name):
    """The driver's settings (main/dmrg/<model>/src/main/main.c): Lanczos_Slow, cg_acc 1e-6 and
    1000 steps for xxz_vf; Lanczos, 1e-7 and 2000 for klm_vf / hubbard_vf."""
    xxz = name.startswith("xxz")
    return dict(slow=xxz, cg_acc=1e-6 if xxz else 1e-7, cg_max_step=1000 if xxz else 2000)


def config_dict(name, n, nnz_full):
    """The workload description both arms print."""
    s = solver_settings(name)
    return {"workload": name, "desc": WORKLOADS[name][1], "source": f"tests/golden/{WORKLOADS[name][0]}", "n": int(n),
            "nnz_full": int(nnz_full), "lanczos_acc": 1e-14, "ii_acc": 1e-9, "cg_acc": s["cg_acc"],
            "l2": ("inputs larger than L2" if spmv_bytes(n, nnz_full) > 2 * L2_BYTES
                   else "flushed (256 MiB rewrite) before every step")}


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons, sampled every 20 ms from before the warm-up; each
    line is time-stamped on arrival and summary() keeps the samples of the timed window
    (window(t0, t1), perf_counter seconds)."""

    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []          # (arrival time, line)
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "20"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def wait_first(self, timeout=3.0):
        """Block until nvidia-smi has produced a line (so that the timed region is covered)."""
        t_end = time.perf_counter() + timeout
        while self.proc and not self.lines and time.perf_counter() < t_end:
            time.sleep(0.005)

    def window(self, t0, t1):
        self.t0, self.t1 = t0, t1

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines
        if self.t0 is not None:
            inside = [x for x in lines if self.t0 <= x[0] <= self.t1 + 0.02]
            # a window shorter than the sampling interval: the nearest sample stands in
            lines = inside or sorted(lines, key=lambda x: abs(x[0] - 0.5 * (self.t0 + self.t1)))[:1]
        for _, ln in lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm),
                "interval_ms": 20}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def spmv_bytes(n, nnz_full, s_val=8, s_vec=8):
    return nnz_full * (s_val + 4) + (n + 1) * 4 + 2 * n * s_vec


def sell_mixed_bytes(m, n, nnz_full):
    """Bytes one FP32 (mixed) product must move in the layout it runs on.  With the 16-bit delta
    stream: every stored slot's delta (2 B) and FP32 value (4 B), the 32-bit checkpoints, the slot
    row map, the per-slice offsets / widths / checkpoint offsets, x (FP32) and y (FP64); else the
    CRS footprint nnz_full*8 + (n+1)*4 + 2*n*4."""
    from dmrg_c_gb300 import lib as L
    cfg = m.sell_config()
    present, _bridges = m.sell_deltas()
    fmt, stored = m.format()
    if fmt != L.DG_FORMAT_SELL or not present or cfg["variant32"] not in (5, 6):
        return spmv_bytes(n, nnz_full, 4, 4), "CRS footprint: nnz_full*8 + (n+1)*4 + 2*n*4"
    nslices = -(-n // 2048) * 2048 // 32
    b = stored * 6 + m.sell_checkpoints() * 4 + nslices * 32 * 4 + nslices * 20 + n * 4 + n * 8
    return b, ("delta layout: stored slots*(2+4) + checkpoints*4 + slot rows*4 + slices*20 + n*4 (x) "
               "+ n*8 (y)")


def traffic_from_profile(name, mixed=False):
    """DRAM bytes (read + write) per launch of the product kernel, from the committed ncu summary of
    this workload (profiles/k_apply_sell_[mixed_]<workload>.md, line traffic_bytes_per_launch)."""
    f = ROOT / "profiles" / f"k_apply_sell_{'mixed_' if mixed else ''}{name}.md"
    if f.exists():
        for line in f.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                return int(line.split(":")[1])
    return None


def oracle_superblock(sb, threads):
    """The workload's lower-triangle CRS built on the host by the oracle (bitwise the device build)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    from dmrg_c_gb300 import abi
    row, col, val = pyoracle.sb_build(sb.model, threads=threads)
    return abi.Crs(row, col, val, n=sb.model.n)


def oracle_solve(low, settings, seed, threads):
    """The CPU path on one solve: oracle LANCZOS[_SLOW]_SYM (Guess "No", seeded start vector) +
    INVERSE_ITERATION_SYM with CG.  Returns (seconds, energy, vector, Lanczos steps, CG steps)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    t0 = time.perf_counter()
    rc, out, v = pyoracle.lanczos(low, True, seed=seed, slow=settings["slow"], threads=threads)
    rc2, oi, v2 = pyoracle.inverse_iteration(low, True, out.eig_val, v, cg_acc=settings["cg_acc"],
                                             cg_max_step=settings["cg_max_step"], threads=threads)
    return time.perf_counter() - t0, out.eig_val, v2, out.steps, oi.cg_total


def cpu_sample(low, settings, seed, threads, min_solves=5, budget_s=30.0):
    """Times whole CPU solves: at least min_solves, more while under budget_s."""
    times, E, v = [], None, None
    while len(times) < min_solves or sum(times) < budget_s * 0.5:
        s, E, v, st, cg = oracle_solve(low, settings, seed, threads)
        times.append(s)
        if sum(times) > budget_s and len(times) >= min_solves:
            break
    return times, E, v, st, cg


def solve_params(L, name, seed, mixed=0):
    s = solver_settings(name)
    return L.default_params(lanczos_acc=1e-14, cg_acc=s["cg_acc"], cg_max_step=s["cg_max_step"],
                            lanczos_slow=int(s["slow"]), seed=seed, mixed=mixed)


def sweeps_leg(L, seed, models=("klm_vf", "hubbard_vf")):
    """Every recorded sweep superblock of the models, FP64 and both mixed forms: |dE|/|E| against
    the reference's gs_val of that superblock, and solve times."""
    from dmrg_c_gb300 import sb_models
    out = {}
    for model in models:
        name = {"klm_vf": "klm_m128", "hubbard_vf": "hubbard_m512", "xxz_vf": "xxz_m64"}[model]
        rows = []
        for path in sorted(GOLDEN.glob(f"dmrg_{model}_sweep*.npz")):
            sb = sb_models.load_dmrg_superblock(path)
            s = L.SuperblockCRS(sb.model)
            m = s.matrix(L.DG_VALUES_BOTH)
            row = {"sweep": sb.sweep, "n": sb.model.n, "gs_val_ref": sb.gs_val}
            for mixed, tag in ((0, "fp64"), (1, "mixed1"), (2, "mixed2")):
                v, info = L.ground_state(m, solve_params(L, name, seed, mixed))
                ov = abs(v @ sb.gs_vec) / (np.linalg.norm(v) * np.linalg.norm(sb.gs_vec))
                row[tag] = {"eig_val": info.eig_val, "dE_rel_vs_ref": abs(info.eig_val - sb.gs_val) / abs(sb.gs_val),
                            "overlap_vs_ref": float(ov), "ms": info.ms_lanczos + info.ms_ii,
                            "lanczos_steps": info.lanczos_steps}
            for tag in ("mixed1", "mixed2"):
                row[tag]["dE_rel_vs_fp64"] = abs(row[tag]["eig_val"] - row["fp64"]["eig_val"]) / abs(row["fp64"]["eig_val"])
            rows.append(row)
            m.close()
            s.close()
        out[model] = rows
    return out


def _engine_run(eng, models, params, arrivals=None):
    """Every model through the engine (arrivals: submission times in s, else all at once); returns
    (wall s, {index: dg_job_result}).  One engine serves the warm-up and the timed runs, as a
    serving process would."""
    res = {}
    t0 = time.perf_counter()
    for i, m in enumerate(models):
        if arrivals is not None:
            while True:
                dt = t0 + arrivals[i] - time.perf_counter()
                if dt <= 0:
                    break
                for r, _ in eng.poll(256, wait_ms=0):
                    res[r.id] = r
                time.sleep(min(dt, 0.002))
        eng.submit(m, params, i)
    while len(res) < len(models):
        for r, _ in eng.poll(256, wait_ms=50):
            res[r.id] = r
    wall = time.perf_counter() - t0
    bad = [i for i, r in res.items() if r.status != 0 or not r.converged]
    if bad:
        raise RuntimeError(f"{len(bad)} engine jobs failed, e.g. {bad[:4]}")
    return wall, res


def oracle_ed_solve(model, threads):
    """One ED instance on the CPU: the oracle's basis and CRS build, LANCZOS (Guess "No", seeded)
    and INVERSE_ITERATION with CG.  Returns (seconds, energy)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    from dmrg_c_gb300 import abi
    t0 = time.perf_counter()
    basis, row, col, val = pyoracle.ed_build(model, threads=threads)
    H = abi.Crs(row, col, val, n=len(basis))
    rc, out, v = pyoracle.lanczos(H, False, seed=7, threads=threads)
    pyoracle.inverse_iteration(H, False, out.eig_val, v, threads=threads)
    return time.perf_counter() - t0, out.eig_val


def batched_leg(L, args):
    """The batched form on the 256 XXZ chains of the batched-ED workload (L in {12..22}, Jz ~ U[0,2],
    hz ~ U[0,1], seed 0): FP64 and mixed (mixed = 2) through the engine (device build + solve per
    chain) with its lock-step Lanczos, beside the engine without it, and through the lock-step API
    (dg_batch_ground_state) on the matrices built once and kept resident; every mixed energy against
    the FP64 one."""
    from dmrg_c_gb300 import workloads
    inst = workloads.xxz_ed_batch(256, seed=0)
    models = [i["model"]() for i in inst]
    out = {"workload": "256 XXZ chains, L in {12,...,22} (n 924 ... 705,432), Jz ~ U[0,2], hz ~ U[0,1], seed 0",
           "unit": "solves/s"}
    E = {}
    for tag, mixed, lb in (("fp64", 0, True), ("mixed", 2, True), ("fp64_streams", 0, False), ("mixed_streams", 2, False)):
        p = L.default_params(seed=7, mixed=mixed)
        # the lock-step legs take the launch shapes tuned per size class (dg_shape_cache_apply);
        # the warm-up runs every chain length once, so the timed runs find every class tuned
        eng = L.Engine(workers=8, lanczos_batch=lb, tune_shapes=lb)
        _engine_run(eng, models[:16], p)                        # warm-up
        if lb:
            _engine_run(eng, models[::8], p)
        walls = []
        for _ in range(2):
            wall, res = _engine_run(eng, models, p)
            walls.append(wall)
        eng.close()
        E[tag] = np.array([res[i].eig_val for i in range(len(models))])
        out[tag] = {"value": len(models) / min(walls), "wall_ms": 1e3 * min(walls), "lanczos_batch": lb,
                    "tune_shapes": lb, "tuned_classes": L.shape_cache_size(),
                    "p50_ms_per_job": float(np.percentile([r.t_done_ms - r.t_submit_ms for r in res.values()], 50))}
    # the lock-step API on the same chains, matrices built once and resident (solves only)
    eds = [L.EDSystem(m) for m in models]
    mats = [e.matrix(L.DG_VALUES_BOTH) for e in eds]
    for e in eds:
        e.close()
    for tag, mixed in (("fp64_api", 0), ("mixed_api", 2)):
        p = L.default_params(seed=7, mixed=mixed)
        L.batch_ground_state(mats[:16], p, want_vectors=False)   # warm-up
        walls = []
        for _ in range(2):
            t0 = time.perf_counter()
            _, infos = L.batch_ground_state(mats, p, want_vectors=False)
            walls.append(time.perf_counter() - t0)
        E[tag] = np.array([i.eig_val for i in infos])
        out[tag] = {"value": len(mats) / min(walls), "wall_ms": 1e3 * min(walls),
                    "entry": "dg_batch_ground_state, matrices resident (build excluded)"}
    del mats
    out["mixed_speedup_vs_fp64_api"] = out["mixed_api"]["value"] / out["fp64_api"]["value"]
    out["max_dE_rel_mixed_vs_fp64_api"] = float(np.max(np.abs(E["mixed_api"] - E["fp64_api"]) / np.abs(E["fp64_api"])))
    out["mixed_speedup_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["lanczos_batch_speedup_fp64"] = out["fp64"]["value"] / out["fp64_streams"]["value"]
    out["max_dE_rel_mixed_vs_fp64"] = float(np.max(np.abs(E["mixed"] - E["fp64"]) / np.abs(E["fp64"])))
    out["max_dE_rel_batch_vs_streams"] = float(np.max(np.abs(E["fp64"] - E["fp64_streams"]) / np.abs(E["fp64_streams"])))
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sample = []
        for Lx in (12, 14, 16, 18, 20, 22):
            sample += [i for i in range(len(inst)) if inst[i]["L"] == Lx][:1]
        secs = {}
        for i in sample:
            t, e = oracle_ed_solve(models[i], threads)
            secs[inst[i]["L"]] = t
        total = sum(secs[i["L"]] for i in inst)     # sequential FIFO over the whole batch
        out["cpu_baseline"] = {"value": len(inst) / total, "unit": "solves/s", "cores": threads, "kind": "port",
                               "cpu": cpu_model(), "sample": "one instance of each L solved by the oracle (ED build + "
                               "LANCZOS + INVERSE_ITERATION), extrapolated to the batch's L mix, one after another",
                               "sec_by_L": {int(k): v for k, v in secs.items()}}
    return out


def served_leg(L, args):
    """The served form: the Hubbard request stream (L in {8,10,12}, U ~ U[0,8], h ~ U[0,0.5], half
    filling, Poisson arrivals at 200/s, seed 1) replayed in real time for --served-seconds, FP64 and
    mixed, through the engine's continuous lock-step batch; p50/p99 latency, solves/s, each mixed
    energy against the FP64 one; and the capacity of each form on an 800/s stream."""
    from dmrg_c_gb300 import workloads
    trace = workloads.hubbard_request_trace(rate=200.0, duration=args.served_seconds, seed=1)
    models = [r["model"]() for r in trace]
    arr = [r["t"] for r in trace]
    out = {"workload": f"Hubbard ED requests, Poisson 200/s for {args.served_seconds:g} s, L in {{8,10,12}}, seed 1",
           "requests": len(trace)}
    E = {}
    for tag, mixed in (("fp64", 0), ("mixed", 2)):
        p = L.default_params(seed=11, mixed=mixed)
        eng = L.Engine(workers=8, lanczos_batch=True)
        _engine_run(eng, models[:16], p)
        wall, res = _engine_run(eng, models, p, arrivals=arr)
        lat = np.array([res[i].t_done_ms - res[i].t_submit_ms for i in range(len(models))])
        first = min(r.t_submit_ms for r in res.values())
        last = max(r.t_done_ms for r in res.values())
        E[tag] = np.array([res[i].eig_val for i in range(len(models))])
        out[tag] = {"solves_per_s": len(models) / ((last - first) * 1e-3), "p50_ms": float(np.percentile(lat, 50)),
                    "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean())}
        # capacity: the same requests offered at 800/s for 5 s
        cap_trace = workloads.hubbard_request_trace(rate=800.0, duration=5.0, seed=2)
        cap_models = [r["model"]() for r in cap_trace]
        wall, res = _engine_run(eng, cap_models, p, arrivals=[r["t"] for r in cap_trace])
        eng.close()
        first = min(r.t_submit_ms for r in res.values())
        last = max(r.t_done_ms for r in res.values())
        out[tag]["capacity_solves_per_s"] = len(cap_models) / ((last - first) * 1e-3)
    out["mixed_capacity_speedup_vs_fp64"] = out["mixed"]["capacity_solves_per_s"] / out["fp64"]["capacity_solves_per_s"]
    out["max_dE_rel_mixed_vs_fp64"] = float(np.max(np.abs(E["mixed"] - E["fp64"]) / np.abs(E["fp64"])))
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        secs = {}
        for Lx in (8, 10, 12):
            i = next(k for k in range(len(trace)) if trace[k]["L"] == Lx)
            secs[Lx], _ = oracle_ed_solve(models[i], threads)
        total = sum(secs[r["L"]] for r in trace)     # sequential FIFO over the stream's requests
        out["cpu_baseline"] = {"value": len(trace) / total, "unit": "solves/s", "cores": threads, "kind": "port",
                               "cpu": cpu_model(), "sample": "one request of each L solved by the oracle (ED build + "
                               "LANCZOS + INVERSE_ITERATION), extrapolated to the stream's L mix, one after another: "
                               "the capacity of a sequential FIFO server",
                               "sec_by_L": {int(k): v for k, v in secs.items()}}
    return out


def run_gb300(args, ws, rank, local_rank):
    import torch
    from dmrg_c_gb300 import abi, lib as L

    torch.cuda.set_device(local_rank)
    sb = load_workload(args.workload)
    settings = solver_settings(args.workload)
    sbc = L.SuperblockCRS(sb.model)                      # the reference's CRS, built on the device
    row_h, col_h, val_h = sbc.download()
    low = abi.Crs(row_h, col_h, val_h, n=sb.model.n)
    n = low.n
    nnz_full = 2 * low.nnz - n
    m = sbc.matrix(L.DG_VALUES_BOTH)
    params = solve_params(L, args.workload, args.seed + 1)
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    small = spmv_bytes(n, nnz_full) <= 2 * L2_BYTES
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")

    def one_solve(p=params, o=out):
        if small:
            flush.fill_(1)
            torch.cuda.synchronize()
        v, info = L.ground_state(m, p, guess=None, out=o)
        if not info.converged:
            raise RuntimeError("Lanczos did not converge")
        return info

    with ClockSampler(local_rank) as clk:
        for _ in range(args.warmup):
            one_solve()
        clk.wait_first()
        replica_barrier(ws)
        torch.cuda.synchronize()
        launches0 = L.kernel_launches()
        dev_ms, infos = [], []
        t0 = time.perf_counter()
        for _ in range(args.steps):
            info = one_solve()
            infos.append(info)
            dev_ms.append(info.ms_lanczos + info.ms_ii)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        wall = t1 - t0
        clk.window(t0, t1)
    launches = L.kernel_launches() - launches0
    replica_barrier(ws)
    total_ms = replica_time(float(sum(dev_ms)), ws)
    eigvec = out.cpu().numpy()
    E = infos[-1].eig_val
    ov_ref = abs(eigvec @ sb.gs_vec) / (np.linalg.norm(eigvec) * np.linalg.norm(sb.gs_vec))

    def mixed_leg(form):
        pm = solve_params(L, args.workload, args.seed + 1, mixed=form)
        o = torch.empty(n, dtype=torch.float64, device="cuda")
        for _ in range(args.warmup):
            one_solve(pm, o)
        ms, infs = [], []
        for _ in range(args.steps):
            info = one_solve(pm, o)
            infs.append(info)
            ms.append(info.ms_lanczos + info.ms_ii)
        v = o.cpu().numpy()
        Em = infs[-1].eig_val
        return {"value": ws * args.steps / (sum(ms) * 1e-3), "unit": "solves/s", "ms_per_step": sum(ms) / args.steps,
                "p50_ms": float(np.percentile(ms, 50)), "p99_ms": float(np.percentile(ms, 99)),
                "speedup_vs_fp64": total_ms / sum(ms), "eig_val": Em, "dE_rel_vs_ref": abs(Em - sb.gs_val) / abs(sb.gs_val),
                "dE_rel_vs_fp64": abs(Em - E) / abs(E), "overlap_vs_ref": float(abs(v @ sb.gs_vec) / np.linalg.norm(sb.gs_vec)),
                "lanczos_steps": infs[-1].lanczos_steps,
                "eig_lanczos_dE_rel": abs(infs[-1].eig_lanczos - E) / abs(E),
                "refine_fp32_products": infs[-1].cg_steps, "refine_steps": infs[-1].ii_steps,
                "residual_l1": infs[-1].error}

    mixed = mixed_leg(1)
    mixed["form"] = ("FP32 values + Krylov vectors (compensated FP32 sums), FP64 recurrence + full "
                     "reorthogonalisation, Jacobi-Davidson refinement against FP64 H")
    mixed_rec = mixed_leg(2)
    mixed_rec["form"] = "FP32 SpMV (compensated FP32 sums) + FP64 three-term recurrence, Jacobi-Davidson refinement"

    # roofline of the product kernels
    x = torch.randn(n, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    fmt, _stored = m.format()
    kernel = ("k_apply_sell (SELL-32 sliced ELL, one lane per row, fused <x,y> epilogue)" if fmt == L.DG_FORMAT_SELL
              else "k_apply (CSR, lanes per row, fused <x,y> epilogue)")
    spmv_ms = m.profile_spmv(x, y, iters=30, flush_bytes=FLUSH_BYTES)
    spmv_warm_ms = m.profile_spmv(x, y, iters=30, flush_bytes=0)
    spmv32_ms = m.profile_spmv_mixed(x.float(), y, iters=30, flush_bytes=FLUSH_BYTES)
    B = spmv_bytes(n, nnz_full)
    B32, B32_basis = sell_mixed_bytes(m, n, nnz_full)
    B32_crs = spmv_bytes(n, nnz_full, 4, 4)
    peak, peak_kind = peaks()
    achieved, achieved32 = B / (spmv_ms * 1e-3) / 1e9, B32 / (spmv32_ms * 1e-3) / 1e9

    # end to end through the reference-facing entry point, from pinned host arrays (the CRS the
    # caller holds and the eigenvector it receives); every step timed on its own
    lib = L.load()
    pinned = [torch.from_numpy(a).pin_memory() for a in (low.row, low.col[:low.nnz], low.val[:low.nnz])]
    low_h = abi.Crs(*(t.numpy() for t in pinned), n=n)
    gs_t = torch.zeros(n, dtype=torch.float64).pin_memory()
    par = abi.DMRG_PARAMETER()
    par.Diag_Method = b"Lanczos_Slow" if settings["slow"] else b"Lanczos"
    par.Lan_Con, par.II_Type, par.Initial_Guess = b"Normal", b"CG", b"No"
    par.diag_acc, par.diag_min_step, par.diag_max_step = 1e-14, 1, 800
    par.cg_acc, par.cg_max_step = settings["cg_acc"], settings["cg_max_step"]
    par.inv_iter_acc, par.inv_iter_diag_add, par.inv_iter_max_step = 1e-9, 1e-11, 3
    gs = gs_t.numpy()
    st = abi.DMRG_STATUS()
    st.GS_Vec = abi.ptr(gs, C.c_double)
    tm = abi.DMRG_TIME()
    e2e_ms = []
    old = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        try:
            for _ in range(args.warmup):
                lib.DMRG_DIAGONALIZE_SUPERBLOCK_SYM(low_h.ref, C.byref(tm), C.byref(par), C.byref(st), 1)
            for _ in range(args.steps):
                if small:
                    flush.fill_(1)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                lib.DMRG_DIAGONALIZE_SUPERBLOCK_SYM(low_h.ref, C.byref(tm), C.byref(par), C.byref(st), 1)
                e2e_ms.append((time.perf_counter() - t0) * 1e3)
        finally:
            os.chdir(old)
    e2e_max_ms = replica_time(float(sum(e2e_ms)), ws)
    h2d = (n + 1) * 8 + low.nnz * 4 + low.nnz * 8
    d2h = n * 8

    result = {
        "metric": METRIC, "value": job_rate(args.steps, ws, total_ms), "unit": "solves/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "superblocks recorded from the reference's own DMRG run (tests/golden)",
        "config": config_dict(args.workload, n, nnz_full),
        "parallelism": f"replicas x{ws}",
        "wall_ms_per_step": wall * 1e3 / args.steps,
        "p50_ms": float(np.percentile(dev_ms, 50)), "p99_ms": float(np.percentile(dev_ms, 99)),
        "ms_lanczos_p50": float(np.percentile([i.ms_lanczos for i in infos], 50)),
        "ms_ii_p50": float(np.percentile([i.ms_ii for i in infos], 50)),
        "lanczos_steps": infos[-1].lanczos_steps, "cg_steps": infos[-1].cg_steps, "spmv_per_solve": infos[-1].spmv_count,
        "ii_error": infos[-1].error, "eig_val": E, "gs_val_ref": sb.gs_val,
        "dE_rel_vs_ref": abs(E - sb.gs_val) / abs(sb.gs_val), "overlap_vs_ref": float(ov_ref),
        "e2e": {"value": job_rate(args.steps, ws, e2e_max_ms), "unit": "solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "entry": "DMRG_DIAGONALIZE_SUPERBLOCK_SYM",
                "p50_ms": float(np.percentile(e2e_ms, 50)), "p99_ms": float(np.percentile(e2e_ms, 99)),
                "gs_val": st.gs_val, "dE_rel_vs_ref": abs(st.gs_val - sb.gs_val) / abs(sb.gs_val)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic_from_profile(args.workload), "peak_source": peak_kind,
                     "kernel": kernel, "ms_per_launch": spmv_ms, "bytes_per_launch": B,
                     "l2": "flushed before every launch: 256 MiB rewritten, then another 256 MiB read",
                     "l2_warm_ms_per_launch": spmv_warm_ms, "l2_warm_gbs": B / (spmv_warm_ms * 1e-3) / 1e9},
        "roofline_mixed": {"bound": "hbm", "achieved": achieved32, "peak": peak, "unit": "GB/s", "frac": achieved32 / peak,
                           "traffic": traffic_from_profile(args.workload, mixed=True), "peak_source": peak_kind,
                           "kernel": "k_apply_sell<float> (FP32 values and x, compensated FP32 sums)",
                           "sell_config": m.sell_config(), "ms_per_launch": spmv32_ms, "bytes_per_launch": B32,
                           "bytes_basis": B32_basis, "crs_bytes_per_launch": B32_crs,
                           "crs_equivalent_gbs": B32_crs / (spmv32_ms * 1e-3) / 1e9},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "mixed": mixed,
        "mixed_fp32_spmv": mixed_rec,
    }
    if rank == 0 and not args.no_sweeps:
        result["sweeps"] = sweeps_leg(L, args.seed + 1)
    if rank == 0 and not args.no_ed:
        result["batched"] = batched_leg(L, args)
        result["served"] = served_leg(L, args)
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        times, E_cpu, v_cpu, st_cpu, cg_cpu = cpu_sample(low, settings, args.seed + 1, threads)
        result["cpu_baseline"] = {"value": len(times) / sum(times), "unit": "solves/s", "cores": threads, "kind": "port",
                                  "cpu": cpu_model(),
                                  "sample": f"{len(times)} full solves (Lanczos + inverse iteration) of the same superblock",
                                  "lanczos_steps": st_cpu, "cg_steps": cg_cpu}
        result["dE_rel_vs_cpu"] = abs(E - E_cpu) / abs(E_cpu)
        result["overlap_vs_cpu"] = float(abs(eigvec @ v_cpu))
    m.close()
    sbc.close()
    return result


def run_reference(args, ws, rank):
    if rank != 0:
        return None
    sb = load_workload(args.workload)
    settings = solver_settings(args.workload)
    threads = os.cpu_count() or 1
    low = oracle_superblock(sb, threads)
    for _ in range(min(args.warmup, 2)):
        oracle_solve(low, settings, args.seed + 1, threads)
    times = []
    E = None
    for _ in range(args.steps):
        s, E, v, st, cg = oracle_solve(low, settings, args.seed + 1, threads)
        times.append(s)
    value = args.steps / sum(times)
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "superblocks recorded from the reference's own DMRG run (tests/golden)",
            "config": config_dict(args.workload, low.n, 2 * low.nnz - low.n),
            "eig_val": E, "dE_rel_vs_ref": abs(E - sb.gs_val) / abs(sb.gs_val),
            "p50_ms": float(np.percentile(times, 50)) * 1e3, "p99_ms": float(np.percentile(times, 99)) * 1e3,
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port", "cpu": cpu_model(),
                             "sample": f"{args.steps} full solves of the workload superblock (oracle restatement of "
                                       f"LANCZOS{'_SLOW' if settings['slow'] else ''}_SYM + INVERSE_ITERATION_SYM, "
                                       "OpenMP on all host cores), after min(W, 2) untimed solves"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="hubbard_m512")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-sweeps", action="store_true", help="skip the per-sweep energy errors")
    ap.add_argument("--no-ed", action="store_true", help="skip the batched and served ED legs")
    ap.add_argument("--served-seconds", type=float, default=20.0, help="length of the served request stream")
    args = ap.parse_args(argv)
    ws, rank, local_rank = dist_info()
    if args.impl == "reference":
        res = run_reference(args, ws, rank)
        if res is not None:
            print(json.dumps(res), flush=True)
        return 0
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    res = run_gb300(args, ws, rank, local_rank)
    if rank == 0:
        print(json.dumps(res), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
