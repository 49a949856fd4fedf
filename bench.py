#!/usr/bin/env python3
"""Benchmark: superblock ground-state solves on GB300 (one JSON line on stdout).

Workload (default ``klm_m128``): the largest superblock of the Kondo-lattice DMRG
configuration (klm_vf, L=24, N_e=12, 2Sz=0, m=128; d=8 sites) -- n = 56,612 states,
3.69e6 stored entries of the full matrix -- built from seeded synthetic block operators
(dmrg_c_gb300.workloads; no DMRG sweep runs).  One step = one ground-state solve exactly as
DMRG_DIAGONALIZE_SUPERBLOCK_SYM does it: Lanczos (acc 1e-14, Normal) then inverse iteration
(CG, ii_acc 1e-9), FP64.

* ``value``: solves/s with the matrix resident on the device, device time (CUDA events of
  the library stream) summed over K steps; L2 is flushed (256 MiB rewrite) before every step.
* ``mixed``: the same solve in the mixed-precision form (FP32 values and Krylov vectors, FP64
  recurrence, reorthogonalisation and refinement), with its energy error and eigenvector
  overlap against the FP64 result.
* ``e2e``: solves/s through the drop-in C entry point DMRG_DIAGONALIZE_SUPERBLOCK_SYM from
  host arrays (upload, device expansion, solve, eigenvector download inside the timing).
* ``roofline``: the fused SpMV kernel (product + <x,y> epilogue), CUDA-event timed with L2
  flushed before each launch (256 MiB rewritten, then another 256 MiB read, so the rewrite's dirty
  lines are written back before the timed launch); algorithmic bytes nnz_full*12 + (n+1)*4 + 2*n*8.
* ``cpu_baseline``: the oracle's OpenMP restatement of the same solve on all host cores.
* ``roofline_hbm_case``: the HBM-bound product (Hubbard m=512 superblock, 0.69 GB), FP64 with the
  autotuned shape and the mixed-precision product, L2 flushed before every launch.

``--impl reference`` times the CPU path (the oracle port of the reference's LANCZOS_SYM +
INVERSE_ITERATION_SYM; the reference itself cannot be built on the benchmark host) on the
same workload.  Multi-GPU runs (torchrun) are independent replicas.
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


def build_workload(name, seed):
    from dmrg_c_gb300 import workloads
    fn = {"klm_m128": workloads.klm_superblock_m128, "xxz_m64": workloads.xxz_superblock_m64,
          "hubbard_m512": workloads.hubbard_superblock_m512}[name]
    sb = fn(seed)
    return sb, sb.explicit_lower()


WORKLOAD_DESC = {
    "klm_m128": "klm_vf DMRG superblock, L=24 N_e=12 2Sz=0 m=128 (synthetic blocks), FP64 Lanczos + inverse iteration",
    "xxz_m64": "xxz_vf DMRG superblock, L=32 2Sz=0 m=64 (synthetic blocks), FP64 Lanczos + inverse iteration",
    "hubbard_m512": "hubbard_vf DMRG superblock, L=64 N_e=64 2Sz=0 m=512 (synthetic blocks), FP64 Lanczos + inverse iteration",
}


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


def oracle_solve(low, seed, threads):
    """The CPU path on one solve: oracle LANCZOS_SYM (Guess "No", same seeded start vector as
    the GPU run) + INVERSE_ITERATION_SYM.  Returns (seconds, energy, vector)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    t0 = time.perf_counter()
    rc, out, v = pyoracle.lanczos(low, True, seed=seed, threads=threads)
    rc2, oi, v2 = pyoracle.inverse_iteration(low, True, out.eig_val, v, cg_acc=1e-7, threads=threads)
    return time.perf_counter() - t0, out.eig_val, v2, out.steps, oi.cg_total


def spmv_bytes(n, nnz_full, s_val=8, s_vec=8):
    return nnz_full * (s_val + 4) + (n + 1) * 4 + 2 * n * s_vec


def traffic_from_profile(workload, mixed=False):
    """DRAM bytes (read + write) per launch of the SpMV kernel, from the committed ncu summary
    of this workload (profiles/k_apply_sell_[mixed_]<workload>.md), if present."""
    f = ROOT / "profiles" / f"k_apply_sell_{'mixed_' if mixed else ''}{workload}.md"
    if f.exists():
        for line in f.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                return int(line.split(":")[1])
    return None


def hbm_case_roofline(peak, peak_kind):
    """The HBM-bound product: the Hubbard m=512 superblock (n = 227,652, 57.1 M stored, 0.69 GB),
    FP64 with the autotuned shape and the mixed-precision product, CUDA-event timed with L2
    flushed before every launch (the matrix is 5x the L2)."""
    import torch
    from dmrg_c_gb300 import lib as L
    low = build_workload("hubbard_m512", 0)[1]
    m = L.DeviceMatrix(low, L.DG_STORE_LOWER_DIAG_LAST, L.DG_VALUES_BOTH)
    x = torch.randn(m.n, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    t_heur = m.profile_spmv(x, y, iters=20, flush_bytes=FLUSH_BYTES)
    t32 = m.profile_spmv_mixed(x.float(), y, iters=20, flush_bytes=FLUSH_BYTES)   # heuristic shape
    tune = m.autotune(iters=5)                                                    # FP64 shapes
    t64 = m.profile_spmv(x, y, iters=20, flush_bytes=FLUSH_BYTES)
    B64, B32 = spmv_bytes(m.n, m.nnz), spmv_bytes(m.n, m.nnz, 4, 4)
    a64, a32 = B64 / (t64 * 1e-3) / 1e9, B32 / (t32 * 1e-3) / 1e9
    out = {"workload": "hubbard_m512 superblock SpMV", "n": m.n, "nnz_full": m.nnz, "bound": "hbm", "unit": "GB/s",
           "peak": peak, "peak_source": peak_kind,
           "l2": "flushed before every launch: 256 MiB rewritten, then another 256 MiB read",
           "fp64": {"kernel": f"k_apply_sell<double> (autotuned: WS={tune.shape} variant={tune.variant} window={tune.window})",
                    "ms_per_launch": t64, "bytes_per_launch": B64, "achieved": a64, "frac": a64 / peak,
                    "traffic": traffic_from_profile("hubbard_m512"), "heuristic_ms_per_launch": t_heur},
           "mixed": {"kernel": "k_apply_sell<float> (compensated FP32 sums, heuristic shape)", "ms_per_launch": t32, "bytes_per_launch": B32,
                     "achieved": a32, "frac": a32 / peak, "traffic": traffic_from_profile("hubbard_m512", mixed=True)}}
    m.close()
    return out


def run_gb300(args, ws, rank, local_rank):
    import torch
    from dmrg_c_gb300 import abi, lib as L

    torch.cuda.set_device(local_rank)
    sb, low = build_workload(args.workload, args.seed)
    n = low.n
    nnz_full = 2 * low.nnz - n
    m = L.DeviceMatrix(low, L.DG_STORE_LOWER_DIAG_LAST, L.DG_VALUES_BOTH)
    params = L.default_params(lanczos_acc=1e-14, cg_acc=1e-7, seed=args.seed + 1)
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")

    def one_solve(p=params, o=out):
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

    # mixed-precision forms on the same superblock and start vector
    def mixed_leg(form):
        pm = L.default_params(lanczos_acc=1e-14, cg_acc=1e-7, seed=args.seed + 1, mixed=form)
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
                "speedup_vs_fp64": total_ms / sum(ms), "eig_val": Em, "dE_rel_vs_fp64": abs(Em - E) / abs(E),
                "overlap_vs_fp64": float(abs(v @ eigvec)), "lanczos_steps": infs[-1].lanczos_steps,
                "eig_lanczos_dE_rel": abs(infs[-1].eig_lanczos - E) / abs(E),
                "refine_fp32_products": infs[-1].cg_steps, "refine_steps": infs[-1].ii_steps,
                "residual_l1": infs[-1].error}

    mixed = mixed_leg(1)
    mixed["form"] = ("FP32 values + Krylov vectors (compensated FP32 sums), FP64 recurrence + full "
                     "reorthogonalisation, Jacobi-Davidson refinement against FP64 H")
    mixed_rec = mixed_leg(2)
    mixed_rec["form"] = "FP32 SpMV (compensated FP32 sums) + FP64 three-term recurrence, Jacobi-Davidson refinement"

    # the steps after the solve on the solved vector: site expectation values, truncation to m
    # states, renormalisation of a block operator (EXPECTATION_VALUES / RENORMALIZE / TRANSFORM_MATRIX)
    try:
        from dmrg_c_gb300 import dmrg_step, workloads
        qb, qs, _target, m_keep = workloads.superblock_labels(args.workload, args.seed)
        n_sites = {"klm_m128": 11, "hubbard_m512": 31, "xxz_m64": 15}[args.workload]
        post = dmrg_step.post_solve(sb, qb, qs, eigvec, m_keep, n_sites)
    except Exception as e:   # recorded, the solve measurement stands
        post = {"error": f"{type(e).__name__}: {e}"}

    # roofline of the SpMV kernel
    x = torch.randn(n, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    fmt, _stored = m.format()
    kernel = ("k_apply_sell (SELL-32 sliced ELL, one lane per row, fused <x,y> epilogue)" if fmt == L.DG_FORMAT_SELL
              else "k_apply (CSR, lanes per row, fused <x,y> epilogue)")
    spmv_ms = m.profile_spmv(x, y, iters=30, flush_bytes=FLUSH_BYTES)
    spmv_warm_ms = m.profile_spmv(x, y, iters=30, flush_bytes=0)
    B = spmv_bytes(n, nnz_full)
    peak, peak_kind = peaks()
    achieved = B / (spmv_ms * 1e-3) / 1e9

    # end to end through the reference-facing entry point, from pinned host arrays (the CRS the
    # caller holds and the eigenvector it receives)
    lib = L.load()
    pinned = [torch.from_numpy(a).pin_memory() for a in (low.row, low.col[:low.nnz], low.val[:low.nnz])]
    low_h = abi.Crs(*(t.numpy() for t in pinned), n=n)
    gs_t = torch.zeros(n, dtype=torch.float64).pin_memory()
    par = abi.DMRG_PARAMETER()
    par.Diag_Method, par.Lan_Con, par.II_Type = b"Lanczos", b"Normal", b"CG"
    par.diag_acc, par.diag_min_step, par.diag_max_step = 1e-14, 1, 800
    par.cg_acc, par.cg_max_step = 1e-7, 1000
    par.inv_iter_acc, par.inv_iter_diag_add, par.inv_iter_max_step = 1e-9, 1e-11, 3
    gs = gs_t.numpy()
    st = abi.DMRG_STATUS()
    st.GS_Vec = abi.ptr(gs, C.c_double)
    tm = abi.DMRG_TIME()
    e2e_steps = max(1, min(args.steps, 10))
    old = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        try:
            lib.DMRG_DIAGONALIZE_SUPERBLOCK_SYM(low_h.ref, C.byref(tm), C.byref(par), C.byref(st), 1)   # warm
            t0 = time.perf_counter()
            for _ in range(e2e_steps):
                flush.fill_(1)
                torch.cuda.synchronize()
                lib.DMRG_DIAGONALIZE_SUPERBLOCK_SYM(low_h.ref, C.byref(tm), C.byref(par), C.byref(st), 1)
            e2e_s = (time.perf_counter() - t0) / e2e_steps
        finally:
            os.chdir(old)
    h2d = (n + 1) * 8 + low.nnz * 4 + low.nnz * 8
    d2h = n * 8

    result = {
        "metric": METRIC, "value": job_rate(args.steps, ws, total_ms), "unit": "solves/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded block operators)",
        "config": {"workload": args.workload, "desc": WORKLOAD_DESC[args.workload], "n": n, "nnz_full": nnz_full,
                   "nnz_lower": low.nnz, "l2": "flushed (256 MiB) before every step", "parallelism": f"replicas x{ws}",
                   "lanczos_acc": 1e-14, "ii_acc": 1e-9, "cg_acc": 1e-7},
        "wall_ms_per_step": wall * 1e3 / args.steps,
        "p50_ms": float(np.percentile(dev_ms, 50)), "p99_ms": float(np.percentile(dev_ms, 99)),
        "ms_lanczos_p50": float(np.percentile([i.ms_lanczos for i in infos], 50)),
        "ms_ii_p50": float(np.percentile([i.ms_ii for i in infos], 50)),
        "lanczos_steps": infos[-1].lanczos_steps, "cg_steps": infos[-1].cg_steps, "spmv_per_solve": infos[-1].spmv_count,
        "ii_error": infos[-1].error, "eig_val": E,
        "e2e": {"value": 1.0 / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "entry": "DMRG_DIAGONALIZE_SUPERBLOCK_SYM", "gs_val": st.gs_val},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic_from_profile(args.workload), "peak_source": peak_kind,
                     "kernel": kernel, "ms_per_launch": spmv_ms,
                     "bytes_per_launch": B, "l2_warm_ms_per_launch": spmv_warm_ms,
                     "l2_warm_gbs": B / (spmv_warm_ms * 1e-3) / 1e9},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "mixed": mixed,
        "mixed_fp32_spmv": mixed_rec,
        "post_solve": post,
    }
    if rank == 0 and not args.no_hbm_case:
        result["roofline_hbm_case"] = hbm_case_roofline(peak, peak_kind)
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        secs, E_cpu, v_cpu, st_cpu, cg_cpu = oracle_solve(low, args.seed + 1, threads)
        result["cpu_baseline"] = {"value": 1.0 / secs, "unit": "solves/s", "cores": threads, "kind": "port",
                                  "sample": "1 full solve (Lanczos + inverse iteration) of the same superblock",
                                  "lanczos_steps": st_cpu, "cg_steps": cg_cpu}
        result["dE_rel_vs_cpu"] = abs(E - E_cpu) / abs(E_cpu)
        result["overlap_vs_cpu"] = float(abs(eigvec @ v_cpu))
    return result


def run_reference(args, ws, rank):
    if rank != 0:
        return None
    sb, low = build_workload(args.workload, args.seed)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        oracle_solve(low, args.seed + 1, threads)
    times = []
    E = None
    for _ in range(args.steps):
        s, E, v, st, cg = oracle_solve(low, args.seed + 1, threads)
        times.append(s)
    value = args.steps / sum(times)
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded block operators)",
            "config": {"workload": args.workload, "desc": WORKLOAD_DESC[args.workload], "n": low.n,
                       "nnz_full": 2 * low.nnz - low.n},
            "eig_val": E,
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} full solves of the workload superblock (oracle restatement of "
                                       "LANCZOS_SYM + INVERSE_ITERATION_SYM, OpenMP on all host cores)"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOAD_DESC), default="klm_m128")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-hbm-case", action="store_true", help="skip the m=512 superblock product roofline")
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
