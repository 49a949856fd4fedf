"""Batched ED ground states: 256 XXZ chains of uneven size through the concurrent engine.

    python -m dmrg_c_gb300.batch_ed [--count 256] [--workers 8] [--mixed] [--lanczos-batch] [--json out.json]

Instances (dmrg_c_gb300.workloads.xxz_ed_batch, seed 0): L uniform in {12,...,22} (Sz = 0
sector dimensions 924 ... 705,432), Jz ~ U[0,2], hz ~ U[0,1], Jxy = 1, OBC.  Each instance's
basis and Hamiltonian are built on the device; solves run concurrently on the engine's
worker streams; with --lanczos-batch their Lanczos phases run in the engine's lock-step batch
(one launch of each kernel a step over all instances).  Reports batch solves/s against the same
batch run one instance at a time.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

from . import lib as L
from . import workloads


def run_batch(instances, params, workers, hbm_budget=0, lanczos_batch=False):
    """Submit every instance, wait for all; returns (wall seconds, results by index)."""
    eng = L.Engine(workers=workers, hbm_budget=hbm_budget, lanczos_batch=lanczos_batch)
    models = [inst["model"]() for inst in instances]
    t0 = time.perf_counter()
    for i, m in enumerate(models):
        eng.submit(m, params, i)
    res = {}
    while len(res) < len(models):
        for r, _ in eng.poll(256, wait_ms=50):
            res[r.id] = r
    wall = time.perf_counter() - t0
    eng.close()
    bad = [i for i, r in res.items() if r.status != 0 or not r.converged]
    if bad:
        raise RuntimeError(f"{len(bad)} instances failed, e.g. {bad[:5]}")
    return wall, res


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--count", type=int, default=256)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--mixed", action="store_true")
    ap.add_argument("--lanczos-batch", action="store_true")
    ap.add_argument("--no-sequential", action="store_true")
    ap.add_argument("--json", default=None)
    a = ap.parse_args(argv)
    inst = workloads.xxz_ed_batch(a.count, seed=0)
    p = L.default_params(seed=7, mixed=2 if a.mixed else 0)
    run_batch(inst[:8], p, a.workers, lanczos_batch=a.lanczos_batch)   # warm-up (pool, kernels)
    wall, res = run_batch(inst, p, a.workers, lanczos_batch=a.lanczos_batch)
    out = {"instances": a.count, "workers": a.workers, "form": "mixed" if a.mixed else "fp64",
           "lanczos_batch": a.lanczos_batch,
           "wall_s": wall, "solves_per_s": a.count / wall,
           "sum_dim": int(sum(r.dim for r in res.values())), "sum_nnz": int(sum(r.nnz for r in res.values()))}
    if not a.no_sequential:
        wall1, res1 = run_batch(inst, p, 1)
        out["sequential_wall_s"] = wall1
        out["sequential_solves_per_s"] = a.count / wall1
        out["max_dE_rel_vs_sequential"] = max(abs(res[i].eig_val - res1[i].eig_val) / abs(res1[i].eig_val) for i in res)
    by_L = {}
    for i, r in res.items():
        Lx = inst[i]["L"]
        d = by_L.setdefault(Lx, [])
        d.append(r.t_done_ms - r.t_start_ms)
    out["ms_per_solve_by_L"] = {int(k): float(np.median(v)) for k, v in sorted(by_L.items())}
    print(json.dumps(out))
    if a.json:
        with open(a.json, "w") as f:
            json.dump({"summary": out, "energies": {int(i): r.eig_val for i, r in res.items()}}, f)
    return 0


if __name__ == "__main__":
    sys.exit(main())
