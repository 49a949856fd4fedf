"""Served ED ground states: a Poisson request stream replayed in real time against the engine.

    python -m dmrg_c_gb300.serve [--rate 200] [--seconds 60] [--workers 8] [--mixed] [--lanczos-batch]

Requests (dmrg_c_gb300.workloads.hubbard_request_trace, seed 1): 1D Hubbard chains, OBC,
half filling, 2Sz = 0, L in {8,10,12} (dimensions 4,900 / 63,504 / 853,776), t = 1,
U ~ U[0,8], h ~ U[0,0.5].  Each request is submitted at its arrival time; the engine admits
it when a worker is free and its memory estimate fits the device budget, so requests that
arrive while others run are solved concurrently with them.  Latency = completion time -
arrival (submission) time on the engine clock; reported as p50 / p99 beside solves/s.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

from . import lib as L
from . import workloads


def serve(trace, params, workers, hbm_budget=0, lanczos_batch=False):
    models = [req["model"]() for req in trace]
    eng = L.Engine(workers=workers, hbm_budget=hbm_budget, lanczos_batch=lanczos_batch)
    res = {}
    max_queue = 0
    t0 = time.perf_counter()
    for i, (req, m) in enumerate(zip(trace, models)):
        while True:
            dt = t0 + req["t"] - time.perf_counter()
            if dt <= 0:
                break
            for r, _ in eng.poll(256, wait_ms=0):
                res[r.id] = r
            time.sleep(min(dt, 0.002))
        eng.submit(m, params, i)
        max_queue = max(max_queue, eng.pending()[0])
    while len(res) < len(models):
        for r, _ in eng.poll(256, wait_ms=50):
            res[r.id] = r
    eng.close()
    return res, max_queue


def summarize(trace, res):
    lat = np.array([res[i].t_done_ms - res[i].t_submit_ms for i in range(len(trace))])
    first = min(r.t_submit_ms for r in res.values())
    last = max(r.t_done_ms for r in res.values())
    failed = sum(1 for r in res.values() if r.status != 0 or not r.converged)
    by_L = {}
    for i, req in enumerate(trace):
        by_L.setdefault(req["L"], []).append(lat[i])
    return {"requests": len(trace), "failed": failed, "solves_per_s": len(trace) / ((last - first) * 1e-3),
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()),
            "p50_ms_by_L": {int(k): float(np.percentile(v, 50)) for k, v in sorted(by_L.items())}}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--seconds", type=float, default=60.0)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--mixed", action="store_true")
    ap.add_argument("--lanczos-batch", action="store_true")
    a = ap.parse_args(argv)
    trace = workloads.hubbard_request_trace(rate=a.rate, duration=a.seconds, seed=1)
    p = L.default_params(seed=11, mixed=2 if a.mixed else 0)
    serve(trace[:16], p, a.workers, lanczos_batch=a.lanczos_batch)   # warm-up
    res, max_queue = serve(trace, p, a.workers, lanczos_batch=a.lanczos_batch)
    out = summarize(trace, res)
    out.update({"offered_rate": a.rate, "seconds": a.seconds, "workers": a.workers, "max_queue": max_queue,
                "lanczos_batch": a.lanczos_batch,
                "form": "mixed" if a.mixed else "fp64"})
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
