"""Superblocks of the reference's own DMRG runs, as fixtures.

Builds the reference's DMRG programs main/dmrg/{xxz_vf,klm_vf,hubbard_vf} from their sources
(`make -C oracle dmrg-dump`, main.c replaced by oracle/ref_dmrg_dump.c, which sets the
parameters below and records what each superblock solve was given and returned), runs them in a
scratch directory and stores, for the largest superblock of every finite sweep:

* the superblock's term list exactly as the model's MAKE_ELEMENT_HAM_LLLRRRRL applies it
  (positions, operators, coefficient, fermion-sign rule), its block and site operators, electron
  numbers and states (LL, LR, RR, RL) -- the inputs of the GPU superblock build;
* dg64 checksums of the reference's lower-triangle CRS (Row, Col, Val) -- the bitwise target;
* the reference's gs_val / gs_error and ground-state vector (DMRG_DIAGONALIZE_SUPERBLOCK_SYM:
  LANCZOS[_SLOW]_SYM + INVERSE_ITERATION_SYM);

and, per run, every superblock solve (sweep, sites, dimension, stored elements, energy) and the
lines of the run's own result files: result/log.txt (PRINT_STATUS), result/SystemInfo/
Energy_<sweep>.txt and result/[...]/AverageValues/energy.txt.

Configurations (the workloads of the benchmark):
  xxz_vf      spin-1/2 XXZ chain, OBC, L=32, Jxy=Jz=1, hz=0, 2Sz=0, m=64, 4 sweeps, Lanczos_Slow
  klm_vf      Kondo lattice, OBC, L=24, spin-1/2 moments (d=8), t=1 (coefficient -1), J=1, h_z=0.1,
              N_e=12, 2Sz=0, m=128, 4 sweeps, Lanczos
  hubbard_vf  Hubbard, OBC, L=64, t=1 (coefficient -1), U=4, N_e=64, 2Sz=0, m=512, 4 sweeps, Lanczos

    python tests/golden/make_dmrg_superblocks.py [--models xxz_vf,klm_vf] [--from-dir DIR]

Needs the reference source tree (env DMRG_REF, default /root/reference) and about 30 minutes on
8 cores for hubbard_vf.  --from-dir converts the output of an earlier run (DIR/<model>/out).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
MODELS = ("xxz_vf", "klm_vf", "hubbard_vf")
# the MODEL_* fields oracle/ref_dmrg_dump.c sets (and the drivers print in energy.txt)
MODEL_PARAMS = {
    "xxz_vf": dict(tot_site=32, spin=1, tot_sz=0, J_xy=1.0, J_z=1.0, D_z=0.0, h_z=0.0, m=64),
    "klm_vf": dict(tot_site=24, tot_ele=12, spin_loc=1, tot_sz=0, t=-1.0, J=1.0, D_z=0.0, I_xy=0.0, I_z=0.0, h_z=0.1, mu=0.0,
                   m=128),
    "hubbard_vf": dict(tot_site=64, tot_ele=64, tot_sz=0, t1=-1.0, t2=0.0, U=4.0, V=0.0, h_z=0.0, mu=0.0, m=512),
}
# ground-state vectors above this many states are stored in float32 (the overlap test is
# insensitive to it: rounding each component by 6e-8 moves the overlap by ~1e-15)
F64_VECTOR_MAX = 100_000


def read_meta(path: Path) -> dict:
    out = {}
    for line in path.read_text().splitlines():
        k, v = line.split(None, 1)
        if k in ("model",):
            out[k] = v
        elif k.endswith("_dg64"):
            out[k] = np.uint64(int(v, 16))
        elif k in ("gs_val", "gs_error"):
            out[k] = float.fromhex(v)
        else:
            out[k] = int(v)
    return out


def read_crs(path: Path):
    raw = path.read_bytes()
    n, nnz = np.frombuffer(raw[:16], np.int64)
    o = 16
    row = np.frombuffer(raw[o:o + 8 * (n + 1)], np.int64)
    o += 8 * (n + 1)
    col = np.frombuffer(raw[o:o + 4 * nnz], np.int32)
    o += 4 * nnz
    val = np.frombuffer(raw[o:o + 8 * nnz], np.float64)
    return row, col, val


def convert_sweep(d: Path) -> dict:
    meta = read_meta(d / "meta.txt")
    n = meta["n"]
    out = {k: np.asarray(v) for k, v in meta.items() if k != "model"}
    out["model"] = np.asarray(meta["model"])
    terms = [line.split() for line in (d / "terms.txt").read_text().splitlines()]
    out["term_int"] = np.array([[int(t[0]), int(t[1]), int(t[2]), int(t[3]), int(t[5]), int(t[6])] for t in terms],
                               np.int32)
    out["term_coef"] = np.array([float.fromhex(t[4]) for t in terms])
    k = 0
    while (d / f"op{k}.bin").exists():
        out[f"op{k}_row"], out[f"op{k}_col"], out[f"op{k}_val"] = read_crs(d / f"op{k}.bin")
        k += 1
    out["n_ops"] = np.int32(k)
    for p in range(4):
        if (d / f"ele{p}.bin").exists():
            out[f"ele{p}"] = np.fromfile(d / f"ele{p}.bin", np.int32)
    out["states"] = np.fromfile(d / "states.bin", np.int16).reshape(4, n)
    gs = np.fromfile(d / "gs.bin", np.float64)
    out["gs_vec"] = gs if n <= F64_VECTOR_MAX else gs.astype(np.float32)
    return out


def convert_run(model: str, run_dir: Path) -> list[Path]:
    out_dir = run_dir / "out"
    written = []
    steps = []
    for line in (out_dir / "steps.txt").read_text().splitlines():
        f = line.split()
        steps.append([int(x) for x in f[:5]] + [float.fromhex(f[5]), float.fromhex(f[6])])
    st = np.array(steps, dtype=object)
    energy_lines = []
    res = run_dir / "result"
    if res.exists():
        for p in sorted(res.glob("*/AverageValues/energy.txt")):
            for line in p.read_text().splitlines():
                energy_lines.append(f"{p.parent.parent.name}\t{line}")
    log_lines = (res / "log.txt").read_text().splitlines() if (res / "log.txt").exists() else []
    sweep_lines = []
    for p in sorted((res / "SystemInfo").glob("Energy_*.txt")) if res.exists() else []:
        k = int(p.stem.split("_")[1])
        sweep_lines += [f"{k}\t{line}" for line in p.read_text().splitlines()]
    summary = dict(sweep=st[:, 0].astype(np.int32), LL_site=st[:, 1].astype(np.int32), RR_site=st[:, 2].astype(np.int32),
                   n=st[:, 3].astype(np.int64), nnz=st[:, 4].astype(np.int64), gs_val=st[:, 5].astype(np.float64),
                   gs_error=st[:, 6].astype(np.float64), energy_txt=np.array(energy_lines), log_txt=np.array(log_lines),
                   energy_sweep_txt=np.array(sweep_lines), model_params=np.array(json.dumps(MODEL_PARAMS[model])))
    p = HERE / f"dmrg_{model}_steps.npz"
    np.savez_compressed(p, **summary)
    written.append(p)
    for sd in sorted(out_dir.glob("sweep*")):
        p = HERE / f"dmrg_{model}_{sd.name}.npz"
        np.savez_compressed(p, **convert_sweep(sd))
        written.append(p)
    return written


def run_model(model: str, work: Path, ref: str) -> Path:
    exe = ROOT / "oracle" / "_ref" / f"dmrg_{model}_dump"
    d = work / model
    d.mkdir(parents=True, exist_ok=True)
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1")
    with open(d / "run.log", "wb") as log:
        subprocess.run([str(exe), str(d / "out")], cwd=d, env=env, stdout=log, stderr=subprocess.STDOUT, check=True)
    return d


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--models", default=",".join(MODELS))
    ap.add_argument("--from-dir", default=None, help="convert DIR/<model>/out of an earlier run")
    args = ap.parse_args()
    models = [m for m in args.models.split(",") if m]
    ref = os.environ.get("DMRG_REF", "/root/reference")
    if args.from_dir is None:
        if not Path(ref, "main", "dmrg").exists():
            raise SystemExit("reference sources not found (set DMRG_REF)")
        subprocess.run(["make", "-C", str(ROOT / "oracle"), f"REF={ref}", "dmrg-dump", "-j8"], check=True,
                       stdout=subprocess.DEVNULL)
        work = Path(tempfile.mkdtemp(prefix="dmrg_dump_"))
    else:
        work = Path(args.from_dir)
    for m in models:
        d = work / m if args.from_dir else run_model(m, work, ref)
        for p in convert_run(m, d):
            print(p.name, p.stat().st_size)


if __name__ == "__main__":
    sys.exit(main())
