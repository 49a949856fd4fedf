"""bench.py's multi-process path (replicas only: no data-path collective) with two gloo
ranks on the CPU: the job's time is the slowest replica's, its rate sums the replicas, and
the reference arm runs on rank 0 only; and the clock record's timed-window filtering."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, port, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=2)
    ws, r, lr = bench.dist_info()
    bench.replica_barrier(ws)
    my_ms = 100.0 if rank == 0 else 150.0          # rank 1 is the slower replica
    t = bench.replica_time(my_ms, ws, device="cpu")
    out[rank] = (ws, r, t, bench.job_rate(10, ws, t))
    dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_time():
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_rank, args=(port, out), nprocs=2, join=True, start_method="spawn")
        res = dict(out)
    for rank in (0, 1):
        ws, r, t, rate = res[rank]
        assert ws == 2 and r == rank
        assert t == 150.0
        assert rate == pytest.approx(2 * 10 / 0.150)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench

    class A:
        workload = "xxz_m64"
        seed = 0
        steps = 1
        warmup = 0
    assert bench.run_reference(A(), 2, 1) is None


def test_clock_summary_keeps_the_timed_window():
    """Only nvidia-smi samples that arrived inside the timed region count; a window shorter than
    the sampling interval falls back to the nearest sample."""
    sys.path.insert(0, str(ROOT))
    import bench
    clk = bench.ClockSampler()
    line = "{sm}, 2070, 900.0, 0x0, Not Active, Not Active, {therm}, Not Active"
    clk.lines = [(0.00, line.format(sm=1500, therm="Active")),      # before the window (warm-up)
                 (1.00, line.format(sm=2070, therm="Not Active")),
                 (1.02, line.format(sm=2050, therm="Not Active")),
                 (1.04, line.format(sm=2070, therm="Not Active")),
                 (3.00, line.format(sm=1400, therm="Active"))]     # after it
    clk.window(0.99, 1.05)
    s = clk.summary()
    assert s["samples"] == 3 and s["sm_mhz"] == 2070 and s["reasons"] == []
    clk.window(2.98, 2.985)
    s = clk.summary()
    assert s["samples"] == 1 and s["sm_mhz"] == 1400 and s["reasons"] == ["sw_thermal_slowdown"]


def test_mixed_roofline_counts_the_layout_it_reads():
    """roofline_mixed's bytes: with the 16-bit delta stream in use, 2 + 4 bytes a stored slot plus
    the checkpoints, slot rows, slice words and the two vectors; without it, the CRS footprint."""
    sys.path.insert(0, str(ROOT))
    import bench

    class M:
        def __init__(self, deltas, variant32):
            self.d, self.v = deltas, variant32

        def sell_config(self):
            return dict(ws=2, grid=1872, variant=3, ws32=1, variant32=self.v)

        def sell_deltas(self):
            return (self.d, 42080 if self.d else 0)

        def format(self):
            return (1, 56362528)

        def sell_checkpoints(self):
            return 1881984 if self.d else 0

    n, nnz = 238462, 56222276
    b, basis = bench.sell_mixed_bytes(M(True, 5), n, nnz)
    nslices = -(-n // 2048) * 2048 // 32
    assert b == 56362528 * 6 + 1881984 * 4 + nslices * 32 * 4 + nslices * 20 + n * 4 + n * 8 == 349672872
    assert basis.startswith("delta layout")
    for m in (M(False, 1), M(True, 1)):          # no stream, or the FP32 product not on it
        b, basis = bench.sell_mixed_bytes(m, n, nnz)
        assert b == bench.spmv_bytes(n, nnz, 4, 4) and basis.startswith("CRS")
