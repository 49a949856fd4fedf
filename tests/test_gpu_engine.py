"""Concurrent engine (batched / served forms): every result equals the same job run alone,
admission respects the memory budget, and energies match the FP64 oracle."""
import numpy as np
import pytest

from dmrg_c_gb300 import ed_models, workloads

TOL_E = 1e-10


def _run(gpu, models, params, workers, budget=0, lanczos_batch=False):
    eng = gpu.Engine(workers=workers, hbm_budget=budget, lanczos_batch=lanczos_batch)
    for i, m in enumerate(models):
        eng.submit(m, params, i)
    res = {}
    while len(res) < len(models):
        for r, _ in eng.poll(64, wait_ms=100):
            res[r.id] = r
    eng.close()
    return res


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [0, 1])
def test_results_same_alone_and_in_the_mix(gpu, mixed):
    trace = workloads.hubbard_request_trace(rate=200.0, duration=0.2, seed=1)
    probe = [ed_models.hubbard_chain(8, U=3.1, hz=0.2), ed_models.hubbard_chain(10, U=6.4, hz=0.05)]
    p = gpu.default_params(seed=3, mixed=mixed)
    alone = _run(gpu, probe, p, workers=1)
    mix = _run(gpu, probe + [req["model"]() for req in trace], p, workers=8)
    for i in range(len(probe)):
        a, b = alone[i].eig_val, mix[i].eig_val
        assert alone[i].status == 0 and mix[i].status == 0
        assert abs(a - b) <= TOL_E * abs(a), (a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [0, 2])
def test_lanczos_batch_same_alone_and_in_the_mix(gpu, mixed):
    """Continuous batching: jobs admitted while others iterate join the lock-step Lanczos; each
    result equals the same job run alone (also through the lock-step batch) and the plain engine."""
    trace = workloads.hubbard_request_trace(rate=200.0, duration=0.2, seed=1)
    probe = [ed_models.hubbard_chain(8, U=3.1, hz=0.2), ed_models.hubbard_chain(10, U=6.4, hz=0.05)]
    p = gpu.default_params(seed=3, mixed=mixed)
    alone = _run(gpu, probe, p, workers=1, lanczos_batch=True)
    plain = _run(gpu, probe, p, workers=1)
    mix = _run(gpu, probe + [req["model"]() for req in trace], p, workers=8, lanczos_batch=True)
    assert all(r.status == 0 and r.converged for r in mix.values())
    for i in range(len(probe)):
        a, b, c = alone[i].eig_val, mix[i].eig_val, plain[i].eig_val
        assert abs(a - b) <= TOL_E * abs(a), (a, b)
        assert abs(a - c) <= TOL_E * abs(c), (a, c)


@pytest.mark.gpu
def test_lanczos_batch_energies_match_oracle(gpu, oracle):
    inst = [m for m in workloads.xxz_ed_batch(40, seed=0) if m["L"] in (14, 16)][:8]
    models = [m["model"]() for m in inst]
    res = _run(gpu, models, gpu.default_params(seed=9), workers=4, lanczos_batch=True)
    from dmrg_c_gb300 import abi
    for i, m in enumerate(models):
        basis, row, col, val = oracle.ed_build(m)
        rc, out, v = oracle.lanczos(abi.Crs(row, col, val, n=len(basis)), False, seed=9)
        assert res[i].status == 0
        assert abs(res[i].eig_val - out.eig_val) <= TOL_E * abs(out.eig_val)


@pytest.mark.gpu
def test_engine_energies_match_oracle(gpu, oracle):
    inst = [m for m in workloads.xxz_ed_batch(24, seed=0) if m["L"] <= 16][:6]
    models = [m["model"]() for m in inst]
    p = gpu.default_params(seed=9)
    res = _run(gpu, models, p, workers=4)
    for i, m in enumerate(models):
        basis, row, col, val = oracle.ed_build(m)
        from dmrg_c_gb300 import abi
        crs = abi.Crs(row, col, val, n=len(basis))
        rc, out, v = oracle.lanczos(crs, False, seed=9)
        assert abs(res[i].eig_val - out.eig_val) <= TOL_E * abs(out.eig_val)


@pytest.mark.gpu
def test_engine_budget_serialises_large_jobs(gpu):
    """A budget below two jobs' estimate keeps them from running together; both still finish."""
    models = [ed_models.xxz_chain(16, Jz=0.5), ed_models.xxz_chain(16, Jz=1.5)]
    p = gpu.default_params(seed=1)
    res = _run(gpu, models, p, workers=4, budget=1)
    r0, r1 = res[0], res[1]
    assert r0.status == 0 and r1.status == 0
    assert r1.t_start_ms >= r0.t_done_ms or r0.t_start_ms >= r1.t_done_ms


@pytest.mark.gpu
def test_engine_refuses_bad_jobs_at_submission(gpu):
    eng = gpu.Engine(workers=2)
    with pytest.raises(gpu.DgError):
        eng.submit(ed_models.xxz_chain(6, twoSz=1), gpu.default_params(), 0)     # empty sector
    bad = ed_models.xxz_chain(6)
    bad.struct.terms[0].op1 = 99
    with pytest.raises(gpu.DgError):
        eng.submit(bad, gpu.default_params(), 1)
    assert eng.pending()[:2] == (0, 0)
    eng.close()
