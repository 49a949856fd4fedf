"""Sliced-ELL shapes tuned per size class (dg_shape_cache_apply) and the engine that uses them.

The first matrix of a class is timed over every sliced-ELL configuration of both products and
the fastest is recorded; later matrices of the class take it without timing.  A shape changes
only the summation order, so solves with tuned shapes agree with the heuristic's to rounding."""
import numpy as np
import pytest

from dmrg_c_gb300 import ed_models, workloads

pytestmark = pytest.mark.gpu

TOL_E = 1e-11


def _matrix(gpu, model, mixed):
    ed = gpu.EDSystem(model)
    m = ed.matrix(gpu.DG_VALUES_BOTH if mixed else gpu.DG_VALUES_F64)
    ed.close()
    return m


def test_tuned_shape_is_recorded_and_reused(gpu):
    gpu.shape_cache_clear()
    assert gpu.shape_cache_size() == 0
    a = _matrix(gpu, ed_models.xxz_chain(16, Jz=0.7, hz=0.3), True)
    assert a.shape_cache_apply(tune=True, iters=2) == 2
    assert gpu.shape_cache_size() == 1
    tuned = a.sell_config()
    b = _matrix(gpu, ed_models.xxz_chain(16, Jz=1.6, hz=0.1), True)      # same size class
    heuristic = b.sell_config()
    assert b.shape_cache_apply(tune=False) == 1
    assert b.sell_config() == tuned
    c = _matrix(gpu, ed_models.xxz_chain(14, Jz=0.7, hz=0.3), True)      # another class, not tuned
    before = c.sell_config()
    assert c.shape_cache_apply(tune=False) == 0 and c.sell_config() == before
    # the tuned shape solves to the heuristic's energy (FP64 and mixed form)
    for mixed in (0, 2):
        p = gpu.default_params(seed=5, mixed=mixed)
        ref = _matrix(gpu, ed_models.xxz_chain(16, Jz=1.6, hz=0.1), True)
        assert ref.sell_config() == heuristic
        _, e_ref = gpu.ground_state(ref, p)
        _, e_tuned = gpu.ground_state(b, p)
        assert e_ref.converged and e_tuned.converged
        assert abs(e_ref.eig_val - e_tuned.eig_val) <= TOL_E * abs(e_ref.eig_val)
    gpu.shape_cache_clear()
    assert gpu.shape_cache_size() == 0


def _run(gpu, models, params, tune):
    eng = gpu.Engine(workers=4, lanczos_batch=True, tune_shapes=tune)
    for i, m in enumerate(models):
        eng.submit(m, params, i)
    res = {}
    while len(res) < len(models):
        for r, _ in eng.poll(64, wait_ms=100):
            res[r.id] = r
    eng.close()
    return res


@pytest.mark.parametrize("mixed", [0, 2])
def test_engine_with_tuned_shapes(gpu, mixed):
    """The engine tunes each size class on its first job and solves every job to the energy of
    the untuned engine."""
    gpu.shape_cache_clear()
    inst = [m for m in workloads.xxz_ed_batch(60, seed=2) if m["L"] in (12, 14, 16)][:16]
    models = [m["model"]() for m in inst]
    p = gpu.default_params(seed=9, mixed=mixed)
    plain = _run(gpu, models, p, tune=False)
    assert gpu.shape_cache_size() == 0
    tuned = _run(gpu, models, p, tune=True)
    assert gpu.shape_cache_size() >= 2          # L = 14 and 16 at least (L = 12 may take the dense route)
    for i in range(len(models)):
        a, b = plain[i], tuned[i]
        assert a.status == 0 and b.status == 0 and a.converged and b.converged
        assert abs(a.eig_val - b.eig_val) <= TOL_E * abs(a.eig_val), (i, a.eig_val, b.eig_val)
    gpu.shape_cache_clear()
