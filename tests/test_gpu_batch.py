"""Independent runs in one launch (a seeded tensile-bar sweep): every
instance of a batch must match the same script run alone on the oracle,
including its own dt and time."""
import numpy as np
import pytest

from karamelo_gb300.batch import Batch, tensile_sweep
from karamelo_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_tensile_sweep_batch_matches_single_runs(gpu_lib, oracle_mod):
    sims, params = tensile_sweep(5, seed=1, nmin=400, nmax=2500, vmin=20.0, vmax=60.0)
    batch = Batch(sims)
    batch.run(1500)
    for i, p in enumerate(params):
        o = W.tensile_bar_2d(oracle_mod.OracleBackend, method="tlmpm", ramp=False, cellsize=p["cellsize"],
                             vend=p["vend"], damage=p["damage"])
        o.run(1500)
        t, dt, n = batch.scalars(i)
        assert n == 1500
        assert abs(t / o.time - 1) < 1e-5 and abs(dt / o.dt - 1) < 1e-4
        assert o.particles(0, "eps_p").max() > 0
        for field, tol in (("x", 1e-6), ("v", 1e-3), ("sigma", 1e-3), ("eps_p", 1e-3), ("damage_init", 1e-3)):
            e = rel(batch.particles(i, field), o.particles(0, field))
            assert e < tol, f"instance {i} {field}: {e:.2e}"


def test_batch_instances_have_their_own_clocks(gpu_lib):
    sims, _ = tensile_sweep(3, seed=2, nmin=400, nmax=3000)
    batch = Batch(sims)
    batch.run(20)
    dts = [batch.scalars(i)[1] for i in range(3)]
    assert len(set(dts)) == 3  # different cell sizes give different CFL steps
