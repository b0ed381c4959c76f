"""kmpm_run_async / kmpm_sync: steps queued without waiting give the bits of
kmpm_run, downloads queued between them see the state of their step, and a
step's error is reported by the next kmpm_sync (GPU)."""
import numpy as np
import pytest

from karamelo_gb300 import workloads as W
from karamelo_gb300.gpu import GpuBackend, KmpmError

pytestmark = pytest.mark.gpu


def _bar():
    sim = W.taylor_bar(None, cellsize=0.8)
    sim.backend = GpuBackend(sim.s, track_strain=False)
    sim.run(1)
    W.taylor_bar_wall(sim)
    return sim


def _state(be):
    return {f: be.particles(0, f) for f in ("x", "v", "sigma", "eps_p")}, be.scalars()


def test_run_async_matches_run(gpu_lib):
    a, b = _bar(), _bar()
    for _ in range(3):
        a.backend.run(7)
    for _ in range(3):
        b.backend.run_async(7)
    b.backend.sync()
    sa, ta = _state(a.backend)
    sb, tb = _state(b.backend)
    assert ta == tb
    for f in sa:
        assert np.array_equal(sa[f], sb[f]), f


def test_async_downloads_between_queued_runs(gpu_lib):
    """A download queued after run_async(k) holds the state after those k
    steps, although more steps are queued before anything is waited for."""
    import torch
    a, b = _bar(), _bar()
    n = a.s.solids[0].np
    outs = [torch.empty(n * 3, dtype=torch.float64, pin_memory=True) for _ in range(3)]
    want = []
    for k in range(3):
        a.backend.run(5)
        want.append(a.backend.particles(0, "x"))
        b.backend.run_async(5)
        b.backend.particles_async(0, "x", outs[k])
    b.backend.run_async(5)
    b.backend.sync()
    b.backend.sync_downloads()
    for k in range(3):
        assert np.array_equal(outs[k].numpy().reshape(n, 3), want[k]), k


def test_run_async_error_reported_by_sync(gpu_lib):
    """The particle that leaves the domain (src/solid.cpp:617-627) raises no
    error while the steps are queued; kmpm_sync reports it."""
    from karamelo_gb300 import MPM
    sim = MPM()
    sim.method("ulmpm/gpu", "FLIP", "linear", 0.99)
    sim.dimension(2, 0, 1, 0, 1, 0.05)
    sim.region("b", "cylinder", 0.7, 0.5, 0.1)
    sim.material("m", "linear", 1000, 1000, 0.3)
    sim.solid("s", "region", "b", 2, "m", 0.05, 0)
    sim.group("g", "particles", "region", "b", "solid", "s")
    sim.fix("v0", "initial_velocity_particles", "g", 10.0, 0.0, None)
    sim.set_dt(1e-3)
    sim.run(1)
    be = sim.backend
    be.run_async(59)
    with pytest.raises(KmpmError) as e:
        be.sync()
    assert e.value.code == -11
