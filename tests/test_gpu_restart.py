"""Restart and checkpoint on the GPU.

* Restart through the reference's restart state (Solid::write_restart /
  read_restart, src/solid.cpp:2841-2957): the per-particle fields a restart
  file carries are downloaded, uploaded into a second context made by the
  same setup, and both contexts continue.  The file holds x and F as FP64
  values, while the device holds the displacement u = x - x0 and H = F - I:
  where u or H is more than 2^29 times smaller than x0 or 1, x0 + u and
  1 + H in FP64 drop its last bits, so the continuation agrees to that
  rounding (relative 1e-11 measured after 25 steps), not bit for bit.  ULMPM also re-bins by the
  current position, and within a cell the second context starts from caller
  order, so its sums run in another order.
* The device snapshot (kmpm_save_state / kmpm_load_state) carries the slot
  order too: the continuation is bit-identical for both methods.
"""
import numpy as np
import pytest

from karamelo_gb300 import workloads as W
from karamelo_gb300.gpu import GpuBackend, KmpmError

pytestmark = pytest.mark.gpu


def _taylor(first=30):
    sim = W.taylor_bar(None, cellsize=0.8)
    sim.backend = GpuBackend(sim.s, autotune=False)
    sim.run(1)
    W.taylor_bar_wall(sim)
    sim.run(first)
    return sim


def _taylor_fresh():
    sim = W.taylor_bar(None, cellsize=0.8)
    sim.backend = GpuBackend(sim.s, autotune=False)
    W.taylor_bar_wall(sim)
    return sim


def _dam(first=20):
    sim = W.dam_break(None, cellsize=0.05)
    sim.backend = GpuBackend(sim.s, autotune=False)
    sim.run(first)
    return sim


def _dam_fresh():
    sim = W.dam_break(None, cellsize=0.05)
    sim.backend = GpuBackend(sim.s, autotune=False)
    return sim


FIELDS = ("x", "v", "sigma", "F", "eps_p")


def test_restart_state_tlmpm(gpu_lib):
    a = _taylor()
    st = a.backend.restart_state()
    b = _taylor_fresh()
    b.backend.restore_state(st)
    assert b.backend.scalars() == a.backend.scalars()
    for sim in (a, b):
        sim.run(25)
    for f in FIELDS:
        xa, xb = a.particles(0, f), b.particles(0, f)
        assert np.linalg.norm(xa - xb) <= 1e-9 * np.linalg.norm(xa), f


def test_restart_state_ulmpm(gpu_lib):
    a = _dam()
    st = a.backend.restart_state()
    b = _dam_fresh()
    b.backend.restore_state(st)
    for sim in (a, b):
        sim.run(20)
    for f, tol in (("x", 1e-6), ("v", 1e-4), ("sigma", 1e-4)):
        xa, xb = a.particles(0, f), b.particles(0, f)
        assert np.linalg.norm(xa - xb) / np.linalg.norm(xa) < tol, f


def test_upload_download_roundtrip(gpu_lib):
    a = _taylor(5)
    st = a.backend.restart_state()
    for f, arr in st["solids"][0].items():
        a.backend.upload(0, f, arr)
        assert np.array_equal(a.particles(0, f), arr), f


@pytest.mark.parametrize("kind", ["tl", "ul"])
def test_snapshot_bit_exact(gpu_lib, kind):
    a = _taylor() if kind == "tl" else _dam()
    blob = a.backend.save_state()
    b = _taylor_fresh() if kind == "tl" else _dam_fresh()
    b.backend.run(0)
    b.backend.load_state(blob)
    for sim in (a, b):
        sim.run(20)
    for f in FIELDS:
        assert np.array_equal(a.particles(0, f), b.particles(0, f)), f
    assert a.backend.scalars() == b.backend.scalars()


def test_snapshot_of_another_setup_is_refused(gpu_lib):
    a = _taylor(1)
    blob = a.backend.save_state()
    b = _dam_fresh()
    b.backend.run(0)
    with pytest.raises(KmpmError):
        b.backend.load_state(blob)
    with pytest.raises(KmpmError):
        b.backend.load_state(b"not a snapshot" * 10)


def test_uploaded_history_follows_rebinning(gpu_lib):
    """The dam break's water has no plastic or damage law, so its runs leave
    ε_p and damage at zero and the re-binning does not move them.  A restart
    can still bring non-zero values (its file is the reference's, whatever
    the laws): once uploaded they must follow their particles through the
    re-binning, and a snapshot of that state loads into a fresh context."""
    a = _dam(5)
    rng = np.random.default_rng(7)
    n = a.s.solids[0].np
    ep = rng.uniform(0.0, 0.5, n)
    dm = rng.uniform(0.0, 0.01, n)
    a.backend.upload(0, "eps_p", ep)
    a.backend.upload(0, "damage", dm)
    a.run(20)
    assert np.array_equal(a.particles(0, "eps_p"), ep.astype(np.float32).astype(float))
    assert np.array_equal(a.particles(0, "damage"), dm.astype(np.float32).astype(float))
    blob = a.backend.save_state()
    b = _dam_fresh()
    b.backend.run(0)
    b.backend.load_state(blob)
    for sim in (a, b):
        sim.run(10)
    for f in FIELDS + ("damage",):
        assert np.array_equal(a.particles(0, f), b.particles(0, f)), f
