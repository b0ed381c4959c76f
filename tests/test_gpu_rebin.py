"""ULMPM re-binning on the GPU: the per-step update of the last binning
against the full stable radix sort of every key (KMPM_FULL_REBIN=1).

Both give the permutation of a stable sort of the new cell keys over the
current slot order, so runs through either must be bit for bit the same,
whether few particles change cell in a step (the dam break, the disks) or all
of them (the first step, where the update starts from every slot in cell 0,
and a restart that uploads new positions).
"""
import os

import numpy as np
import pytest

from karamelo_gb300 import workloads as W
from karamelo_gb300.gpu import GpuBackend

pytestmark = pytest.mark.gpu


def _pair(make, **kw):
    """Two simulations of one script: the first bins by update, the second
    by the full sort (the switch is read when the context is built)."""
    a = make()
    a.backend = GpuBackend(a.s, autotune=False, **kw)
    a.backend.run(0)
    os.environ["KMPM_FULL_REBIN"] = "1"
    try:
        b = make()
        b.backend = GpuBackend(b.s, autotune=False, **kw)
        b.backend.run(0)
    finally:
        del os.environ["KMPM_FULL_REBIN"]
    return a, b


def _same(a, b, fields=("x", "v", "sigma")):
    for si in range(len(a.s.solids)):
        for f in fields:
            assert np.array_equal(a.particles(si, f), b.particles(si, f)), (si, f)
    assert a.backend.scalars() == b.backend.scalars()


def test_dam_break_update_equals_full_sort(gpu_lib):
    a, b = _pair(lambda: W.dam_break(None, cellsize=0.05))
    for sim in (a, b):
        sim.run(60)
    _same(a, b)


def test_two_disks_update_equals_full_sort(gpu_lib):
    a, b = _pair(lambda: W.two_disks(None))
    for sim in (a, b):
        sim.run(2000)  # through the impact (about t = 1.5)
    _same(a, b)


def test_spinning_disk_apic_update_equals_full_sort(gpu_lib):
    a, b = _pair(lambda: W.spinning_disk(None, omega=20.0))
    for sim in (a, b):
        sim.run(100)
    _same(a, b)


def test_rebin_after_position_upload(gpu_lib):
    """Uploaded positions (a restart) move every particle at once."""
    a, b = _pair(lambda: W.dam_break(None, cellsize=0.05))
    for sim in (a, b):
        sim.run(10)
    rng = np.random.default_rng(3)
    x = a.particles(0, "x")
    x = x + rng.uniform(-0.02, 0.02, x.shape) * np.array([1.0, 1.0, 0.0])
    x = np.clip(x, 0.06, [1.5, 0.34, 0.74])
    for sim in (a, b):
        sim.backend.upload(0, "x", x)
        sim.run(20)
    _same(a, b)
