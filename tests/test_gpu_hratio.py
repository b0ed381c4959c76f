"""The h ratio of the TLMPM time step (src/solid.cpp:1399-1409): the smallest
min(1, |Re lambda(F)|) over each solid's particles.

The stress kernel solves the characteristic cubic of F only for particles
whose Gershgorin lower bound (on the spectrum of sym F, which holds every
real part) lies below a per-range bound, 1.001 times the last step's minimum;
the others report the bound.  When a range's reduced minimum reaches its
bound, k_h_exact recomputes the range from every particle.  The result is
the exact minimum whatever the bound, so runs are bit-identical to those
that solve the cubic for every particle (KMPM_EXACT_H=1): checked here over
the Taylor bar's impact and across an upload of F = I that raises every
minimum above its bound (the exact pass must run).  Independent instances
(batches of bars, each its own clock) solve every particle's cubic, as the
last test checks against the same switch."""
import os

import numpy as np
import pytest

from karamelo_gb300 import batch as B
from karamelo_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FIELDS = ("x", "v", "sigma", "F", "eps_p")


def _taylor(exact):
    if exact:
        os.environ["KMPM_EXACT_H"] = "1"
    try:
        sim = W.taylor_bar(None, cellsize=0.8)
        sim.run(1)
        W.taylor_bar_wall(sim)
        clocks = []
        for _ in range(3):
            sim.run(10)
            clocks.append(sim.backend.scalars())
        n = sim.s.solids[0].np
        sim.backend.upload(0, "F", np.tile(np.eye(3).ravel(), n))
        for _ in range(2):
            sim.run(3)
            clocks.append(sim.backend.scalars())
        out = {f: sim.particles(0, f) for f in FIELDS}
        sim.backend.close()
    finally:
        os.environ.pop("KMPM_EXACT_H", None)
    return clocks, out


def test_bounded_h_ratio_matches_exact(gpu_lib):
    ca, a = _taylor(False)
    cb, b = _taylor(True)
    assert ca == cb
    # the upload raised the minimum to 1: dt grows, and the bounded run found it
    assert ca[-1][1] > ca[2][1]
    for f in FIELDS:
        assert np.array_equal(a[f], b[f]), f


def _batch(exact):
    if exact:
        os.environ["KMPM_EXACT_H"] = "1"
    try:
        sims, _ = B.tensile_sweep(6, seed=3, nmin=400, nmax=3000, vmin=20.0, vmax=60.0)
        bt = B.Batch(sims)
        bt.run(40)
        out = [bt.scalars(i) for i in range(6)], [bt.particles(i, "x") for i in range(6)]
        bt.backend.close()
    finally:
        os.environ.pop("KMPM_EXACT_H", None)
    return out


def test_bounded_h_ratio_batch(gpu_lib):
    (ca, xa), (cb, xb) = _batch(False), _batch(True)
    assert ca == cb
    for a, b in zip(xa, xb):
        assert np.array_equal(a, b)
