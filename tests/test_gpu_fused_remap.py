"""The MUSL gather and re-map in one pass (k_g2p1_remap_row) against the two
separate kernels it replaces (k_g2p1, then k_p2g_row<.., P2G_VEL>;
KMPM_SPLIT_MUSL=1 selects them).  The fused kernel forms every sum in the
order of the separate kernels, so the particle and grid fields agree bit for
bit: over the Taylor bar (TLMPM, weights from x0) and the dam break (ULMPM,
re-binned every step, positions moved into the second buffer), and in 2-D
(k_p2g_row2's re-map mode against k_g2p1 and the 2-D velocity scatter) over a
tensile bar (TLMPM) and a spinning disk (ULMPM), with the cubic and the
quadratic spline."""
import os

import numpy as np
import pytest

from karamelo_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FIELDS = ("x", "v", "sigma", "F", "eps_p")


def _taylor(basis):
    sim = W.taylor_bar(None, cellsize=0.8, basis=basis)
    sim.run(1)
    W.taylor_bar_wall(sim)
    sim.run(30)
    return sim


def _dam(basis):
    sim = W.dam_break(None, cellsize=0.05, basis=basis)
    sim.run(40)
    return sim


def _tensile_2d(basis):
    sim = W.tensile_bar_2d(None, basis=basis, vend=5.0)
    sim.run(40)
    return sim


def _disk_ulmpm_2d(basis):
    sim = W.spinning_disk(None, sub="FLIP", basis=basis, omega=3.0)
    sim.run(40)
    return sim


def _run(make, basis, split):
    if split:
        os.environ["KMPM_SPLIT_MUSL"] = "1"
    try:
        sim = make(basis)
        phases = sim.backend.profile(1)
        out = {f: sim.particles(0, f) for f in FIELDS}
        out["grid_v"] = sim.backend.grid(0, "v")
        out["grid_mass"] = sim.backend.grid(0, "mass")
        sim.backend.close()
    finally:
        os.environ.pop("KMPM_SPLIT_MUSL", None)
    return phases, out


@pytest.mark.parametrize("make", [_taylor, _dam, _tensile_2d, _disk_ulmpm_2d],
                         ids=["taylor_tlmpm", "dam_ulmpm", "tensile_tlmpm_2d", "disk_ulmpm_2d"])
@pytest.mark.parametrize("basis", ["cubic-spline", "quadratic-spline"])
def test_fused_remap_matches_separate_kernels(gpu_lib, make, basis):
    ph_f, fused = _run(make, basis, split=False)
    ph_s, split = _run(make, basis, split=True)
    # the fused kernel ran in one, the two kernels in the other
    assert "g2p_advance_remap" in ph_f and "g2p_advance" not in ph_f and "p2g_velocity" not in ph_f
    assert "g2p_advance" in ph_s and "p2g_velocity" in ph_s and "g2p_advance_remap" not in ph_s
    for k in fused:
        assert np.array_equal(fused[k], split[k]), f"{k}: max |diff| {np.max(np.abs(fused[k] - split[k])):.3e}"
