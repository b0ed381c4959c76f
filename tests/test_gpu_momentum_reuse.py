"""TLMPM MUSL momentum reuse against a momentum scatter every step.

TLMPM's weights and masses never change, and no particle velocity changes
between a step's re-map (velocities_to_grid, src/musl.cpp:59-67) and the next
step's scatter (particles_to_grid): the nodal momentum that scatter would sum
is the re-map's, bit for bit.  The step's scatter sums the forces only
(k_p2g_force_row); with the reuse the velocity pass of the grid keeps the
re-map's momentum for the next grid update, and KMPM_NO_MOMENTUM_REUSE=1
runs the velocity row scatter (the re-map's sums) before it every step.
Both must give the same bits, including after an upload between steps
(which must make the next step scatter the momentum of the new state) and
across kmpm_run calls: on the 3-D Taylor bar (cubic and quadratic splines)
and on a 2-D tensile bar with Johnson-Cook damage (the 2-D row scatter)."""
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
    return sim


def _tensile(basis):
    sim = W.tensile_bar_2d(None, basis=basis, vend=5.0)
    sim.run(1)
    return sim


CASES = {"taylor_cubic": (_taylor, "cubic-spline"), "taylor_quadratic": (_taylor, "quadratic-spline"),
         "tensile_2d_cubic": (_tensile, "cubic-spline")}


def _run(case, reuse, upload):
    make, basis = CASES[case]
    if not reuse:
        os.environ["KMPM_NO_MOMENTUM_REUSE"] = "1"
    try:
        sim = make(basis)
        sim.run(12)
        if upload:
            v = sim.particles(0, "v")
            sim.backend.upload(0, "v", v * 0.97)
        for _ in range(3):  # several run calls: the reuse carries across them
            sim.run(6)
        phases = sim.backend.profile(1)
        out = {f: sim.particles(0, f) for f in FIELDS}
        out["grid_v"] = sim.backend.grid(0, "v")
        out["scalars"] = np.array(sim.backend.scalars(), float)
        sim.backend.close()
    finally:
        os.environ.pop("KMPM_NO_MOMENTUM_REUSE", None)
    return phases, out


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("upload", [False, True], ids=["steps", "upload_between"])
def test_momentum_reuse_bit_identical(gpu_lib, case, upload):
    ph_r, a = _run(case, True, upload)
    ph_f, b = _run(case, False, upload)
    # both run the force-only scatter; without the reuse a velocity scatter
    # forms the momentum first every step
    assert "p2g_force" in ph_r and "p2g_momentum" not in ph_r and "p2g" not in ph_r
    assert "p2g_force" in ph_f and "p2g_momentum" in ph_f and "p2g" not in ph_f
    for k in a:
        assert np.array_equal(a[k], b[k]), f"{k}: max |diff| {np.max(np.abs(a[k] - b[k])):.3e}"


def test_upload_changes_the_run(gpu_lib):
    """The upload case above is not vacuous: the scaled velocities change the
    state that the steps after it produce."""
    _, a = _run("taylor_cubic", True, False)
    _, b = _run("taylor_cubic", True, True)
    assert not np.array_equal(a["x"], b["x"])
