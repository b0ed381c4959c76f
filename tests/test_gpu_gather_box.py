"""3-D TLMPM: the stress kernel's node box per 256-particle block, computed
once at setup from x0 (k_gather_box), against the box each launch computes
from the same particles (KMPM_BOX_PER_LAUNCH=1): the staged gathers read the
same nodes in the same order, so every field agrees bit for bit.  The Taylor
bar (cubic and quadratic splines) and two spheres in Hertz contact (two
solids, each its own block range and grid).  2-D runs compute the box in
every launch either way."""
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
    return [{f: sim.particles(0, f) for f in FIELDS}], sim.backend


def _spheres(basis):
    sim = W.hertz_spheres(None, basis=basis)
    sim.run(60)
    return [{f: sim.particles(i, f) for f in FIELDS} for i in range(2)], sim.backend


def _run(make, basis, box):
    if not box:
        os.environ["KMPM_BOX_PER_LAUNCH"] = "1"
    try:
        out, be = make(basis)
        be.close()
    finally:
        os.environ.pop("KMPM_BOX_PER_LAUNCH", None)
    return out


@pytest.mark.parametrize("make,basis", [(_taylor, "cubic-spline"), (_taylor, "quadratic-spline"),
                                        (_spheres, "cubic-spline")],
                         ids=["taylor_cubic", "taylor_quadratic", "hertz_spheres"])
def test_setup_box_matches_per_launch_box(gpu_lib, make, basis):
    a = _run(make, basis, box=True)
    b = _run(make, basis, box=False)
    for i, (ra, rb) in enumerate(zip(a, b)):
        for f in FIELDS:
            assert np.array_equal(ra[f], rb[f]), f"instance {i} {f}: max |diff| {np.max(np.abs(ra[f] - rb[f])):.3e}"
