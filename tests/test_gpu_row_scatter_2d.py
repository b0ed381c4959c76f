"""The 2-D row scatter (k_p2g_row2: four lane groups per warp, rows of four
cells) against the FP64 oracle, beside the per-cell scatter it replaces for
the plain 2-D modes (k_p2g; KMPM_CELL_SCATTER=1 selects it).  Both sum the
same particles in a fixed order but group them differently, so they part at
FP32 rounding, which the collisions of these runs amplify; each is held to
the oracle and is bit-reproducible from run to run.  Covered: TLMPM forces
and the MUSL re-map (the tensile bar of the batched sweep), ULMPM forces
with the mass (two disks, cubic, USL) and the quadratic spline."""
import os

import numpy as np
import pytest

from karamelo_gb300 import workloads as W

pytestmark = pytest.mark.gpu

CASES = {
    "tensile_tl_musl": (lambda f, m: W.tensile_bar_2d(f, cellsize=0.4, vend=20.0, ramp=False, method=m), "tlmpm",
                        300, {"x": 1e-6, "v": 1e-3, "sigma": 1e-3}),
    "disks_ul_usl": (lambda f, m: W.two_disks(f, basis="cubic-spline", scheme="usl", method=m), "ulmpm",
                     300, {"x": 1e-5, "v": 1e-3, "sigma": 1e-2}),
    "disk_ul_musl_quadratic": (lambda f, m: W.spinning_disk(f, sub="FLIP", basis="quadratic-spline", omega=5.0,
                                                            method=m), "ulmpm", 200,
                               {"x": 1e-6, "v": 1e-4, "sigma": 1e-3}),
}


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _gpu(name, cell):
    make, method, steps, tol = CASES[name]
    if cell:
        os.environ["KMPM_CELL_SCATTER"] = "1"
    try:
        sim = make(None, method + "/gpu")
        sim.run(steps)
        out = {f: sim.particles(0, f) for f in tol}
        sim.backend.close()
    finally:
        os.environ.pop("KMPM_CELL_SCATTER", None)
    return out


@pytest.mark.parametrize("name", list(CASES))
def test_row_scatter_2d_against_oracle(gpu_lib, oracle_mod, name):
    make, method, steps, tol = CASES[name]
    o = make(oracle_mod.OracleBackend, method)
    o.run(steps)
    ref = {f: o.particles(0, f) for f in tol}
    row, row2, cell = _gpu(name, False), _gpu(name, False), _gpu(name, True)
    print(f"\n{name}: " + ", ".join(f"{f} row {_rel(row[f], ref[f]):.2e} cell {_rel(cell[f], ref[f]):.2e}"
                                    for f in tol))
    for f, t in tol.items():
        assert np.array_equal(row[f], row2[f]), f"{f}: two runs differ"
        assert _rel(row[f], ref[f]) < t, f"{f}: rel L2 {_rel(row[f], ref[f]):.3e} >= {t}"
