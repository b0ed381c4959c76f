"""The FP64 islands against the FP64 oracle, result by result.

KMPM_PREC_FP64_ISLANDS keeps three computations in FP64 on the GPU: the nodal
sums and v = p/m, det and inverse of F, and the EOS + Johnson-Cook return.
On the Taylor bar (3-D TLMPM MUSL cubic, Johnson-Cook + linear EOS, cellsize
0.8 mm, 50 steps after the wall) this test measures, in FP32 and with the
islands, the relative L2 error against the oracle of the result each island
produces:
  - v = p/m: the grid velocities, over every node with mass and over the
    near-empty nodes (mass below 1 % of the largest nodal mass);
  - det and inverse of F: F and J = det F;
  - the return: the stress σ and the plastic strain ε_p;
and the positions.  Both modes are held to the parity test's bounds; the
measured errors are printed (pytest -s)."""
import numpy as np
import pytest

from karamelo_gb300 import workloads as W
from karamelo_gb300.gpu import GpuBackend

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _run(factory, precision=None):
    sim = W.taylor_bar(factory, cellsize=0.8, method="tlmpm" if factory else "tlmpm/gpu")
    if precision is not None:
        sim.backend = GpuBackend(sim.s, precision=precision)
    sim.run(1)
    W.taylor_bar_wall(sim)
    sim.run(50)
    be = sim._ensure_backend() if factory else sim.backend
    out = {f: sim.particles(0, f) for f in ("x", "sigma", "F", "eps_p")}
    out["J"] = np.linalg.det(out["F"].reshape(-1, 3, 3))
    out["grid_v"] = be.grid(0, "v").reshape(-1, 3)
    out["grid_mass"] = be.grid(0, "mass").reshape(-1)
    return out


def test_fp64_islands_error_by_result(gpu_lib, oracle_mod):
    o = _run(oracle_mod.OracleBackend)
    m = o["grid_mass"]
    has = m > 0
    sparse = has & (m < 0.01 * m.max())
    assert sparse.sum() > 0
    table = {}
    for name, prec in (("fp32", 0), ("islands", 1)):
        g = _run(None, prec)
        table[name] = {
            "grid v (all nodes with mass)": _rel(g["grid_v"][has], o["grid_v"][has]),
            "grid v (near-empty nodes)": _rel(g["grid_v"][sparse], o["grid_v"][sparse]),
            "F": _rel(g["F"], o["F"]),
            "J": _rel(g["J"], o["J"]),
            "sigma": _rel(g["sigma"], o["sigma"]),
            "eps_p": _rel(g["eps_p"], o["eps_p"]),
            "x": _rel(g["x"], o["x"]),
        }
    for k in table["fp32"]:
        print(f"{k:30s} fp32 {table['fp32'][k]:.2e}   islands {table['islands'][k]:.2e}")
    bounds = {"x": 1e-6, "F": 1e-6, "J": 1e-6, "sigma": 1e-4, "eps_p": 1e-4,
              "grid v (all nodes with mass)": 1e-4, "grid v (near-empty nodes)": 1e-3}
    for mode in table:
        for k, b in bounds.items():
            assert table[mode][k] < b, (mode, k, table[mode][k])
