"""Axisymmetric set-up on the host and in the oracle (CPU): the populate
scaling of masses and volumes by x0_r (Solid::populate,
src/solid.cpp:2292-2295), the 2-D / mechanical restriction, and a short
oracle run."""
import numpy as np
import pytest

from karamelo_gb300 import MPM, workloads as W
from karamelo_gb300.model import KarameloError


def test_populate_scaling(oracle_mod):
    sim = W.taylor_bar_axisymmetric(oracle_mod.OracleBackend, method="tlmpm", cellsize=0.8)
    s = sim.s.solids[0]
    rho = W.COPPER["rho"]
    # mass per radian of the bar: rho R^2 L / 2
    assert abs(s.mass.sum() / (rho * 3.2 ** 2 * 32.4 / 2) - 1) < 1e-12
    np.testing.assert_allclose(s.mass, rho * (0.8 ** 2 / 4) * s.x0[:, 0], rtol=1e-13)
    np.testing.assert_allclose(s.vol0, s.mass / rho, rtol=0)
    assert sim.s.axisymmetric and np.all(s.x0[:, 0] > 0)


def test_only_2d_mechanical(oracle_mod):
    sim = MPM(oracle_mod.OracleBackend)
    sim.method("tlmpm", "FLIP", "cubic-spline", 0.99)
    sim.dimension(3, 0, 1, 0, 1, 0, 1, 0.1)
    with pytest.raises(KarameloError):
        sim.axisymmetric("true")
    sim = MPM(oracle_mod.OracleBackend)
    sim.method("tlmpm", "FLIP", "cubic-spline", 0.99, "thermo-mechanical")
    sim.dimension(2, 0, 1, 0, 1, 0.1)
    with pytest.raises(KarameloError):
        sim.axisymmetric("true")


def test_oracle_run_hoop_stress(oracle_mod):
    """A short run: the bar hits the wall, spreads radially, and carries a
    hoop stress sigma_theta-theta (stored as sigma_zz)."""
    sim = W.taylor_bar_axisymmetric(oracle_mod.OracleBackend, method="tlmpm", cellsize=0.8)
    sim.run(1)
    W.taylor_bar_axisymmetric_wall(sim)
    sim.run(300)
    x, sg = sim.particles(0, "x"), sim.particles(0, "sigma")
    assert x[:, 0].max() > 3.2 + 0.1        # the impact end has spread
    assert np.abs(sg[:, 2, 2]).max() > 0.01  # GPa
    assert np.all(x[:, 0] > 0)
