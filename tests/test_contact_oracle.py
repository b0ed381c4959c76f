"""The oracle's contact fixes (oracle/mpm_oracle.cpp contact_forces) against
closed forms written from the reference fixes, on CPU.

FixContactMinPenetration::initial_integrate
(src/fix_contact_min_penetration.cpp:83-235) and FixContactHertz::initial_integrate
(src/fix_contact_hertz.cpp:82-197) have no test or golden vector in the
reference; these checks restate their pair formula for one pair of particles
and compare it with the oracle's total force after one step (the fix runs at
the start of the step on the initial state), plus the momentum balance of a
whole collision."""
import math

import numpy as np
import pytest

from karamelo_gb300 import MPM
from karamelo_gb300 import workloads as W


def _two_particles(oracle_mod, dim, contact, mu=0.0, sep=0.9, h=0.1, v1=(0.0, 0.0, 0.0), v2=(0.0, 0.0, 0.0),
                   dt=1e-3, rho=1000.0, E=1e3, nu=0.3, gpu=False):
    """Two one-particle solids (TLMPM, one cell each) whose particles are
    sep * h apart along x (on the oracle, or on the GPU with gpu=True)."""
    sim = MPM(None if gpu else oracle_mod.OracleBackend)
    sim.method("tlmpm/gpu" if gpu else "tlmpm", "FLIP", "linear", 0.99)
    sim.scheme("musl")
    if dim == 2:
        sim.dimension(2, -1, 1, -1, 1, h)
        sim.region("r1", "block", 0.0, h, 0.0, h)
        sim.region("r2", "block", sep * h, (1 + sep) * h, 0.0, h)
    else:
        sim.dimension(3, -1, 1, -1, 1, -1, 1, h)
        sim.region("r1", "block", 0.0, h, 0.0, h, 0.0, h)
        sim.region("r2", "block", sep * h, (1 + sep) * h, 0.0, h, 0.0, h)
    sim.material("m", "linear", rho, E, nu)
    sim.solid("s1", "region", "r1", 1, "m", h, 0)
    sim.solid("s2", "region", "r2", 1, "m", h, 0)
    assert [s.np for s in sim.s.solids] == [1, 1]
    sim.s.solids[0].v[:] = v1
    sim.s.solids[1].v[:] = v2
    if contact == "contact/hertz":
        sim.fix("c", contact, "s1", "s2")
    else:
        sim.fix("c", contact, "s1", "s2", mu)
    sim.set_dt(dt)
    sim.run(1)
    s1, s2 = sim.s.solids
    return sim, s1, s2


def _expected(dim, kind, s1, s2, mu, dt, E, nu):
    x1, x2 = s1.x0[0], s2.x0[0]
    dx = x2 - x1
    vol1, vol2 = s1.vol0[0], s2.vol0[0]
    if dim == 3:
        R1 = 0.5 * (vol1 ** 0.333333333 if kind == "hertz" else np.cbrt(vol1))
        R2 = 0.5 * (vol2 ** 0.333333333 if kind == "hertz" else np.cbrt(vol2))
    else:
        R1, R2 = 0.5 * math.sqrt(vol1), 0.5 * math.sqrt(vol2)
    Rp = R1 + R2
    r = np.linalg.norm(dx)
    assert r < Rp
    Es = 1.0 / (2 * (1 - nu * nu) / E)
    if kind == "hertz":
        coef = 1.333333333 if dim == 3 else 0.25 * math.pi
        return coef * Es * math.sqrt(R1 * R2 / (R1 + R2) * (Rp - r) ** 3) * dx / r
    m1, m2 = s1.mass[0], s2.mass[0]
    fmag = m1 * m2 / ((m1 + m2) * dt * dt) * (1 - Rp / r)
    f = fmag * dx
    if mu:
        dv = s2.v[0] - s1.v[0]
        vt = dv - dv.dot(dx) / (r * r) * dx
        n = np.linalg.norm(vt)
        if n:
            f = f - mu * fmag * r * vt / n
    return f


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kind,mu", [("min", 0.0), ("min", 0.4), ("hertz", 0.0)])
def test_pair_force_closed_form(oracle_mod, dim, kind, mu):
    contact = "contact/hertz" if kind == "hertz" else "contact/minimize_penetration"
    vz = 1.0 if dim == 3 else 0.0
    sim, s1, s2 = _two_particles(oracle_mod, dim, contact, mu=mu, v1=(0.3, 0.2, -0.1 * vz),
                                 v2=(-0.1, -0.3, 0.2 * vz))
    f = sim.contact_force("c")
    exp = _expected(dim, kind, s1, s2, mu, 1e-3, 1e3, 0.3)
    assert np.linalg.norm(exp) > 0
    np.testing.assert_allclose(f, exp, rtol=1e-12, atol=1e-12 * np.linalg.norm(exp))


def test_no_force_beyond_contact_radius(oracle_mod):
    sim, s1, s2 = _two_particles(oracle_mod, 2, "contact/minimize_penetration", sep=1.01)
    assert np.all(sim.contact_force("c") == 0)


@pytest.mark.parametrize("contact,mu,offset", [("contact/minimize_penetration", 0.0, 0.0),
                                               ("contact/minimize_penetration", 0.3, 0.1),
                                               ("contact/hertz", 0.0, 0.0)])
def test_collision_momentum(oracle_mod, contact, mu, offset):
    """Through a whole collision of two balls the pair forces cancel: the total
    momentum stays zero while each ball's changes."""
    sim = W.bouncing_balls(oracle_mod.OracleBackend, method="tlmpm", centre=0.14 if offset else 0.16,
                           contact=contact, mu=mu, offset=offset)
    m = [s.mass for s in sim.s.solids]
    seen = 0.0
    for _ in range(30):
        sim.run(10)
        seen = max(seen, float(np.abs(sim.contact_force("contact")).max()))
        P = sum((mi[:, None] * sim.particles(k, "v")).sum(0) for k, mi in enumerate(m))
        assert np.abs(P).max() < 1e-11
    assert seen > 0
    v1 = (m[0][:, None] * sim.particles(0, "v")).sum(0) / m[0].sum()
    assert v1[0] < 0.1 - 1e-5  # ball 1 was slowed by the contact
