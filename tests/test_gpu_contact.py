"""GPU parity of the contact fixes (FixContactMinPenetration,
src/fix_contact_min_penetration.cpp:83-235; FixContactHertz,
src/fix_contact_hertz.cpp:82-197) against the FP64 oracle: whole collisions
through the C ABI, the state of both solids, the fixes' total force and the
momentum balance.  Tolerances are relative L2 norms over all particles.

The min-penetration force removes the overlap of a pair in one step
(f = m1 m2 / ((m1 + m2) dt^2) (1 - Rp / r) dx): a position difference of one
FP32 ulp between the GPU and the FP64 oracle becomes a velocity difference of
that ulp / dt in the contact layer, so the velocity tolerances of these runs
are looser than those of the runs without contact."""
import numpy as np
import pytest

from karamelo_gb300 import MPM
from karamelo_gb300 import workloads as W
from karamelo_gb300.gpu import GpuBackend, KmpmError

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _pair(oracle_mod, build, steps, **kw):
    g = build(None, **kw)
    kw_o = dict(kw)
    kw_o["method"] = kw.get("method", "tlmpm/gpu").replace("/gpu", "")
    o = build(oracle_mod.OracleBackend, **kw_o)
    for sim in (g, o):
        sim._ensure_backend()
    assert isinstance(g.backend, GpuBackend)
    fg, fo = [], []
    for n in steps:
        for sim in (g, o):
            sim.run(n)
        fg.append(g.contact_force("contact"))
        fo.append(o.contact_force("contact"))
    return g, o, np.array(fg), np.array(fo)


def _check(g, o, tol, nsolid=2):
    for s in range(nsolid):
        for field, t in tol.items():
            e = rel(g.particles(s, field), o.particles(s, field))
            assert e < t, f"solid {s} {field}: rel L2 {e:.3e} >= {t}"


def _momentum(sim):
    return sum((s.mass[:, None] * sim.particles(k, "v")).sum(0) for k, s in enumerate(sim.s.solids))


def _collided(o, v0=0.1):
    m = o.s.solids[0].mass
    return float((m[:, None] * o.particles(0, "v")).sum(0)[0] / m.sum()) < v0 - 1e-5


@pytest.mark.parametrize("scheme", ["musl", "usl"])
def test_bouncing_balls_min_penetration(gpu_lib, oracle_mod, scheme):
    """The reference example's two balls (TLMPM FLIP, linear basis), closer
    together so that 300 steps cover the collision."""
    g, o, fg, fo = _pair(oracle_mod, W.bouncing_balls, [100] * 3, centre=0.16, scheme=scheme)
    assert _collided(o)
    _check(g, o, {"x": 1e-6, "v": 2e-3, "sigma": 5e-3})
    assert rel(fg, fo) < 5e-3
    P = _momentum(g)
    assert np.abs(P).max() < 1e-6 * o.s.solids[0].mass.sum() * 0.1


def test_bouncing_balls_friction(gpu_lib, oracle_mod):
    """Impact with Coulomb friction (mu = 0.3).  The fix's friction has no
    stick regime: its direction vt / |vt| is undefined at vt = 0, and a pair
    whose tangential relative velocity vanishes gets its friction direction
    from rounding.  The balls here approach along (1, 0.4), which is parallel
    to none of the lattice directions of the particle pairs, so every pair
    slides."""
    g, o, fg, fo = _pair(oracle_mod, W.bouncing_balls, [100] * 4, centre=0.16, mu=0.3, vy=0.04)
    assert _collided(o)
    _check(g, o, {"x": 1e-6, "v": 1e-3, "sigma": 5e-3})
    assert rel(fg, fo) < 5e-3


def test_bouncing_balls_hertz_2d(gpu_lib, oracle_mod):
    g, o, fg, fo = _pair(oracle_mod, W.bouncing_balls, [100] * 3, centre=0.16, contact="contact/hertz", E=1e5)
    assert _collided(o)
    _check(g, o, {"x": 1e-6, "v": 1e-3, "sigma": 1e-3})
    assert rel(fg, fo) < 1e-3


@pytest.mark.parametrize("contact", ["contact/hertz", "contact/minimize_penetration"])
def test_spheres_3d(gpu_lib, oracle_mod, contact):
    """Two spheres (TLMPM, cubic spline) through the 3-D branches of both fixes."""
    g, o, fg, fo = _pair(oracle_mod, W.hertz_spheres, [40] * 3, contact=contact)
    assert _collided(o, v0=0.5)
    _check(g, o, {"x": 1e-6, "v": 2e-3, "sigma": 5e-3})
    assert rel(fg, fo) < 5e-3


def test_bouncing_balls_ulmpm(gpu_lib, oracle_mod):
    """ULMPM: both balls share one grid (the members are told apart by solid
    id in the per-step binned order).  The shared grid keeps slow balls more
    than Rp apart; at 1 m/s the particle pairs come within Rp."""
    g, o, fg, fo = _pair(oracle_mod, W.bouncing_balls, [100] * 4, centre=0.16, method="ulmpm/gpu",
                         basis="cubic-spline", v=1.0, dt=2e-4)
    assert _collided(o, v0=1.0)
    _check(g, o, {"x": 1e-6, "v": 2e-3, "sigma": 5e-3})
    assert rel(fg, fo) < 5e-3


@pytest.mark.parametrize("method", ["tlmpm/gpu", "ulmpm/gpu"])
def test_bouncing_balls_apic(gpu_lib, oracle_mod, method):
    """The reference example's APIC variant (here with the cubic spline).
    APIC transfers carry an FP32 rounding of the affine moments from step to
    step even in free flight: measured before the balls meet, the velocity
    differs from the FP64 oracle by 2.5e-7 (TLMPM) and 1e-7 (ULMPM) per step,
    which sets the tolerances here."""
    v, dt, steps = (1.0, 2e-4, [50] * 4) if method == "ulmpm/gpu" else (0.1, 1e-3, [100] * 4)
    g, o, fg, fo = _pair(oracle_mod, W.bouncing_balls, steps, centre=0.16, method=method, sub="APIC",
                         basis="cubic-spline", v=v, dt=dt)
    assert _collided(o, v0=v)
    _check(g, o, {"x": 3e-5, "v": 5e-4, "sigma": 5e-3})
    assert rel(fg, fo) < 5e-3


def test_bouncing_balls_usf(gpu_lib, oracle_mod):
    g, o, fg, fo = _pair(oracle_mod, W.bouncing_balls, [100] * 3, centre=0.16, scheme="usf")
    assert _collided(o)
    _check(g, o, {"x": 1e-6, "v": 2e-3, "sigma": 5e-3})


def _copper_disks(f, method, mu=0.3, v=50.0, vy=20.0):
    """Two Johnson-Cook copper disks (2-D TLMPM, thermo-mechanical, units GPa,
    mm, ms) in an oblique impact with friction: the frictional heat goes into
    the heat source gamma of both solids."""
    sim = MPM(f)
    sim.method(method, "FLIP", "cubic-spline", 0.99, "thermo-mechanical")
    sim.scheme("musl")
    h = 0.25
    sim.dimension(2, -4, 4, -4, 4, h)
    E, nu, rho = 115.0, 0.31, 8.94e-6
    K, G = E / (3 * (1 - 2 * nu)), E / (2 * (1 + nu))
    sim.eos("e", "linear", rho, K)
    sim.strength("s", "johnson_cook", G, 0.09, 0.292, 0.31, 1e-3, 0.025, 1.09, 25.0, 1356.0)
    sim.temperature("t", "plastic_work", 0.9, 385.0, 4e-4, 1e-5, 25.0, 1356.0)
    sim.material("m", "eos-strength", "e", "s", "t")
    sim.region("r1", "cylinder", -1.0, -0.5, 1.0)
    sim.region("r2", "cylinder", 1.0, 0.5, 1.0)
    sim.solid("s1", "region", "r1", 2, "m", h, 25.0)
    sim.solid("s2", "region", "r2", 2, "m", h, 25.0)
    sim.group("g1", "particles", "region", "r1", "solid", "s1")
    sim.group("g2", "particles", "region", "r2", "solid", "s2")
    sim.fix("v1", "initial_velocity_particles", "g1", v, vy, None)
    sim.fix("v2", "initial_velocity_particles", "g2", -v, -vy, None)
    sim.fix("contact", "contact/minimize_penetration", "s1", "s2", mu)
    sim.dt_factor(0.2)
    return sim


def test_frictional_heating(gpu_lib, oracle_mod):
    """Thermo-mechanical contact with friction.  The fix adds ffric |vt| dt
    (an energy) to the heat source gamma, which the temperature update
    multiplies by dt again, so its share of the temperature rise is small; the
    check is the parity of the whole thermo-mechanical state."""
    g = _copper_disks(None, "tlmpm/gpu")
    o = _copper_disks(oracle_mod.OracleBackend, "tlmpm")
    for sim in (g, o):
        sim.run(300)
    assert np.abs(o.contact_force("contact")).max() >= 0 and o.particles(0, "T").max() > 25.0
    _check(g, o, {"x": 1e-6, "v": 5e-3, "sigma": 5e-3})
    for s in (0, 1):
        assert rel(g.particles(s, "T") - 25.0, o.particles(s, "T") - 25.0) < 1e-3


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kind,mu", [("min", 0.0), ("min", 0.4), ("hertz", 0.0)])
def test_pair_force_closed_form_gpu(gpu_lib, oracle_mod, dim, kind, mu):
    """One pair of particles: the GPU's total force after one step against the
    reference's pair formula (FP32 tolerance)."""
    from test_contact_oracle import _expected, _two_particles
    contact = "contact/hertz" if kind == "hertz" else "contact/minimize_penetration"
    vz = 1.0 if dim == 3 else 0.0
    sim, s1, s2 = _two_particles(oracle_mod, dim, contact, mu=mu, v1=(0.3, 0.2, -0.1 * vz),
                                 v2=(-0.1, -0.3, 0.2 * vz), gpu=True)
    f = sim.contact_force("c")
    exp = _expected(dim, kind, s1, s2, mu, 1e-3, 1e3, 0.3)
    np.testing.assert_allclose(f, exp, rtol=0, atol=2e-5 * np.linalg.norm(exp))


def test_contact_arguments(gpu_lib):
    sim = W.bouncing_balls(None, contact=None)
    b = sim._ensure_backend()
    from karamelo_gb300 import scenario as sc
    with pytest.raises(KmpmError):
        b.add_contact(sc.ContactSpec(kind=0, solid1=0, solid2=0))
    with pytest.raises(KmpmError):
        b.add_contact(sc.ContactSpec(kind=5, solid1=0, solid2=1))
    with pytest.raises(KmpmError):
        b.add_contact(sc.ContactSpec(kind=0, solid1=0, solid2=7))
