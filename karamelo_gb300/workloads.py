"""The benchmark / parity workloads, written as Karamelo input scripts through
the :class:`~karamelo_gb300.model.MPM` command mirror.

* ``two_disks``  -- 2-D ULMPM, USL, linear basis, two colliding linear-elastic
  disks (docs/examples/two-disks.mpm:4-60 with the disks at (0.25,0.25) and
  (0.75,0.75) in a unit square, h = 0.05, 2x2 particles per cell, +-0.1 m/s
  per axis, dt = 1e-3).
* ``taylor_bar`` -- 3-D TLMPM, MUSL, cubic B-spline, copper bar on a rigid wall
  (examples/Taylor-bar/cylindrical/TLMPM/cylindrical_taylor_bar.mpm:1-89 with
  R = 3.2 mm, L = 32.4 mm, 2x2x2 particles per cell, Johnson-Cook strength +
  linear EOS; units GPa, mm, ms).
* ``dam_break``  -- 3-D ULMPM, MUSL, cubic B-spline, water column in a slip-wall
  box (examples/Dam-break/water-dam.mpm:1-73 in 3-D; Tait EOS, Newtonian
  viscosity, gravity).
* ``tensile_bars`` -- 2-D TLMPM, MUSL, cubic, Johnson-Cook strength + damage,
  velocity-driven ends (examples/Tensile_with_damage/.../inputfile:1-92 in 2-D).

All inputs are synthetic and deterministic (the populate lattice has no RNG);
parameter sweeps use seeded generators.
"""
from __future__ import annotations

import numpy as np

from .model import MPM, TimeFn


def two_disks(backend_factory=None, cellsize=0.05, ppc=2, v0=0.1, method="ulmpm/gpu", scheme="usl",
              basis="linear", pic_flip=0.99):
    sim = MPM(backend_factory)
    sim.method(method, "FLIP", basis, pic_flip)
    sim.scheme(scheme)
    sim.dimension(2, 0, 1, 0, 1, cellsize)
    sim.region("rBall1", "cylinder", 0.25, 0.25, 0.2)
    sim.region("rBall2", "cylinder", 0.75, 0.75, 0.2)
    sim.material("mat1", "linear", 1000, 1000, 0.3)
    sim.solid("sBall1", "region", "rBall1", ppc, "mat1", cellsize, 0)
    sim.solid("sBall2", "region", "rBall2", ppc, "mat1", cellsize, 0)
    sim.group("gBall1", "particles", "region", "rBall1", "solid", "sBall1")
    sim.group("gBall2", "particles", "region", "rBall2", "solid", "sBall2")
    sim.fix("v0Ball1", "initial_velocity_particles", "gBall1", v0, v0, None)
    sim.fix("v0Ball2", "initial_velocity_particles", "gBall2", -v0, -v0, None)
    sim.fix("Ek", "kinetic_energy", "all")
    sim.fix("Es", "strain_energy", "all")
    sim.set_dt(1e-3)
    return sim


def spinning_disk(backend_factory=None, cellsize=0.05, ppc=2, omega=1.0, method="ulmpm/gpu", scheme="musl",
                  sub="APIC", pic_flip=0.99, dt=1e-3, basis="cubic-spline"):
    """A linear-elastic disk (R = 0.2 m at the centre of a unit square) in
    rigid rotation at omega rad/s: the case that separates APIC,
    which transfers the rotation without loss, from PIC, which damps it."""
    import numpy as np
    sim = MPM(backend_factory)
    _method(sim, method, sub, basis, pic_flip)
    sim.scheme(scheme)
    sim.dimension(2, 0, 1, 0, 1, cellsize)
    sim.region("rDisk", "cylinder", 0.5, 0.5, 0.2)
    sim.material("mat1", "linear", 1000, 1e4, 0.3)
    sim.solid("sDisk", "region", "rDisk", ppc, "mat1", cellsize, 0)
    sol = sim.s.solids[0]
    r = sol.x0 - np.array([0.5, 0.5, 0.0])
    sol.v[:, 0] = -omega * r[:, 1]
    sol.v[:, 1] = omega * r[:, 0]
    sim.set_dt(dt)
    return sim


def angular_momentum(sim, centre=(0.5, 0.5)):
    """L_z of solid 0 about centre: sum m ((x - xc) v_y - (y - yc) v_x)."""
    import numpy as np
    x, v = sim.particles(0, "x"), sim.particles(0, "v")
    m = sim.s.solids[0].mass
    return float(np.sum(m * ((x[:, 0] - centre[0]) * v[:, 1] - (x[:, 1] - centre[1]) * v[:, 0])))


# Copper, units GPa / mm / ms.  E = 115 GPa and nu = 0.31 give the shear
# modulus the Johnson-Cook law needs (examples/Taylor-bar/.../cylindrical_taylor_bar.mpm:5-8).
COPPER = dict(E=115.0, nu=0.31, rho=8.94e-6, K=137.0, A=0.09, B=0.292, n=0.31, C=0.025, epsdot0=1e-3,
              m=0.0, Tr=25.0, Tm=1600.0)


def _method(sim, method, sub, basis, pic_flip):
    if sub in ("FLIP", "AFLIP", "ASFLIP"):
        sim.method(method, sub, basis, pic_flip)
    else:
        sim.method(method, sub, basis)


def taylor_bar(backend_factory=None, cellsize=0.2, R=3.2, L=32.4, ppc=2, v0=190.0, method="tlmpm/gpu",
               scheme="musl", basis="cubic-spline", pic_flip=0.99, dt_factor=0.1, params=None, sub="FLIP"):
    p = dict(COPPER)
    if params:
        p.update(params)
    G = p["E"] / (2 * (1 + p["nu"]))
    hL = L / 2
    sim = MPM(backend_factory)
    _method(sim, method, sub, basis, pic_flip)
    sim.scheme(scheme)
    x_wall = hL
    Df = 2.5 * R
    sim.dimension(3, -hL, x_wall, -Df, Df, -Df, Df, cellsize)
    sim.eos("eosl", "linear", p["rho"], p["K"])
    sim.strength("jc", "johnson_cook", G, p["A"], p["B"], p["n"], p["epsdot0"], p["C"], p["m"], p["Tr"], p["Tm"])
    sim.material("mat", "eos-strength", "eosl", "jc")
    sim.region("cyl", "cylinder", "x", 0, 0, R, -hL, hL)
    sim.solid("solid1", "region", "cyl", ppc, "mat", cellsize, p["Tr"])
    sim.region("region2", "block", x_wall - 0.5 * cellsize, "INF", "INF", "INF", "INF", "INF")
    sim.group("groupn2", "nodes", "region", "region2", "solid", "solid1")
    sim.group("gBall1", "particles", "region", "cyl", "solid", "solid1")
    sim.fix("v0Ball1", "initial_velocity_particles", "gBall1", v0, None, None)
    sim.dt_factor(dt_factor)
    return sim


def taylor_bar_wall(sim):
    """The wall fix the Taylor-bar script adds after run(1) (cylindrical_taylor_bar.mpm:86-89)."""
    sim.fix("BC_Wall", "velocity_nodes", "groupn2", 0, None, None)


def dam_break(backend_factory=None, cellsize=0.005, Lx=1.6, Ly=0.4, Lz=0.8, wx=0.4, wy=0.4, wz=0.8, ppc=2,
              method="ulmpm/gpu", scheme="musl", basis="cubic-spline", pic_flip=0.99, dt_factor=0.1,
              K=2e6, gamma=7.0, rho0=1000.0, mu=1e-3, g=-9.81, sub="FLIP"):
    sim = MPM(backend_factory)
    _method(sim, method, sub, basis, pic_flip)
    sim.scheme(scheme)
    sim.dimension(3, 0, Lx, 0, Ly, 0, Lz, cellsize)
    sim.eos("eosf", "fluid", rho0, K, gamma)
    sim.strength("sf", "fluid", mu)
    sim.material("water", "eos-strength", "eosf", "sf")
    sim.region("water", "block", 0, wx, 0, wy, 0, wz)
    sim.solid("w", "region", "water", ppc, "water", cellsize, 0)
    q = cellsize / 4
    # slip walls on the six faces: the normal velocity component is zero
    sim.region("xlo", "block", "-INF", q, "-INF", "INF", "-INF", "INF")
    sim.region("xhi", "block", Lx - q, "INF", "-INF", "INF", "-INF", "INF")
    sim.region("ylo", "block", "-INF", "INF", "-INF", q, "-INF", "INF")
    sim.region("yhi", "block", "-INF", "INF", Ly - q, "INF", "-INF", "INF")
    sim.region("zlo", "block", "-INF", "INF", "-INF", "INF", "-INF", q)
    sim.region("zhi", "block", "-INF", "INF", "-INF", "INF", Lz - q, "INF")
    for name, axis in (("xlo", 0), ("xhi", 0), ("ylo", 1), ("yhi", 1), ("zlo", 2), ("zhi", 2)):
        sim.group("g" + name, "nodes", "region", name, "solid", "w")
        vals = [None, None, None]
        vals[axis] = 0.0
        sim.fix("bc" + name, "velocity_nodes", "g" + name, *vals)
    sim.fix("fbody", "body_force", "all", None, None, g)
    sim.dt_factor(dt_factor)
    return sim


WELDOX = dict(E=211.0, nu=0.33, rho=7.75e-6, A=0.499, B=0.382, n=0.458, S=1.5, c0=5030.0)
DAMAGE = dict(d1=0.54, d2=4.89, d3=-3.03, d4=0.014, d5=1.12)


def tensile_bar_2d(backend_factory=None, cellsize=0.4, hLx=10.0, hLy=2.0, ppc=2, vend=1.0, damage=None,
                   method="tlmpm/gpu", scheme="musl", basis="cubic-spline", pic_flip=0.99, dt_factor=0.1, ramp=True):
    """One 2-D TLMPM tensile bar, aspect ratio hLx/hLy, ends pulled at +-vend
    (ramped as vend (1 - exp(-time)) like the reference script, or constant)."""
    d = dict(DAMAGE)
    if damage:
        d.update(damage)
    p = WELDOX
    K = p["E"] / (3 * (1 - 2 * p["nu"]))
    G = p["E"] / (2 * (1 + p["nu"]))
    sim = MPM(backend_factory)
    sim.method(method, "FLIP", basis, pic_flip)
    sim.scheme(scheme)
    sim.dimension(2, -2 * hLx, 2 * hLx, -2 * hLy, 2 * hLy, cellsize)
    sim.eos("eoss", "shock", p["rho"], K, p["c0"], p["S"], 0, 0, 0, 0, 0)
    sim.strength("sjc", "johnson_cook", G, p["A"], p["B"], p["n"], 1.0, 0.0, 0.0, 0.0, 1000.0)
    sim.damage("djc", "damage_johnson_cook", d["d1"], d["d2"], d["d3"], d["d4"], d["d5"], 1.0, 0.0, 1000.0)
    sim.material("mat", "eos-strength", "eoss", "sjc", "djc")
    sim.region("box", "block", -hLx, hLx, -hLy, hLy)
    sim.solid("bar", "region", "box", ppc, "mat", cellsize, 0)
    xbc = hLx - cellsize
    sim.region("left", "block", "-INF", -xbc, "-INF", "INF")
    sim.region("right", "block", xbc, "INF", "-INF", "INF")
    sim.group("gl", "nodes", "region", "left", "solid", "bar")
    sim.group("gr", "nodes", "region", "right", "solid", "bar")
    if ramp:
        sim.fix("BC_left", "velocity_nodes", "gl", TimeFn(-vend, 0, vend, -1.0), None)
        sim.fix("BC_right", "velocity_nodes", "gr", TimeFn(vend, 0, -vend, -1.0), None)
    else:
        sim.fix("BC_left", "velocity_nodes", "gl", -vend, None)
        sim.fix("BC_right", "velocity_nodes", "gr", vend, None)
    sim.dt_factor(dt_factor)
    return sim


def bouncing_balls(backend_factory=None, method="tlmpm/gpu", sub="FLIP", basis="linear", pic_flip=0.99,
                   contact="contact/minimize_penetration", mu=0.0, N=40, ppc=2, v=0.1, R=0.2, centre=0.3,
                   offset=0.0, dt=1e-3, E=1e3, scheme="musl", vy=None):
    """Two linear-elastic balls meeting through a contact fix
    (examples/Bouncing_balls/TLMPM/FLIP/bouncing_balls2.mpm:1-68: 2-D unit box,
    N = 40 cells per side, R = 0.2, 2x2 particles per cell, +-v per axis,
    E = 1e3, nu = 0.3, rho = 1000, dt = 1e-3).  The balls sit at +-(centre,
    centre); ``offset`` shifts both across the line of approach (+-offset along
    (1, -1)/sqrt 2) for an oblique impact; ``vy`` replaces the y velocity."""
    L = 1.0
    hL = 0.5 * L
    cellsize = L / N
    sim = MPM(backend_factory)
    _method(sim, method, sub, basis, pic_flip)
    sim.scheme(scheme)
    sim.dimension(2, -hL, hL, -hL, hL, cellsize)
    s = offset / np.sqrt(2.0)
    sim.region("rBall1", "cylinder", -centre + s, -centre - s, R)
    sim.region("rBall2", "cylinder", centre - s, centre + s, R)
    sim.material("mat1", "linear", 1000, E, 0.3)
    sim.solid("sBall1", "region", "rBall1", ppc, "mat1", cellsize, 0)
    sim.solid("sBall2", "region", "rBall2", ppc, "mat1", cellsize, 0)
    sim.group("gBall1", "particles", "region", "rBall1", "solid", "sBall1")
    sim.group("gBall2", "particles", "region", "rBall2", "solid", "sBall2")
    vy = v if vy is None else vy
    sim.fix("v0Ball1", "initial_velocity_particles", "gBall1", v, vy, None)
    sim.fix("v0Ball2", "initial_velocity_particles", "gBall2", -v, -vy, None)
    if contact == "contact/hertz":
        sim.fix("contact", contact, "sBall1", "sBall2")
    elif contact:
        sim.fix("contact", contact, "sBall1", "sBall2", mu)
    sim.fix("Ek", "kinetic_energy", "all")
    sim.fix("Es", "strain_energy", "all")
    sim.set_dt(dt)
    return sim


def hertz_spheres(backend_factory=None, method="tlmpm/gpu", sub="FLIP", basis="cubic-spline", pic_flip=0.99,
                  contact="contact/hertz", mu=0.0, cellsize=0.05, ppc=2, v=0.5, R=0.1, gap=0.01, dt=2e-4,
                  E=1e4, scheme="musl"):
    """Two linear-elastic spheres approaching along x in a 3-D box, in contact
    through a contact fix (the 3-D branch of both fixes)."""
    sim = MPM(backend_factory)
    _method(sim, method, sub, basis, pic_flip)
    sim.scheme(scheme)
    sim.dimension(3, -0.5, 0.5, -0.25, 0.25, -0.25, 0.25, cellsize)
    c = R + 0.5 * gap
    sim.region("rA", "sphere", -c, 0.0, 0.0, R)
    sim.region("rB", "sphere", c, 0.0, 0.0, R)
    sim.material("mat1", "linear", 1000, E, 0.3)
    sim.solid("sA", "region", "rA", ppc, "mat1", cellsize, 0)
    sim.solid("sB", "region", "rB", ppc, "mat1", cellsize, 0)
    sim.group("gA", "particles", "region", "rA", "solid", "sA")
    sim.group("gB", "particles", "region", "rB", "solid", "sB")
    sim.fix("vA", "initial_velocity_particles", "gA", v, 0.0, 0.0)
    sim.fix("vB", "initial_velocity_particles", "gB", -v, 0.0, 0.0)
    if contact == "contact/hertz":
        sim.fix("contact", contact, "sA", "sB")
    else:
        sim.fix("contact", contact, "sA", "sB", mu)
    sim.set_dt(dt)
    return sim


def taylor_bar_axisymmetric(backend_factory=None, cellsize=0.2, R=3.2, L=32.4, ppc=2, v0=190.0,
                            method="tlmpm/gpu", scheme="musl", basis="cubic-spline", pic_flip=0.99,
                            dt_factor=0.1, sub="FLIP"):
    """The copper Taylor bar as a 2-D axisymmetric run (x = r in [0, R], y = z;
    units GPa, mm, ms): the bar of ``taylor_bar`` on its meridian plane, moving
    along y towards the wall at y = L/2, with the axis nodes held at v_r = 0."""
    p = dict(COPPER)
    G = p["E"] / (2 * (1 + p["nu"]))
    hL = L / 2
    sim = MPM(backend_factory)
    _method(sim, method, sub, basis, pic_flip)
    sim.scheme(scheme)
    sim.dimension(2, 0.0, 2.5 * R, -hL, hL, cellsize)
    sim.axisymmetric("true")
    sim.eos("eosl", "linear", p["rho"], p["K"])
    sim.strength("jc", "johnson_cook", G, p["A"], p["B"], p["n"], p["epsdot0"], p["C"], p["m"], p["Tr"], p["Tm"])
    sim.material("mat", "eos-strength", "eosl", "jc")
    sim.region("bar", "block", 0.0, R, -hL, hL)
    sim.solid("solid1", "region", "bar", ppc, "mat", cellsize, p["Tr"])
    sim.region("wall", "block", "-INF", "INF", hL - 0.5 * cellsize, "INF")
    sim.region("axis", "block", "-INF", 0.25 * cellsize, "-INF", "INF")
    sim.group("gwall", "nodes", "region", "wall", "solid", "solid1")
    sim.group("gaxis", "nodes", "region", "axis", "solid", "solid1")
    sim.group("gbar", "particles", "region", "bar", "solid", "solid1")
    sim.fix("v0", "initial_velocity_particles", "gbar", None, v0, None)
    sim.fix("BC_axis", "velocity_nodes", "gaxis", 0, None)
    sim.dt_factor(dt_factor)
    return sim


def taylor_bar_axisymmetric_wall(sim):
    """The wall of the axisymmetric bar, added after the first step."""
    sim.fix("BC_Wall", "velocity_nodes", "gwall", None, 0)


def vertical_bar(backend_factory=None, N=10, ppc=1, method="tlmpm/gpu", sub="FLIP", basis="cubic-spline",
                 pic_flip=0.99, scheme="musl"):
    """A neo-Hookean bar (1 m long, 1 m x 1 m section; E = 1e6 Pa, nu = 0.3,
    rho = 1050 kg/m^3) hanging from its top face under 1000 m/s^2 of gravity
    (examples/Vertical_bar/Cubic_spline/N_20/FLIP/vertical_bar.mpm): the nodes
    at y >= -cellsize/4 hold v_y = 0, dt_factor 0.2, N cells along the bar.
    The reference logs dy_tip, the vertical displacement of the centre of
    mass of the particles in the bottom corner cell (``vertical_bar_tip``)."""
    L = 1.0
    hL = 0.5 * L
    h = L / N
    sim = MPM(backend_factory)
    _method(sim, method, sub, basis, pic_flip)
    sim.scheme(scheme)
    sim.dimension(3, -hL, hL, -L, 0.0, -hL, hL, h)
    sim.region("box", "block", -hL, hL, -L, 0.0, -hL, hL)
    sim.material("mat1", "neo-hookean", 1050.0, 1e6, 0.3)
    sim.solid("solid1", "region", "box", ppc, "mat1", h, 0)
    sim.region("rBCLX", "block", "INF", "INF", -h / 4, "INF", "INF", "INF")
    sim.group("gBCLX", "nodes", "region", "rBCLX", "solid", "solid1")
    sim.fix("fBCLX", "velocity_nodes", "gBCLX", None, 0, None)
    sim.fix("fbody", "body_force", "all", 0, -1e3, 0)
    sim.dt_factor(0.2)
    return sim


def vertical_bar_tip(sim, x=None):
    """Mass-weighted centre of the particles in the region
    block(INF, -hL + h/2, INF, -L + 3h/4, INF, -hL + h/2) of the script
    (its group gTip), from positions x (default: the initial lattice)."""
    import numpy as np
    s = sim.s.solids[0]
    x0 = s.x0
    h = sim.cellsize
    sel = (x0[:, 0] <= -0.5 + h / 2 + 1e-12) & (x0[:, 1] <= -1.0 + 3 * h / 4 + 1e-12) & \
          (x0[:, 2] <= -0.5 + h / 2 + 1e-12)
    xs = x0 if x is None else x
    m = s.mass[sel]
    return (m[:, None] * xs[sel]).sum(0) / m.sum()


def block_bar(f, method, strength, eos="linear", thermal=False, damage=None, basis="cubic-spline",
               scheme="musl", v0=100.0, mat_kind="eos-strength"):
    """Small 3-D bar (2 x 1.2 x 1.2 mm, cellsize 0.4) hitting a wall, with the
    given strength / EOS / temperature laws (units GPa, mm, ms)."""
    sim = MPM(f)
    extra = ["thermo-mechanical"] if thermal else []
    sim.method(method, "FLIP", basis, 0.99, *extra)
    sim.scheme(scheme)
    sim.dimension(3, -4, 1.2, -1.2, 1.2, -1.2, 1.2, 0.4)
    E, nu, rho = 115.0, 0.31, 8.94e-6
    K, G = E / (3 * (1 - 2 * nu)), E / (2 * (1 + nu))
    if mat_kind == "eos-strength":
        if eos == "linear":
            sim.eos("e", "linear", rho, K)
        else:
            sim.eos("e", "shock", rho, K, 3940.0, 1.49, 2.0, 3.8e-7, 25.0, 1.0, 0.1)
        args = {"johnson_cook": (G, 0.09, 0.292, 0.31, 1e-3, 0.025, 1.09, 25.0, 1356.0),
                "plastic": (G, 0.2), "swift": (G, 0.09, 0.3, 0.01, 0.4), "linear": (G,)}[strength]
        sim.strength("s", strength, *args)
        laws = ["e", "s"]
        if thermal:
            sim.temperature("t", "plastic_work", 0.9, 385.0, 4e-4, 1e-5, 25.0, 1356.0)
            laws.append("t")
        sim.material("m", "eos-strength", *laws)
    else:
        sim.material("m", mat_kind, rho, E, nu)
    sim.region("bar", "block", -2, 0.8, -0.8, 0.8, -0.8, 0.8)
    sim.solid("s1", "region", "bar", 2, "m", 0.4, 25.0)
    sim.region("wall", "block", 0.6, "INF", "-INF", "INF", "-INF", "INF")
    sim.group("gw", "nodes", "region", "wall", "solid", "s1")
    sim.group("gp", "particles", "region", "bar", "solid", "s1")
    sim.fix("v0", "initial_velocity_particles", "gp", v0, None, None)
    sim.dt_factor(0.2)
    return sim
