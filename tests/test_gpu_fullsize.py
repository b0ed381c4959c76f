"""Size-independent properties of the benchmark workload at its full size:
the copper Taylor bar at cellsize 0.1 mm (8,354,016 particles, 1,373,125
nodes, TLMPM MUSL cubic spline, Johnson-Cook), where the FP64 oracle is too
slow to run beside it.

* mass: the nodal masses sum to the particle masses (Solid::compute_mass_nodes,
  src/solid.cpp:317-335, is a partition of unity);
* momentum: in free flight (before the wall) the bar keeps M v0 and no
  transverse momentum;
* determinism: two contexts run the same steps to bit-identical states;
* symmetry: the populate lattice and the bar are symmetric under y -> -y and
  z -> -z, and so is the solution: mirrored particles stay mirror images;
* energy: after impact the kinetic energy only falls and the kinetic plus
  strain energy stays below the initial kinetic energy (plastic work
  dissipates it), and no particle passes the wall.
"""
import numpy as np
import pytest

from karamelo_gb300 import workloads as W
from karamelo_gb300.gpu import GpuBackend

pytestmark = pytest.mark.gpu

H = 0.1       # mm, the benchmark's cellsize
V0 = 190.0    # mm/ms


def _bar():
    sim = W.taylor_bar(None, cellsize=H)
    sim.backend = GpuBackend(sim.s, track_strain=True, autotune=False)
    return sim


@pytest.fixture(scope="module")
def bar50():
    """The bar after its first step, the wall, and 50 more steps."""
    sim = _bar()
    sim.run(1)
    p1 = sim.particles(0, "v")
    W.taylor_bar_wall(sim)
    e0 = sim.energies()
    sim.run(50)
    return sim, p1, e0


def test_full_size_counts(gpu_lib, bar50):
    sim, _, _ = bar50
    assert sim.s.solids[0].np == 8354016 and sim.s.grids[0].nnodes == 1373125


def test_mass_conservation(gpu_lib, bar50):
    sim, _, _ = bar50
    mp = sim.s.solids[0].mass.sum()
    mg = sim.backend.grid(0, "mass").sum()
    assert abs(mg / mp - 1) < 1e-5


def test_free_flight_momentum(gpu_lib, bar50):
    sim, v1, _ = bar50
    m = sim.s.solids[0].mass
    P = (m[:, None] * v1).sum(0)
    M = m.sum()
    assert abs(P[0] / (M * V0) - 1) < 1e-6
    assert np.abs(P[1:]).max() < 1e-6 * M * V0


def test_bit_identical_replay(gpu_lib, bar50):
    sim, _, _ = bar50
    b = _bar()
    b.run(1)
    W.taylor_bar_wall(b)
    b.run(50)
    for f in ("x", "v", "sigma", "eps_p"):
        assert np.array_equal(sim.particles(0, f), b.particles(0, f)), f
    assert sim.backend.scalars() == b.backend.scalars()


def test_mirror_symmetry(gpu_lib, bar50):
    sim, _, _ = bar50
    x0 = sim.s.solids[0].x0
    x = sim.particles(0, "x")
    ep = sim.particles(0, "eps_p")
    # pair every particle with its y -> -y mirror through the lattice keys
    key = np.round(x0 / (H / 4)).astype(np.int64)
    order = np.lexsort((key[:, 2], key[:, 1], key[:, 0]))
    mirror_key = key * np.array([1, -1, 1])
    morder = np.lexsort((mirror_key[:, 2], mirror_key[:, 1], mirror_key[:, 0]))
    assert np.array_equal(key[order], mirror_key[morder])
    a, b = order, morder
    span = x[:, 0].max() - x[:, 0].min()
    assert np.abs(x[a, 0] - x[b, 0]).max() < 1e-5 * span
    assert np.abs(x[a, 1] + x[b, 1]).max() < 1e-5 * span
    assert np.abs(ep[a] - ep[b]).max() < 1e-3 * ep.max()


def test_energy_and_wall(gpu_lib, bar50):
    sim, _, e0 = bar50
    ek0 = e0[0]
    ek, es = sim.energies()
    assert ek < ek0 and ek + es < ek0
    sim.run(50)
    ek2, es2 = sim.energies()
    assert ek2 < ek
    assert sim.particles(0, "x")[:, 0].max() <= 32.4 / 2 + 1e-6
    assert sim.particles(0, "eps_p").max() > 0.1


def test_dam_break_full_size(gpu_lib):
    """The dam break at its full size (cellsize 5 mm, 8,192,000 particles, ULMPM
    with re-binning every step): bit-identical replay, mass on the grid,
    and the vertical momentum between free fall and rest."""
    def dam():
        sim = W.dam_break(None)
        sim.backend = GpuBackend(sim.s, track_strain=False, autotune=False)
        return sim
    a, b = dam(), dam()
    assert a.s.solids[0].np == 8192000
    m = a.s.solids[0].mass
    for sim in (a, b):
        sim.run(20)
    for f in ("x", "v", "sigma"):
        assert np.array_equal(a.particles(0, f), b.particles(0, f)), f
    mg = a.backend.grid(0, "mass").sum()
    assert abs(mg / m.sum() - 1) < 1e-5
    # vertical momentum = gravity's impulse -M g t plus the floor's (>= 0)
    t = a.time
    pz = (m * a.particles(0, "v")[:, 2]).sum()
    assert -1.001 * m.sum() * 9.81 * t <= pz <= 0.0
