"""Host setup (populate, Grid::init, groups, fixes) against the oracle and the
reference's documented numbers (CPU)."""
import numpy as np
import pytest

from karamelo_gb300 import KarameloError, MPM, workloads as W
from karamelo_gb300 import scenario as sc


def test_two_disk_particle_count():
    sim = W.two_disks()
    assert [s.np for s in sim.s.solids] == [208, 208]
    g = sim.s.grids[0]
    assert (g.nx, g.ny, g.nz) == (21, 21, 1)
    assert np.allclose(sim.s.solids[0].mass, 1000 * 0.05 ** 2 / 4)


def test_taylor_bar_particle_counts():
    s02 = W.taylor_bar(cellsize=0.2).s
    assert s02.solids[0].np == 1045872
    g = s02.grids[0]
    assert (g.nx, g.ny, g.nz) == (163, 33, 33)


def test_grid_geometry_matches_oracle(oracle_mod):
    for cs, basis in ((0.8, "cubic-spline"), (0.8, "Bernstein-quadratic"), (0.5, "linear")):
        sim = W.taylor_bar(oracle_mod.OracleBackend, cellsize=cs, basis=basis, method="tlmpm")
        b = sim._ensure_backend()
        info = b.grid_info(0)
        g = sim.s.grids[0]
        assert info["dims"] == [g.nx, g.ny, g.nz, g.nxg, g.nyg, g.nzg]
        assert info["h"] == g.h


def test_ntype_matches_oracle(oracle_mod):
    sim = W.taylor_bar(oracle_mod.OracleBackend, cellsize=0.8, method="tlmpm")
    nt = sim._ensure_backend().grid_ntype(0)
    g = sim.s.grids[0]
    i, j, k = np.meshgrid(np.arange(g.nx), np.arange(g.ny), np.arange(g.nz), indexing="ij")
    f = lambda a, n: np.minimum(2, a) - np.minimum(n - 1 - a, 2)  # src/grid.cpp:237-239
    assert np.array_equal(nt[:, 0], f(i.ravel(), g.nxg))
    assert np.array_equal(nt[:, 2], f(k.ravel(), g.nzg))


def test_wall_group_nodes():
    sim = W.taylor_bar(cellsize=0.8)
    m = sim.groups["groupn2"]["masks"][0]
    x = sim.s.grids[0].node_positions(3)
    assert np.array_equal(m, x[:, 0] >= 16.2 - 0.4)


def test_unsupported_inputs_raise():
    sim = MPM()
    with pytest.raises(KarameloError):
        sim.method("tlmpm", "FLIP", "cubic-spline", 0.99)      # CPU style: not this package's
    sim.method("ulmpm/gpu", "FLIP", "linear", 0.99)
    with pytest.raises(KarameloError):
        sim.method("ulmpm/gpu", "FLIP", "Bernstein-quadratic", 0.99)
    with pytest.raises(KarameloError):
        sim.method("ulmpm/gpu", "APIC", "linear")   # src/solid.cpp:1452: linear APIC is TLMPM only
    with pytest.raises(KarameloError):
        sim.method("tlmpm/gpu", "APIC", "Bernstein-quadratic")
    sim.dimension(2, 0, 1, 0, 1, 0.1)
    with pytest.raises(KarameloError):
        sim.material("r", "rigid", 1000)
    sim.region("b", "block", 0.2, 0.4, 0.2, 0.4)
    sim.material("m", "linear", 1000, 1e3, 0.3)
    sim.solid("s", "region", "b", 2, "m", 0.1, 0)
    with pytest.raises(KarameloError):
        sim.fix("c", "contact_hertz", "all")


def test_fix_lowering_time_function():
    sim = W.tensile_bar_2d(cellsize=0.8)
    f = [x for x in sim.s.fixes if x.name == "BC_right"][0]
    assert f.kind == sc.FIX_VELOCITY_NODES and f.set == (1, 0, 0)
    assert np.allclose(f.coef[0], [1.0, 0.0, -1.0, -1.0])  # 1 - exp(-time)


def test_initial_velocity_applied_before_first_step():
    sim = W.two_disks()
    assert np.allclose(sim.s.solids[0].v[:, :2], 0.1)
    assert np.allclose(sim.s.solids[1].v[:, :2], -0.1)


def test_batch_merges_scripts():
    from karamelo_gb300.batch import Batch, tensile_sweep
    sims, params = tensile_sweep(4, seed=3, nmin=500, nmax=4000)
    got = {}
    b = Batch(sims, backend_factory=lambda s: got.setdefault("s", s))
    s = b.scenario
    assert len(s.solids) == 4 and len(s.grids) == 4 and len(s.materials) == 4
    assert [x.grid for x in s.solids] == [0, 1, 2, 3] and [x.mat for x in s.solids] == [0, 1, 2, 3]
    assert sorted({f.grid for f in s.fixes}) == [0, 1, 2, 3]
    counts = [x.np for x in s.solids]
    assert min(counts) >= 300 and max(counts) <= 6000
    d1 = [m.dam_p[0] for m in s.materials]
    assert all(0.54 * 0.7 <= v <= 0.54 * 1.3 for v in d1) and len(set(d1)) == 4
