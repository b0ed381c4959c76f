"""GPU parity: the CUDA step (through the C ABI) against the FP64 oracle on
the same scripts.  Tolerances are relative L2 norms over all particles,
stated per test; the GPU computes in FP32 (see the precision notes in each
test)."""
import numpy as np
import pytest

from karamelo_gb300 import workloads as W
from karamelo_gb300.gpu import GpuBackend, KmpmError

pytestmark = pytest.mark.gpu


def rel(a, b, floor=0.0):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), floor, 1e-300))


def pair(oracle_mod, build, steps, **kw):
    """Run one script on the GPU and on the oracle; ``steps`` mixes step
    counts and callables (fixes added between runs)."""
    g = build(None, **kw)
    o = build(oracle_mod.OracleBackend, **{**kw, "method": kw.get("method", _cpu(build)).replace("/gpu", "")})
    for sim in (g, o):
        sim._ensure_backend()
    for st in steps:
        for sim in (g, o):
            st(sim) if callable(st) else sim.run(st)
    assert isinstance(g.backend, GpuBackend)
    return g, o


def _cpu(build):
    return {W.taylor_bar: "tlmpm", W.two_disks: "ulmpm", W.dam_break: "ulmpm", W.tensile_bar_2d: "tlmpm",
            W.spinning_disk: "ulmpm", W.bouncing_balls: "tlmpm"}[build]


def check(g, o, tol, solid=0):
    for field, t in tol.items():
        e = rel(g.particles(solid, field), o.particles(solid, field))
        assert e < t, f"{field}: rel L2 {e:.3e} >= {t}"


TAYLOR_TOL = {"x": 1e-6, "v": 1e-4, "sigma": 1e-4, "eps_p": 1e-4}


@pytest.mark.parametrize("basis,scheme", [("cubic-spline", "musl"), ("cubic-spline", "usl"), ("linear", "usl"),
                                          ("linear", "musl"), ("Bernstein-quadratic", "musl"),
                                          ("quadratic-spline", "musl"), ("quadratic-spline", "usl")])
def test_taylor_bar_tlmpm(gpu_lib, oracle_mod, basis, scheme):
    """3-D TLMPM Johnson-Cook + linear EOS bar hitting the wall (the benchmark's
    physics at cellsize 0.8 mm): 1 step, wall fix, 50 steps."""
    g, o = pair(oracle_mod, W.taylor_bar, [1, W.taylor_bar_wall, 50], cellsize=0.8, basis=basis, scheme=scheme,
                method="tlmpm/gpu")
    tol = dict(TAYLOR_TOL)
    if basis == "linear":
        tol.pop("eps_p")
    check(g, o, tol)
    # dt (adjust_dt) and time agree
    assert abs(g.dt / o.dt - 1) < 1e-5 and abs(g.time / o.time - 1) < 1e-6


def test_taylor_bar_fp64_islands(gpu_lib, oracle_mod):
    """The FP64 islands (det/inverse of F, Johnson-Cook return) give the same parity."""
    def build(f, **kw):
        sim = W.taylor_bar(f, **kw)
        if f is None:
            sim.backend = GpuBackend(sim.s, precision=1)
        return sim
    g = build(None, cellsize=0.8)
    o = build(oracle_mod.OracleBackend, cellsize=0.8, method="tlmpm")
    for st in (1, W.taylor_bar_wall, 50):
        for sim in (g, o):
            st(sim) if callable(st) else sim.run(st)
    check(g, o, TAYLOR_TOL)


def test_taylor_bar_rotated_stress_and_grid(gpu_lib, oracle_mod):
    g, o = pair(oracle_mod, W.taylor_bar, [1, W.taylor_bar_wall, 30], cellsize=0.8, method="tlmpm/gpu")
    assert rel(g.particles(0, "sigma_raw"), o.particles(0, "sigma_raw")) < 1e-4
    assert rel(g.particles(0, "F"), o.particles(0, "F")) < 1e-6
    assert rel(g.particles(0, "J"), o.particles(0, "J")) < 1e-6
    assert rel(g.backend.grid(0, "mass"), o.backend.grid(0, "mass")) < 1e-6
    assert rel(g.backend.grid(0, "x"), o.backend.grid(0, "x")) < 1e-6


def test_dam_break_ulmpm(gpu_lib, oracle_mod):
    """3-D ULMPM MUSL cubic dam break (Tait EOS, viscosity, gravity, slip walls),
    cellsize 0.05 m, 100 steps: the per-step re-binning by cell is exercised."""
    g, o = pair(oracle_mod, W.dam_break, [100], cellsize=0.05, method="ulmpm/gpu")
    check(g, o, {"x": 1e-6, "v": 1e-4, "sigma": 1e-3})
    assert abs(g.time / o.time - 1) < 1e-6


def test_two_disks_cubic_collision(gpu_lib, oracle_mod):
    """2-D ULMPM MUSL cubic, two solids sharing one grid, through the collision."""
    g, o = pair(oracle_mod, W.two_disks, [2000], basis="cubic-spline", scheme="musl", method="ulmpm/gpu")
    for s in (0, 1):
        check(g, o, {"x": 1e-5, "v": 1e-4, "sigma": 1e-3}, solid=s)
    eg, eo = g.energies(), o.energies()
    assert abs(eg[0] - eo[0]) < 1e-4 * (eo[0] + eo[1]) and abs(eg[1] - eo[1]) < 1e-4 * (eo[0] + eo[1])


def test_two_disks_linear_usl(gpu_lib, oracle_mod):
    """The two-disk configuration (2-D ULMPM USL linear).  Its rigid free flight has
    exactly zero stress in FP64; FP32 rounding of p/m leaves ~1e-5 Pa of stress
    noise, which near-empty nodes amplify once particles land exactly on nodes
    (step ~125).  Parity is therefore checked before that event."""
    g, o = pair(oracle_mod, W.two_disks, [100], method="ulmpm/gpu")
    for s in (0, 1):
        check(g, o, {"x": 1e-6, "v": 1e-6}, solid=s)
    assert abs(g.energies()[0] - o.energies()[0]) < 1e-6


def test_tensile_bar_damage(gpu_lib, oracle_mod):
    """2-D TLMPM cubic, shock EOS + Johnson-Cook strength + damage, velocity-driven ends."""
    g, o = pair(oracle_mod, W.tensile_bar_2d, [3000], cellsize=0.8, vend=50.0, ramp=False, method="tlmpm/gpu")
    assert o.particles(0, "eps_p").max() > 0.05 and o.particles(0, "damage_init").max() > 0
    check(g, o, {"x": 1e-6, "v": 1e-3, "sigma": 1e-3, "eps_p": 1e-3})
    dg, do = g.particles(0, "damage_init"), o.particles(0, "damage_init")
    assert rel(dg, do) < 1e-3


def test_deterministic_replay(gpu_lib):
    """Two identical runs are bit-identical (fixed-order scatter, no float atomics)."""
    out = []
    for _ in range(2):
        sim = W.taylor_bar(None, cellsize=0.8)
        sim.run(1)
        W.taylor_bar_wall(sim)
        sim.run(40)
        out.append([sim.particles(0, f) for f in ("x", "v", "sigma")])
    for a, b in zip(*out):
        assert np.array_equal(a, b)
    out = []
    for _ in range(2):
        sim = W.dam_break(None, cellsize=0.05)
        sim.run(60)
        out.append([sim.particles(0, f) for f in ("x", "v", "sigma")])
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_run_time_matches_oracle(gpu_lib, oracle_mod):
    g, o = pair(oracle_mod, W.dam_break, [], cellsize=0.05, method="ulmpm/gpu")
    ng = g.backend.run_time(0.005)
    no = o.backend.run_time(0.005)
    assert ng == no
    assert abs(g.time - o.time) < 1e-9


def test_particle_leaving_domain_is_reported(gpu_lib):
    """src/solid.cpp:617-627 as a status code: the kernel records the particle
    and the host reads the status after the step (no device fault)."""
    from karamelo_gb300 import MPM
    sim = MPM()
    sim.method("ulmpm/gpu", "FLIP", "linear", 0.99)
    sim.dimension(2, 0, 1, 0, 1, 0.05)
    sim.region("b", "cylinder", 0.7, 0.5, 0.1)
    sim.material("m", "linear", 1000, 1000, 0.3)
    sim.solid("s", "region", "b", 2, "m", 0.05, 0)
    sim.group("g", "particles", "region", "b", "solid", "s")
    sim.fix("v0", "initial_velocity_particles", "g", 10.0, 0.0, None)
    sim.set_dt(1e-3)
    with pytest.raises(KmpmError) as e:
        sim.run(60)
    assert e.value.code == -11


_block_bar = W.block_bar


def _pair_block(oracle_mod, steps, **kw):
    g = _block_bar(None, "tlmpm/gpu", **kw)
    o = _block_bar(oracle_mod.OracleBackend, "tlmpm", **kw)
    for sim in (g, o):
        sim.run(1)
        sim.fix("wall", "velocity_nodes", "gw", 0, None, None)
        sim.run(steps)
    return g, o


def test_thermal_plastic_work(gpu_lib, oracle_mod):
    """thermo-mechanical TLMPM: plastic-work heating, heat flux, JC thermal softening
    (src/temperature_plastic_work.cpp, src/solid.cpp:2743-2839)."""
    g, o = _pair_block(oracle_mod, 150, strength="johnson_cook", thermal=True)
    assert o.particles(0, "T").max() > 25.0
    check(g, o, {"x": 1e-6, "v": 1e-3, "sigma": 1e-3, "eps_p": 1e-3, "T": 1e-5})


@pytest.mark.parametrize("strength", ["plastic", "swift", "linear"])
def test_strength_laws(gpu_lib, oracle_mod, strength):
    g, o = _pair_block(oracle_mod, 150, strength=strength)
    tol = {"x": 1e-6, "v": 1e-3, "sigma": 1e-3}
    if strength != "linear":
        assert o.particles(0, "eps_p").max() > 0
        tol["eps_p"] = 1e-3
    check(g, o, tol)


def test_shock_eos_artificial_viscosity(gpu_lib, oracle_mod):
    """Mie-Grueneisen EOS with artificial viscosity (src/eos_shock.cpp:99-133)."""
    g, o = _pair_block(oracle_mod, 150, strength="johnson_cook", eos="shock")
    check(g, o, {"x": 1e-6, "v": 1e-3, "sigma": 1e-3, "eps_p": 1e-3})


@pytest.mark.parametrize("kind", ["neo-hookean", "linear"])
def test_hyperelastic_and_linear_materials(gpu_lib, oracle_mod, kind):
    g, o = _pair_block(oracle_mod, 150, strength="linear", mat_kind=kind, v0=30.0)
    check(g, o, {"x": 1e-6, "v": 1e-3, "sigma": 1e-3})


# ---------------------------------------------------------------- APIC
@pytest.mark.parametrize("scheme", ["musl", "usl"])
def test_taylor_bar_apic(gpu_lib, oracle_mod, scheme):
    """TLMPM with APIC transfers (compute_velocity_nodes_APIC and
    compute_rate_deformation_gradient_TL_APIC, src/solid.cpp:392-426,
    1006-1080): the Johnson-Cook bar at the wall, cubic spline."""
    g, o = pair(oracle_mod, W.taylor_bar, [1, W.taylor_bar_wall, 50], cellsize=0.8, scheme=scheme,
                method="tlmpm/gpu", sub="APIC")
    check(g, o, {"x": 1e-6, "v": 1e-4, "sigma": 1e-4, "eps_p": 1e-4, "F": 1e-6})


@pytest.mark.parametrize("method,scheme", [("ulmpm/gpu", "musl"), ("ulmpm/gpu", "usl"), ("tlmpm/gpu", "musl")])
def test_spinning_disk_apic(gpu_lib, oracle_mod, method, scheme):
    """A spinning linear-elastic disk with APIC (ULMPM takes x_p before the
    move for USL and after it for MUSL): state and angular momentum.  The
    stress is the small centrifugal load (rho omega^2 R^2 = 40 Pa against
    E = 1e4 Pa), so its FP32 relative error is larger than in the loaded cases."""
    g, o = pair(oracle_mod, W.spinning_disk, [1, 150], method=method, scheme=scheme)
    check(g, o, {"x": 1e-6, "v": 1e-4, "sigma": 3e-3})
    Lg, Lo = W.angular_momentum(g), W.angular_momentum(o)
    assert abs(Lg / Lo - 1) < 1e-4


def test_dam_break_apic(gpu_lib, oracle_mod):
    """The ULMPM dam break (fluid EOS, viscosity, gravity, slip walls) with APIC."""
    g, o = pair(oracle_mod, W.dam_break, [60], cellsize=0.05, method="ulmpm/gpu", sub="APIC")
    check(g, o, {"x": 1e-6, "v": 1e-4, "sigma": 1e-3})


def test_async_downloads_match_sync(gpu_lib):
    """A download queued between runs holds the state of that moment, while
    later steps run on (gather in stream order, copy on a second stream)."""
    import torch
    g = W.taylor_bar(None, cellsize=0.8)
    g._ensure_backend()
    g.run(1)
    W.taylor_bar_wall(g)
    g.run(20)
    be = g.backend
    ref = {f: be.particles(0, f) for f in ("x", "sigma", "eps_p")}
    n = g.s.solids[0].np
    out = {f: torch.empty(n * w, dtype=torch.float64, pin_memory=True) for f, w in (("x", 3), ("sigma", 9), ("eps_p", 1))}
    for f, t in out.items():
        be.particles_async(0, f, t)
    g.run(30)
    be.sync_downloads()
    for f in ref:
        assert np.array_equal(out[f].numpy().reshape(ref[f].shape), ref[f]), f
    assert not np.array_equal(be.particles(0, "x"), ref["x"])


def test_wait_download_of_one_buffer(gpu_lib):
    """kmpm_wait_download: waiting for one buffer's copy leaves the others
    queued; each buffer holds the state of the step its download was queued
    at, and a second download into a buffer replaces the first."""
    torch = pytest.importorskip("torch")
    g = W.taylor_bar(None, cellsize=0.8)
    g.backend = GpuBackend(g.s, autotune=False)
    be = g.backend
    g.run(1)
    W.taylor_bar_wall(g)
    n = g.s.solids[0].np
    bufs = [torch.empty(n * 3, dtype=torch.float64, pin_memory=True) for _ in range(3)]
    refs = []
    for k in range(3):
        g.run(10)
        refs.append(be.particles(0, "x"))
        be.particles_async(0, "x", bufs[k])
    be.wait_download(bufs[0])
    assert np.array_equal(bufs[0].numpy().reshape(-1, 3), refs[0])
    g.run(10)
    refs[0] = be.particles(0, "x")
    be.particles_async(0, "x", bufs[0])  # the buffer again: its new content
    for k in (2, 0, 1):
        be.wait_download(bufs[k])
        assert np.array_equal(bufs[k].numpy().reshape(-1, 3), refs[k]), k
    be.wait_download(bufs[1])  # nothing in flight for it: returns at once
    be.sync_downloads()


# ---------------------------------------------------------------- USF
@pytest.mark.parametrize("basis", ["cubic-spline", "linear"])
def test_taylor_bar_usf(gpu_lib, oracle_mod, basis):
    """USF::run (src/usf.cpp:34-95): stress from the first scatter's grid
    velocities, then the forces of the new stress (TLMPM, Johnson-Cook bar)."""
    g, o = pair(oracle_mod, W.taylor_bar, [1, W.taylor_bar_wall, 50], cellsize=0.8, basis=basis, scheme="usf",
                method="tlmpm/gpu")
    tol = dict(TAYLOR_TOL)
    if basis == "linear":
        tol.pop("eps_p")
    check(g, o, tol)
    assert abs(g.dt / o.dt - 1) < 1e-5


def test_dam_break_usf(gpu_lib, oracle_mod):
    g, o = pair(oracle_mod, W.dam_break, [60], cellsize=0.05, method="ulmpm/gpu", scheme="usf")
    check(g, o, {"x": 1e-6, "v": 1e-4, "sigma": 1e-3})


def test_tensile_bar_usf(gpu_lib, oracle_mod):
    """2-D TLMPM tensile bar with Johnson-Cook damage under USF."""
    g, o = pair(oracle_mod, W.tensile_bar_2d, [400], cellsize=0.5, scheme="usf", vend=20.0, ramp=False)
    check(g, o, {"x": 1e-6, "v": 1e-3, "sigma": 1e-3})


# ---------------------------------------------------------------- quadratic spline
def test_dam_break_quadratic(gpu_lib, oracle_mod):
    """ULMPM dam break with the quadratic B-spline (src/basis_functions.h:140-241)."""
    g, o = pair(oracle_mod, W.dam_break, [60], cellsize=0.05, method="ulmpm/gpu", basis="quadratic-spline")
    check(g, o, {"x": 1e-6, "v": 1e-4, "sigma": 1e-3})


def test_spinning_disk_apic_quadratic(gpu_lib, oracle_mod):
    """APIC with the quadratic spline (Di = 4 / h^2)."""
    g, o = pair(oracle_mod, W.spinning_disk, [1, 150], method="ulmpm/gpu", scheme="musl", basis="quadratic-spline")
    check(g, o, {"x": 1e-6, "v": 1e-4, "sigma": 3e-3})
    assert abs(W.angular_momentum(g) / W.angular_momentum(o) - 1) < 1e-4


# ---------------------------------------------------------------- AFLIP / ASFLIP / MLS
@pytest.mark.parametrize("sub", ["AFLIP", "ASFLIP", "MLS"])
def test_dam_break_affine_submethods(gpu_lib, oracle_mod, sub):
    """ULMPM dam break with the other affine sub-methods: AFLIP and ASFLIP
    (affine transfers with the FLIP blend; ASFLIP moves particles with the
    blended velocity, src/ulmpm.cpp:453-473) and MLS (internal forces from
    moments, src/solid.cpp:524-574)."""
    g, o = pair(oracle_mod, W.dam_break, [60], cellsize=0.05, method="ulmpm/gpu", sub=sub)
    check(g, o, {"x": 1e-6, "v": 1e-4, "sigma": 1e-3})


@pytest.mark.parametrize("sub", ["ASFLIP", "MLS"])
def test_spinning_disk_affine_submethods(gpu_lib, oracle_mod, sub):
    g, o = pair(oracle_mod, W.spinning_disk, [1, 150], method="ulmpm/gpu", scheme="musl", sub=sub)
    check(g, o, {"x": 1e-6, "v": 1e-4, "sigma": 3e-3})
    assert abs(W.angular_momentum(g) / W.angular_momentum(o) - 1) < 1e-4


# ---------------------------------------------------------------- APIC, linear basis (TLMPM)
@pytest.mark.parametrize("ppc", [1, 2])
def test_bouncing_balls_apic_linear(gpu_lib, oracle_mod, ppc):
    """The reference's bouncing-balls example in its APIC form (TLMPM, linear
    basis, examples/Bouncing_balls/TLMPM/APIC/bouncing_balls2.mpm): Di = 16/4
    or 16/3 over cellsize^2 by the particles per cell (src/solid.cpp:1447-1462),
    through the contact fix."""
    g, o = pair(oracle_mod, W.bouncing_balls, [300], method="tlmpm/gpu", sub="APIC", basis="linear",
                centre=0.16, ppc=ppc)
    for s in (0, 1):
        check(g, o, {"x": 3e-5, "v": 5e-4, "sigma": 5e-3}, solid=s)


def test_taylor_bar_apic_linear(gpu_lib, oracle_mod):
    g, o = pair(oracle_mod, W.taylor_bar, [1, W.taylor_bar_wall, 50], cellsize=0.8, method="tlmpm/gpu",
                sub="APIC", basis="linear")
    check(g, o, {"x": 1e-6, "v": 1e-4, "sigma": 1e-4, "F": 1e-6})


def test_run_until_batches_match_run_time(gpu_lib):
    """kmpm_run_until (a run_time that ends at the output steps, as the GPU
    scheme's loop does) in batches of 7 steps reaches the same state as one
    kmpm_run_time to the same end time, bit for bit."""
    import ctypes
    out = []
    for batched in (False, True):
        sim = W.taylor_bar(None, cellsize=0.8)
        sim.run(1)
        W.taylor_bar_wall(sim)
        be = sim.backend
        t_end = sim.time + 1e-3
        if batched:
            done, total = ctypes.c_int(0), 0
            while True:
                assert be.L.kmpm_run_until(be.h, 7, t_end, ctypes.byref(done)) == 0
                total += done.value
                assert done.value <= 7
                if done.value < 7 or sim.time >= t_end:
                    break
            assert total > 7
        else:
            sim.run_time(1e-3)
        out.append((sim.time, sim.particles(0, "x"), sim.particles(0, "sigma")))
    assert out[0][0] == out[1][0]
    for a, b in zip(out[0][1:], out[1][1:]):
        assert np.array_equal(a, b)


def test_sigma6_download_is_the_dumped_components(gpu_lib):
    """KMPM_P_SIGMA_ROT6: s11 s22 s33 s12 s13 s23 of the rotated stress, as
    the reference's particle dump writes them, equal to the 3x3 download."""
    sim = W.taylor_bar(None, cellsize=0.8)
    sim.run(1)
    W.taylor_bar_wall(sim)
    sim.run(20)
    s9, s6 = sim.particles(0, "sigma"), sim.particles(0, "sigma6")
    assert s6.shape == (s9.shape[0], 6)
    for k, (a, b) in enumerate(((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))):
        assert np.array_equal(s6[:, k], s9[:, a, b])
