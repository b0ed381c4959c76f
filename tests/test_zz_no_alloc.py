"""kmpm_p2g_mass_noalloc: the nodal-mass scatter for applications that own
all of their GPU memory through their own pool allocator and may not call
cudaMalloc themselves.  Its output is checked, through the C ABI, against the
nodal mass that the regular entry points compute (kmpm_run, then
kmpm_download_grid), bit for bit, on two calls in a row; against an FP64
scatter on the CPU where no regular context is built; and across calls that
leave different contents in the shared scratch array.  This file is collected
last on purpose: a run that stops at the first failure has run every other
test before it."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ERR_LEFT_DOMAIN = -11
STENCIL = {0: (2, 0, 1), 1: (4, 1, 1), 2: (3, 0, 2), 3: (4, 1, 1)}  # basis: width, low offset, nodes per cell


def _noalloc_mass(L, torch, x, m, g, dim, basis, stream=0):
    """One call on device copies of x (n x 3) and m; returns (status, nodal
    mass as FP64, message)."""
    xd = torch.tensor(np.ascontiguousarray(x, np.float32).ravel(), device="cuda")
    md = torch.tensor(np.ascontiguousarray(m, np.float32), device="cuda")
    out = torch.full((g.nnodes,), -1.0, dtype=torch.float32, device="cuda")
    lo = (ctypes.c_double * 3)(*[float(v) for v in g.lo])
    nn = (ctypes.c_int * 3)(g.nx, g.ny, g.nz)
    ng = (ctypes.c_int * 3)(g.nxg, g.nyg, g.nzg)
    err = ctypes.create_string_buffer(256)
    r = L.kmpm_p2g_mass_noalloc(xd.data_ptr(), md.data_ptr(), len(m), dim, basis, lo, g.cellsize, nn, ng,
                                out.data_ptr(), stream, err, 256)
    torch.cuda.synchronize()
    return r, out.cpu().numpy().astype(np.float64), err.value.decode()


def _ok(*a):
    r, out, msg = _noalloc_mass(*a)
    assert r == 0, msg
    return out


def _cpu_mass(x, m, g, dim, basis):
    """FP64 nodal mass on the CPU: Solid::compute_mass_nodes
    (src/solid.cpp:317-335) with the oracle's 1-D basis functions, over each
    particle's stencil (the cell of its position)."""
    import oracle as orc
    S, LO, SC = STENCIL[basis]
    n = [g.nx, g.ny, g.nz]
    ngl = [g.nxg, g.nyg, g.nzg]
    h = g.cellsize / SC
    np_ = len(m)
    idx = np.zeros((np_, 3, S), np.int64)
    val = np.ones((np_, 3, S))
    for d in range(3):
        if d >= dim:
            val[:, d, 1:] = 0.0
            continue
        c = np.floor((x[:, d] - g.lo[d]) / g.cellsize).astype(np.int64)
        for k in range(S):
            i = c * SC - LO + k
            ok = (i >= 0) & (i < n[d])
            ic = np.clip(i, 0, n[d] - 1)
            if basis in (1, 3):
                nt = np.minimum(2, ic) - np.minimum(ngl[d] - 1 - ic, 2)
            elif basis == 2:
                nt = ic & 1
            else:
                nt = np.zeros_like(ic)
            r = (x[:, d] - (g.lo[d] + ic * h)) / g.cellsize  # in cellsizes for every basis (src/tlmpm.cpp:274)
            s = np.array([orc.basis(basis, 0, float(rr), int(tt)) for rr, tt in zip(r, nt)])
            val[:, d, k] = np.where(ok, s, 0.0)
            idx[:, d, k] = ic
    out = np.zeros(g.nnodes)
    for a in range(S):
        for b in range(S):
            for cc in range(S):
                w = val[:, 0, a] * val[:, 1, b] * val[:, 2, cc]
                node = (idx[:, 0, a] * n[1] + idx[:, 1, b]) * n[2] + idx[:, 2, cc]
                np.add.at(out, node, w * m)
    return out


def _regular(dim, basis_name):
    """A TLMPM context built by the regular entry points, its solid and grid,
    and the nodal mass it computed (kmpm_download_grid)."""
    from karamelo_gb300 import workloads as W
    from karamelo_gb300.gpu import GpuBackend
    if dim == 3:
        sim = W.taylor_bar(None, cellsize=0.8, basis=basis_name)
    else:
        sim = W.spinning_disk(None, cellsize=0.025, method="tlmpm/gpu", sub="FLIP", basis=basis_name)
    be = GpuBackend(sim.s)
    be.run(0)  # builds the device state; TLMPM computes the nodal mass once
    ref = be.grid(0, "mass")
    assert ref.sum() > 0
    return sim.s.solids[0], sim.s.grids[0], ref


BASES = [("linear", 0), ("cubic-spline", 1), ("Bernstein-quadratic", 2), ("quadratic-spline", 3)]


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("basis_name,basis", BASES)
def test_noalloc_mass_matches_regular_path(gpu_lib, dim, basis_name, basis):
    import torch
    s, g, ref = _regular(dim, basis_name)
    # two calls in a row on the same scratch array: both equal the regular
    # path's nodal mass bit for bit (same sort, same scatter, same sums)
    for _ in range(2):
        got = _ok(gpu_lib, torch, s.x0, s.mass, g, dim, basis)
        assert np.array_equal(got, ref), f"max |diff| {np.max(np.abs(got - ref)):.3e}"


def test_noalloc_scratch_keeps_no_trace_of_the_previous_call(gpu_lib):
    import torch
    s, g, ref = _regular(3, "cubic-spline")
    full = _ok(gpu_lib, torch, s.x0, s.mass, g, 3, 1)
    assert np.array_equal(full, ref)
    # after a call that filled more tiles, a call on half of the particles
    # must see none of the previous ranges or partials
    half = slice(0, s.np // 2)
    got = _ok(gpu_lib, torch, s.x0[half], s.mass[half], g, 3, 1)
    want = _cpu_mass(s.x0[half], s.mass[half], g, 3, 1)
    assert np.max(np.abs(got - want)) <= 1e-6 * np.max(want)
    assert np.array_equal(got == 0, want == 0)
    # and the full set again after it
    assert np.array_equal(_ok(gpu_lib, torch, s.x0, s.mass, g, 3, 1), ref)


@pytest.mark.parametrize("basis", [0, 1, 2, 3])
def test_noalloc_mass_1d_matches_cpu_scatter(gpu_lib, basis):
    import torch
    from karamelo_gb300 import scenario as sc
    cellsize = 0.05
    g = sc.grid_geometry(1, basis, np.array([0.2, 0.0, 0.0]), np.array([0.8, 0.0, 0.0]),
                         np.array([1.0, 0.0, 0.0]), cellsize)
    rng = np.random.default_rng(basis)
    x = np.zeros((97, 3))
    x[:, 0] = rng.uniform(0.2, 0.8, 97)
    m = rng.uniform(0.5, 2.0, 97)
    want = _cpu_mass(x, m, g, 1, basis)
    for _ in range(2):
        got = _ok(gpu_lib, torch, x, m, g, 1, basis)
        assert np.max(np.abs(got - want)) <= 1e-6 * np.max(want)


def test_noalloc_reports_particles_outside_the_grid(gpu_lib):
    import torch
    s, g, ref = _regular(3, "cubic-spline")
    x = s.x0.copy()
    x[17, 0] = g.lo[0] - 2.0 * g.cellsize
    r, _, msg = _noalloc_mass(gpu_lib, torch, x, s.mass, g, 3, 1)
    assert r == ERR_LEFT_DOMAIN and "outside the grid" in msg
    x[17, 0] = np.nan
    r, _, msg = _noalloc_mass(gpu_lib, torch, x, s.mass, g, 3, 1)
    assert r == ERR_LEFT_DOMAIN
    # the next valid call is unaffected
    assert np.array_equal(_ok(gpu_lib, torch, s.x0, s.mass, g, 3, 1), ref)


def test_noalloc_rejects_oversized_problems(gpu_lib):
    import torch
    from karamelo_gb300 import scenario as sc
    n = 131072 + 1
    g = sc.GridSpec(lo=np.zeros(3), cellsize=1.0, h=1.0, nx=4, ny=4, nz=4, nxg=4, nyg=4, nzg=4)
    x = np.full((n, 3), 1.5)
    r, _, msg = _noalloc_mass(gpu_lib, torch, x, np.ones(n), g, 3, 1)
    assert r != 0 and "KMPM_NOALLOC_MAX_PARTICLES" in msg
    g2 = sc.GridSpec(lo=np.zeros(3), cellsize=1.0, h=1.0, nx=200, ny=200, nz=200, nxg=200, nyg=200, nzg=200)
    r, _, msg = _noalloc_mass(gpu_lib, torch, np.full((8, 3), 1.5), np.ones(8), g2, 3, 1)
    assert r != 0 and "KMPM_NOALLOC_MAX_CELLS" in msg
