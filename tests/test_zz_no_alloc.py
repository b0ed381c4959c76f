"""kmpm_p2g_mass_noalloc: the nodal-mass scatter for callers that cannot
allocate device memory (code running during CUDA-graph capture, or hosts
whose device memory belongs to their own pool).  Its output is checked,
through the C ABI, against the nodal mass that the regular entry points
compute (kmpm_run then kmpm_download_grid), on two calls in a row.  This file
is collected last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc_mass(L, torch, x, m, g, stream=0):
    xd = torch.tensor(np.ascontiguousarray(x, np.float32).ravel(), device="cuda")
    md = torch.tensor(np.ascontiguousarray(m, np.float32), device="cuda")
    out = torch.full((g.nnodes,), -1.0, dtype=torch.float32, device="cuda")
    lo = (ctypes.c_double * 3)(*[float(v) for v in g.lo])
    nn = (ctypes.c_int * 3)(g.nx, g.ny, g.nz)
    ng = (ctypes.c_int * 3)(g.nxg, g.nyg, g.nzg)
    err = ctypes.create_string_buffer(256)
    r = L.kmpm_p2g_mass_noalloc(xd.data_ptr(), md.data_ptr(), len(m), 3, 1, lo, g.cellsize, nn, ng, out.data_ptr(),
                                stream, err, 256)
    assert r == 0, err.value.decode()
    torch.cuda.synchronize()
    return out.cpu().numpy().astype(np.float64)


def test_noalloc_mass_matches_regular_path(gpu_lib):
    import torch
    from karamelo_gb300 import workloads as W
    from karamelo_gb300.gpu import GpuBackend

    sim = W.taylor_bar(None, cellsize=0.8)
    s = sim.s.solids[0]
    g = sim.s.grids[0]
    be = GpuBackend(sim.s)
    be.run(0)  # builds the device state; TLMPM computes the nodal mass once
    ref = be.grid(0, "mass")
    assert ref.sum() > 0
    # two calls in a row on the same scratch: both must match
    for _ in range(2):
        got = _noalloc_mass(gpu_lib, torch, s.x0, s.mass, g)
        np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-12 * ref.max())
    # a different particle set in between must not leave traces in the scratch
    half = slice(0, s.np // 2)
    _noalloc_mass(gpu_lib, torch, s.x0[half], s.mass[half], g)
    got = _noalloc_mass(gpu_lib, torch, s.x0, s.mass, g)
    np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-12 * ref.max())


def test_noalloc_rejects_oversized_problems(gpu_lib):
    import torch
    from karamelo_gb300 import scenario as sc
    n = 131072 + 1
    g = sc.GridSpec(lo=np.zeros(3), cellsize=1.0, h=1.0, nx=4, ny=4, nz=4, nxg=4, nyg=4, nzg=4)
    x = np.full((n, 3), 1.5)
    with pytest.raises(AssertionError, match="KMPM_NOALLOC_MAX_PARTICLES"):
        _noalloc_mass(gpu_lib, torch, x, np.ones(n), g)
    g2 = sc.GridSpec(lo=np.zeros(3), cellsize=1.0, h=1.0, nx=200, ny=200, nz=200, nxg=200, nyg=200, nzg=200)
    with pytest.raises(AssertionError, match="KMPM_NOALLOC_MAX_CELLS"):
        _noalloc_mass(gpu_lib, torch, np.full((8, 3), 1.5), np.ones(8), g2)
