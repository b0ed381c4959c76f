"""Independent TLMPM runs executed together on one GPU.

A parameter sweep in Karamelo is many separate runs of one script (one process
each).  :class:`Batch` takes several :class:`~karamelo_gb300.model.MPM`
scripts that share the method, scheme, basis and dimension, merges their
materials, grids, solids and fixes into one device state, and runs them with
``kmpm_params.independent``: every phase of the step is one launch over all
instances, the whole step is one captured CUDA graph, and every instance
keeps its own dt and time (its own ``adjust_dt`` / ``update_time``), exactly
as if it ran alone.
"""
from __future__ import annotations

import copy
from typing import List

import numpy as np

from . import scenario as sc
from .model import KarameloError


class Batch:
    def __init__(self, sims, backend_factory=None, **backend_kw):
        if not sims:
            raise KarameloError("empty batch")
        first = sims[0].s
        if first.method != sc.TLMPM:
            raise KarameloError("independent runs need TLMPM (ULMPM solids share one grid)")
        merged = sc.Scenario(method=first.method, scheme=first.scheme, basis=first.basis, dim=first.dim,
                             pic_flip=first.pic_flip, thermal=first.thermal, dt=first.dt, dt_factor=first.dt_factor,
                             dt_constant=first.dt_constant, boxlo=first.boxlo.copy(), boxhi=first.boxhi.copy())
        self.solid_index: List[List[int]] = []
        for sim in sims:
            s = sim.s
            for key in ("method", "scheme", "basis", "dim", "pic_flip", "thermal", "dt", "dt_factor", "dt_constant"):
                if getattr(s, key) != getattr(first, key):
                    raise KarameloError(f"batched runs must share {key}")
            m0, g0, s0 = len(merged.materials), len(merged.grids), len(merged.solids)
            merged.materials.extend(s.materials)
            merged.grids.extend(s.grids)
            idx = []
            for sol in s.solids:
                ns = copy.copy(sol)
                ns.grid, ns.mat = sol.grid + g0, sol.mat + m0
                merged.solids.append(ns)
                idx.append(len(merged.solids) - 1)
            for f in s.fixes:
                nf = copy.copy(f)
                nf.grid = f.grid + g0
                merged.fixes.append(nf)
            self.solid_index.append(idx)
        self.scenario = merged
        self.n = len(sims)
        if backend_factory is None:
            from .gpu import GpuBackend
            self.backend = GpuBackend(merged, independent=True, **backend_kw)
        else:
            self.backend = backend_factory(merged)

    @property
    def total_particles(self) -> int:
        return self.scenario.total_particles

    def run(self, n: int):
        self.backend.run(int(n))

    def particles(self, instance: int, field: str, solid: int = 0):
        return self.backend.particles(self.solid_index[instance][solid], field)

    def scalars(self, instance: int):
        """(time, dt, step) of one instance."""
        return self.backend.solid_scalars(self.solid_index[instance][0])


def tensile_sweep(n, seed=0, nmin=2000, nmax=64000, vmin=1.0, vmax=20.0, spread=0.3, build=None, **kw):
    """A seeded parameter sweep: n 2-D TLMPM tensile bars (aspect ratio
    5:1, 2x2 particles per cell) with Johnson-Cook strength and damage, the
    damage constants D1..D5 drawn uniformly within +-spread of their nominal
    values, particle counts log-uniform in [nmin, nmax] (through the cell
    size) and end speeds uniform in [vmin, vmax] m/s.  Seeded."""
    from .workloads import DAMAGE, tensile_bar_2d
    rng = np.random.default_rng(seed)
    hLx, hLy = 10.0, 2.0
    sims, params = [], []
    for _ in range(n):
        npart = float(np.exp(rng.uniform(np.log(nmin), np.log(nmax))))
        # 4 * (2 hLx / h) * (2 hLy / h) particles  ->  h
        h = float(np.sqrt(4 * (2 * hLx) * (2 * hLy) / npart))
        d = {k: v * rng.uniform(1 - spread, 1 + spread) for k, v in DAMAGE.items()}
        v = float(rng.uniform(vmin, vmax))
        sims.append((build or tensile_bar_2d)(cellsize=h, hLx=hLx, hLy=hLy, vend=v, damage=d, ramp=False, **kw))
        params.append(dict(cellsize=h, vend=v, damage=d))
    return sims, params
