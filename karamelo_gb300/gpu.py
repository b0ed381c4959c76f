"""ctypes driver of libkmpm.so (include/kmpm.h) for a :class:`Scenario`.

This is the Python side of the drop-in boundary: it makes exactly the calls a
Karamelo ``tlmpm/gpu`` / ``ulmpm/gpu`` method style makes from C++.  There is no fallback: if the library or a CUDA device is
missing, construction raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import scenario as sc

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libkmpm.so")

KMPM_OK = 0
ERRORS = {-1: "KMPM_ERR_ARG", -2: "KMPM_ERR_CUDA", -3: "KMPM_ERR_STATE", -10: "KMPM_ERR_J",
          -11: "KMPM_ERR_LEFT_DOMAIN", -12: "KMPM_ERR_NAN", -13: "KMPM_ERR_POLDEC", -14: "KMPM_ERR_DTCFL"}

PARTICLE_FIELDS = {"x": (0, 3), "x0": (1, 3), "v": (2, 3), "sigma_raw": (3, 9), "sigma": (4, 9), "F": (5, 9),
                   "eps_p": (6, 1), "epsdot_p": (7, 1), "damage": (8, 1), "damage_init": (9, 1), "T": (10, 1),
                   "J": (11, 1), "vol": (12, 1), "strain_el": (13, 9), "mass": (15, 1)}
GRID_FIELDS = {"mass": (0, 1), "v": (1, 3), "v_update": (2, 3), "x": (3, 3), "T": (6, 1)}

EXPORTED = ["kmpm_create", "kmpm_destroy", "kmpm_last_error", "kmpm_add_material", "kmpm_add_grid",
            "kmpm_add_solid", "kmpm_add_fix", "kmpm_run", "kmpm_run_time", "kmpm_scalars",
            "kmpm_download_particles", "kmpm_upload_particles", "kmpm_download_grid", "kmpm_energy",
            "kmpm_stream", "kmpm_launches_per_step", "kmpm_profile", "kmpm_profile_phase",
            "kmpm_p2g_mass_noalloc", "kmpm_solid_scalars"]


class KmpmParams(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int), ("scheme", ctypes.c_int), ("basis", ctypes.c_int), ("dim", ctypes.c_int),
                ("pic_flip", ctypes.c_double), ("thermal", ctypes.c_int), ("dt", ctypes.c_double),
                ("dt_factor", ctypes.c_double), ("dt_constant", ctypes.c_int), ("boxlo", ctypes.c_double * 3),
                ("boxhi", ctypes.c_double * 3), ("precision", ctypes.c_int), ("sort_every", ctypes.c_int),
                ("track_strain", ctypes.c_int), ("independent", ctypes.c_int)]


class KmpmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def load(path: str = LIB_PATH):
    """Load libkmpm.so; raises if it has not been built (no fallback path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libkmpm.so not built at {path}: run karamelo_gb300.build.build()")
    L = ctypes.CDLL(path)
    p, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    L.kmpm_create.argtypes = [ctypes.POINTER(KmpmParams), ctypes.POINTER(p)]
    L.kmpm_destroy.argtypes = [p]
    L.kmpm_last_error.restype = ctypes.c_char_p
    L.kmpm_last_error.argtypes = [p]
    L.kmpm_add_material.argtypes = [p, ctypes.POINTER(sc.MaterialParams)]
    L.kmpm_add_grid.argtypes = [p, dp, d, ip, ip]
    L.kmpm_add_solid.argtypes = [p, i, i, i, dp, dp, dp, dp, dp, d]
    L.kmpm_add_fix.argtypes = [p, i, i, ctypes.POINTER(ctypes.c_ubyte), ip, dp]
    L.kmpm_run.argtypes = [p, i]
    L.kmpm_run_time.argtypes = [p, d, ip]
    L.kmpm_scalars.argtypes = [p, dp, dp, ctypes.POINTER(ctypes.c_longlong)]
    L.kmpm_solid_scalars.argtypes = [p, i, dp, dp, ctypes.POINTER(ctypes.c_longlong)]
    L.kmpm_download_particles.argtypes = [p, i, i, dp]
    L.kmpm_upload_particles.argtypes = [p, i, i, dp]
    L.kmpm_download_grid.argtypes = [p, i, i, dp]
    L.kmpm_energy.argtypes = [p, dp]
    L.kmpm_stream.restype = p
    L.kmpm_stream.argtypes = [p]
    L.kmpm_launches_per_step.argtypes = [p]
    L.kmpm_profile.argtypes = [p, i, dp, i, ip]
    L.kmpm_profile_phase.restype = ctypes.c_char_p
    L.kmpm_profile_phase.argtypes = [p, i]
    fp = ctypes.c_void_p
    L.kmpm_p2g_mass_noalloc.argtypes = [fp, fp, i, i, i, dp, d, ip, ip, fp, p, ctypes.c_char_p, i]
    _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class GpuBackend:
    """Runs a Scenario on the GPU through the C ABI."""

    def __init__(self, s: sc.Scenario, precision: int = 0, track_strain: bool = True, independent: bool = False):
        L = load()
        self.L, self.s = L, s
        prm = KmpmParams()
        prm.method, prm.scheme, prm.basis, prm.dim = s.method, s.scheme, s.basis, s.dim
        prm.pic_flip, prm.thermal = s.pic_flip, int(s.thermal)
        prm.dt, prm.dt_factor, prm.dt_constant = s.dt, s.dt_factor, int(s.dt_constant)
        for k in range(3):
            prm.boxlo[k], prm.boxhi[k] = float(s.boxlo[k]), float(s.boxhi[k])
        prm.precision = precision
        prm.sort_every = 1
        prm.track_strain = int(track_strain)
        prm.independent = int(independent)
        h = ctypes.c_void_p()
        r = L.kmpm_create(ctypes.byref(prm), ctypes.byref(h))
        if r != KMPM_OK:
            raise KmpmError(r, "kmpm_create failed (no CUDA device?)")
        self.h = h
        for m in s.materials:
            self._ck(L.kmpm_add_material(h, ctypes.byref(m)), allow_id=True)
        for g in s.grids:
            lo = np.ascontiguousarray(g.lo, float)
            n = (ctypes.c_int * 3)(g.nx, g.ny, g.nz)
            ng = (ctypes.c_int * 3)(g.nxg, g.nyg, g.nzg)
            self._ck(L.kmpm_add_grid(h, _dp(lo), g.cellsize, n, ng), allow_id=True)
        for sol in s.solids:
            x0 = np.ascontiguousarray(sol.x0, float)
            v = np.ascontiguousarray(sol.v, float)
            m = np.ascontiguousarray(sol.mass, float)
            vo = np.ascontiguousarray(sol.vol0, float)
            self._ck(L.kmpm_add_solid(h, sol.grid, sol.mat, sol.np, _dp(x0), _dp(x0), _dp(v), _dp(m), _dp(vo),
                                      sol.T0), allow_id=True)
        for f in s.fixes:
            self.add_fix(f)

    def _ck(self, r, allow_id=False):
        if r < 0 or (r != KMPM_OK and not allow_id):
            raise KmpmError(r, self.L.kmpm_last_error(self.h).decode())
        return r

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.L.kmpm_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def add_fix(self, f: sc.FixSpec):
        mask = np.ascontiguousarray(f.node_mask, np.uint8)
        st = (ctypes.c_int * 3)(*f.set)
        coef = np.ascontiguousarray(f.coef, float).ravel()
        self._ck(self.L.kmpm_add_fix(self.h, f.kind, f.grid, mask.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)),
                                     st, _dp(coef)), allow_id=True)

    def run(self, n: int):
        self._ck(self.L.kmpm_run(self.h, int(n)))

    def run_time(self, t: float) -> int:
        done = ctypes.c_int(0)
        self._ck(self.L.kmpm_run_time(self.h, self.scalars()[0] + float(t), ctypes.byref(done)))
        return done.value

    def scalars(self):
        t, dt, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        self._ck(self.L.kmpm_scalars(self.h, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(n)))
        return t.value, dt.value, n.value

    def solid_scalars(self, si: int):
        t, dt, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        self._ck(self.L.kmpm_solid_scalars(self.h, si, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(n)))
        return t.value, dt.value, n.value

    def particles(self, si: int, field: str):
        code, w = PARTICLE_FIELDS[field]
        n = self.s.solids[si].np
        out = np.zeros(n * w)
        self._ck(self.L.kmpm_download_particles(self.h, si, code, _dp(out)))
        return out.reshape(n, 3, 3) if w == 9 else (out.reshape(n, 3) if w == 3 else out)

    def upload_velocity(self, si: int, v):
        v = np.ascontiguousarray(v, float)
        self._ck(self.L.kmpm_upload_particles(self.h, si, 2, _dp(v)))

    def grid(self, gi: int, field: str):
        code, w = GRID_FIELDS[field]
        g = self.s.grids[gi]
        out = np.zeros(g.nnodes * w)
        self._ck(self.L.kmpm_download_grid(self.h, gi, code, _dp(out)))
        return out.reshape(-1, 3) if w == 3 else out

    def energies(self):
        out = np.zeros(2)
        self._ck(self.L.kmpm_energy(self.h, _dp(out)))
        return float(out[0]), float(out[1])

    def stream(self):
        return self.L.kmpm_stream(self.h)

    def launches_per_step(self):
        return self.L.kmpm_launches_per_step(self.h)

    def profile(self, nsteps: int):
        """Mean device time (ms) of every phase of a step, from CUDA events on
        the library's stream (eager launches, not the captured graph)."""
        out = np.zeros(32)
        n = ctypes.c_int(0)
        self._ck(self.L.kmpm_profile(self.h, int(nsteps), _dp(out), 32, ctypes.byref(n)))
        return {self.L.kmpm_profile_phase(self.h, k).decode(): float(out[k]) for k in range(n.value)}
