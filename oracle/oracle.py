"""ctypes front end of the FP64 oracle (oracle/mpm_oracle.cpp).

TEST INFRASTRUCTURE ONLY: used by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of bench.py as the checker.  The product package never
imports this module.

``OracleBackend`` has the same interface as ``karamelo_gb300.gpu.GpuBackend``
(``run``, ``run_time``, ``add_fix``, ``particles``, ``grid``, ``scalars``,
``energies``) so a test can drive both from one script.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_basis.so")

PARTICLE_FIELDS = {"x": (0, 3), "x0": (1, 3), "v": (2, 3), "sigma_raw": (3, 9), "sigma": (4, 9), "F": (5, 9),
                   "eps_p": (6, 1), "epsdot_p": (7, 1), "damage": (8, 1), "damage_init": (9, 1), "T": (10, 1),
                   "J": (11, 1), "vol": (12, 1), "strain_el": (13, 9), "vol0PK1": (14, 9), "mass": (15, 1)}
GRID_FIELDS = {"mass": (0, 1), "v": (1, 3), "v_update": (2, 3), "x": (3, 3), "f": (4, 3), "mb": (5, 3), "T": (6, 1)}

_lib = None


def build(force=False):
    """Compile liboracle.so (and _ref/ when the reference tree is present)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "mpm_oracle.cpp")):
        subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])
    subprocess.call(["make", "-s", "-C", HERE, "ref"], stdout=subprocess.DEVNULL)


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        d, i, p = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        L.om_create.restype = p
        L.om_create.argtypes = [i, i, i, i, d, i, d, d, i, dp, dp]
        L.om_destroy.argtypes = [p]
        L.om_set_transfer.argtypes = [p, i]
        L.om_error.restype = ctypes.c_char_p
        L.om_error.argtypes = [p]
        L.om_add_material.argtypes = [p, p]
        L.om_add_grid.argtypes = [p, dp, dp, d]
        L.om_grid_info.argtypes = [p, i, ctypes.POINTER(ctypes.c_int), dp]
        L.om_grid_ntype.argtypes = [p, i, ctypes.POINTER(ctypes.c_int)]
        L.om_add_solid.argtypes = [p, i, i, i, dp, dp, dp, dp, d]
        L.om_add_fix.argtypes = [p, i, i, ctypes.POINTER(ctypes.c_uint8), ctypes.POINTER(ctypes.c_int), dp]
        L.om_run.argtypes = [p, i]
        L.om_run_time.argtypes = [p, d]
        L.om_scalars.argtypes = [p, dp]
        L.om_set_scalars.argtypes = [p, ctypes.c_double, ctypes.c_double]
        L.om_get_particles.argtypes = [p, i, i, dp]
        L.om_get_grid.argtypes = [p, i, i, dp]
        L.om_energy.argtypes = [p, dp]
        L.om_round_state_f32.argtypes = [p]
        L.om_basis.restype = d
        L.om_basis.argtypes = [i, i, d, i, d]
        L.om_constitutive.argtypes = [p, i, dp, dp, dp, dp]
        L.om_poldec.argtypes = [dp, dp]
        L.om_eig_real.argtypes = [dp, dp]
        L.om_set_threads.argtypes = [i]
        L.om_add_contact.argtypes = [p, i, i, i, d]
        L.om_set_axisymmetric.argtypes = [p, i]
        L.om_set_np_per_cell.argtypes = [p, i, i]
        L.om_contact_force.argtypes = [p, i, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class OracleError(RuntimeError):
    pass


class OracleBackend:
    """Runs a :class:`karamelo_gb300.scenario.Scenario` on the FP64 oracle."""

    def __init__(self, s, threads=0):
        L = lib()
        if threads:
            L.om_set_threads(threads)
        self.s = s
        lo = np.ascontiguousarray(s.boxlo, float)
        hi = np.ascontiguousarray(s.boxhi, float)
        self.h = L.om_create(s.method, s.scheme, s.basis, s.dim, s.pic_flip, int(s.thermal), s.dt, s.dt_factor,
                             int(s.dt_constant), _dp(lo), _dp(hi))
        self.L = L
        if getattr(s, "transfer", 0) != 0 and L.om_set_transfer(self.h, int(s.transfer)) != 0:
            raise RuntimeError(L.om_error(self.h).decode())
        if getattr(s, "axisymmetric", False) and L.om_set_axisymmetric(self.h, 1) != 0:
            raise RuntimeError(L.om_error(self.h).decode())
        for m in s.materials:
            L.om_add_material(self.h, ctypes.byref(m))
        # grids: the oracle restates Grid::init itself from the bounds
        self.grid_nn = []
        if s.method == 1:  # ULMPM: one grid over the box
            L.om_add_grid(self.h, _dp(lo), _dp(hi), s.grids[0].cellsize)
        else:
            for sol in s.solids:
                g = s.grids[sol.grid]
                glo = np.ascontiguousarray(g.lo, float)
                # solid bounds are the region limits that produced grid g
                ghi = np.ascontiguousarray(self._solid_hi(sol), float)
                L.om_add_grid(self.h, _dp(glo), _dp(ghi), g.cellsize)
        for gi in range(len(s.grids)):
            dims = (ctypes.c_int * 6)()
            loh = np.zeros(4)
            self.grid_nn.append(L.om_grid_info(self.h, gi, dims, _dp(loh)))
        for sol in s.solids:
            x0 = np.ascontiguousarray(sol.x0, float)
            v = np.ascontiguousarray(sol.v, float)
            m = np.ascontiguousarray(sol.mass, float)
            vo = np.ascontiguousarray(sol.vol0, float)
            si = L.om_add_solid(self.h, sol.grid, sol.mat, sol.np, _dp(x0), _dp(v), _dp(m), _dp(vo), sol.T0)
            if getattr(sol, "ppc", 0) and L.om_set_np_per_cell(self.h, si, int(sol.ppc)) != 0:
                raise RuntimeError(L.om_error(self.h).decode())
        for f in s.fixes:
            self.add_fix(f)
        for c in getattr(s, "contacts", []):
            self.add_contact(c)

    def _solid_hi(self, sol):
        return self.s.grids[sol.grid].hi

    def __del__(self):
        try:
            self.L.om_destroy(self.h)
        except Exception:
            pass

    def grid_info(self, gi):
        dims = (ctypes.c_int * 6)()
        loh = np.zeros(4)
        nn = self.L.om_grid_info(self.h, gi, dims, _dp(loh))
        return dict(nn=nn, dims=list(dims), lo=loh[:3].copy(), h=float(loh[3]))

    def grid_ntype(self, gi):
        out = np.zeros((self.grid_nn[gi], 3), dtype=np.int32)
        self.L.om_grid_ntype(self.h, gi, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        return out

    def add_fix(self, f):
        mask = np.ascontiguousarray(f.node_mask, np.uint8)
        st = (ctypes.c_int * 3)(*f.set)
        coef = np.ascontiguousarray(f.coef, float).ravel()
        self.L.om_add_fix(self.h, f.kind, f.grid, mask.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), st, _dp(coef))

    def add_contact(self, c):
        return self.L.om_add_contact(self.h, c.kind, c.solid1, c.solid2, c.mu)

    def contact_force(self, k):
        out = np.zeros(3)
        self.L.om_contact_force(self.h, int(k), _dp(out))
        return out

    def run(self, n):
        if self.L.om_run(self.h, int(n)) != 0:
            raise OracleError(self.L.om_error(self.h).decode())

    def run_time(self, t):
        r = self.L.om_run_time(self.h, self.scalars()[0] + float(t))
        if r < 0:
            raise OracleError(self.L.om_error(self.h).decode())
        return r

    def scalars(self):
        out = np.zeros(3)
        self.L.om_scalars(self.h, _dp(out))
        return out[0], out[1], int(out[2])

    def set_scalars(self, time, dt, ntimestep=None):
        """Set the clock (the next step runs with this dt); the signature of
        GpuBackend.set_scalars, whose step counter the oracle keeps itself."""
        self.L.om_set_scalars(self.h, float(time), float(dt))

    def particles(self, si, field):
        code, w = PARTICLE_FIELDS[field]
        n = self.s.solids[si].np
        out = np.zeros(n * w)
        self.L.om_get_particles(self.h, si, code, _dp(out))
        return out.reshape(n, 3, 3) if w == 9 else (out.reshape(n, 3) if w == 3 else out)

    def grid(self, gi, field):
        code, w = GRID_FIELDS[field]
        out = np.zeros(self.grid_nn[gi] * w)
        self.L.om_get_grid(self.h, gi, code, _dp(out))
        return out.reshape(-1, 3) if w == 3 else out

    def round_state_f32(self):
        """Particle state rounded to single precision (sensitivity-floor runs)."""
        self.L.om_round_state_f32(self.h)

    def energies(self):
        out = np.zeros(2)
        self.L.om_energy(self.h, _dp(out))
        return float(out[0]), float(out[1])


def basis(basis, kind, r, ntype, icellsize=1.0):
    return lib().om_basis(basis, kind, float(r), int(ntype), float(icellsize))


def ref_basis_lib():
    """The reference's own basis functions (oracle/_ref), present only where the
    reference tree was available to compile them."""
    if not os.path.exists(REF_LIB):
        return None
    L = ctypes.CDLL(REF_LIB)
    L.ref_basis.restype = ctypes.c_double
    L.ref_basis.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double]
    return L
