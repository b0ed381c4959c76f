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
                   "J": (11, 1), "vol": (12, 1), "strain_el": (13, 9), "vol0PK1": (14, 9), "mass": (15, 1),
                   "sigma6": (16, 6)}
# the particle state Solid::read_restart restores (src/solid.cpp:2894-2957)
RESTART_FIELDS_TL = ("x", "v", "sigma_raw", "strain_el", "vol0PK1", "F", "eps_p", "epsdot_p", "damage",
                     "damage_init")
RESTART_FIELDS_UL = ("x", "v", "sigma_raw", "strain_el", "F", "eps_p", "epsdot_p", "damage", "damage_init")
GRID_FIELDS = {"mass": (0, 1), "v": (1, 3), "v_update": (2, 3), "x": (3, 3), "T": (6, 1)}

EXPORTED = ["kmpm_create", "kmpm_destroy", "kmpm_last_error", "kmpm_add_material", "kmpm_add_grid",
            "kmpm_add_solid", "kmpm_add_fix", "kmpm_run", "kmpm_run_async", "kmpm_sync", "kmpm_run_time", "kmpm_run_until", "kmpm_scalars",
            "kmpm_download_particles", "kmpm_upload_particles", "kmpm_download_grid", "kmpm_energy",
            "kmpm_stream", "kmpm_launches_per_step", "kmpm_profile", "kmpm_profile_phase",
            "kmpm_p2g_mass_noalloc", "kmpm_solid_scalars",
            "kmpm_mlp_create", "kmpm_mlp_destroy", "kmpm_mlp_last_error", "kmpm_mlp_init", "kmpm_mlp_set_params",
            "kmpm_mlp_get_params", "kmpm_mlp_set_norm", "kmpm_mlp_get_norm", "kmpm_mlp_loss_grad", "kmpm_mlp_train",
            "kmpm_mlp_predict", "kmpm_mlp_predict_tc", "kmpm_log_start", "kmpm_log_stop", "kmpm_log_data",
            "kmpm_jc_label", "kmpm_set_surrogate", "kmpm_surrogate_stats", "kmpm_tuning",
            "kmpm_download_particles_async", "kmpm_sync_downloads", "kmpm_wait_download", "kmpm_add_contact", "kmpm_contact_force",
            "kmpm_set_scalars", "kmpm_state_size", "kmpm_save_state", "kmpm_load_state", "kmpm_set_np_per_cell"]

MLP_NIN, MLP_NOUT, MLP_NPARAMS, MLP_NNORM = 15, 7, 35975, 74


class KmpmParams(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int), ("scheme", ctypes.c_int), ("basis", ctypes.c_int), ("dim", ctypes.c_int),
                ("pic_flip", ctypes.c_double), ("thermal", ctypes.c_int), ("dt", ctypes.c_double),
                ("dt_factor", ctypes.c_double), ("dt_constant", ctypes.c_int), ("boxlo", ctypes.c_double * 3),
                ("boxhi", ctypes.c_double * 3), ("precision", ctypes.c_int),
                ("track_strain", ctypes.c_int), ("independent", ctypes.c_int), ("autotune", ctypes.c_int),
                ("transfer", ctypes.c_int), ("axisymmetric", ctypes.c_int)]


class TrainOpts(ctypes.Structure):
    _fields_ = [("batch", ctypes.c_int), ("steps", ctypes.c_longlong), ("lr", ctypes.c_double),
                ("lr_final_ratio", ctypes.c_double), ("seed", ctypes.c_ulonglong), ("report_every", ctypes.c_int)]


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
    L.kmpm_run_async.argtypes = [p, i]
    L.kmpm_sync.argtypes = [p]
    L.kmpm_run_time.argtypes = [p, d, ip]
    L.kmpm_run_until.argtypes = [p, i, d, ip]
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
    ll, ull = ctypes.c_longlong, ctypes.c_ulonglong
    f32p = ctypes.POINTER(ctypes.c_float)
    L.kmpm_mlp_create.argtypes = [i, ctypes.POINTER(p)]
    L.kmpm_mlp_destroy.argtypes = [p]
    L.kmpm_mlp_destroy.restype = None
    L.kmpm_mlp_last_error.argtypes = [p]
    L.kmpm_mlp_last_error.restype = ctypes.c_char_p
    L.kmpm_mlp_init.argtypes = [p, ull]
    L.kmpm_mlp_set_params.argtypes = [p, f32p]
    L.kmpm_mlp_get_params.argtypes = [p, f32p]
    L.kmpm_mlp_set_norm.argtypes = [p, f32p]
    L.kmpm_mlp_get_norm.argtypes = [p, f32p]
    L.kmpm_mlp_loss_grad.argtypes = [p, fp, fp, i, f32p, f32p]
    L.kmpm_mlp_train.argtypes = [p, fp, fp, ll, ctypes.POINTER(TrainOpts), f32p]
    L.kmpm_mlp_predict.argtypes = [p, fp, ll, fp]
    L.kmpm_mlp_predict_tc.argtypes = [p, fp, ll, fp, fp]
    L.kmpm_log_start.argtypes = [p, ll, d, ull]
    L.kmpm_log_stop.argtypes = [p]
    L.kmpm_log_data.argtypes = [p, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ll)]
    L.kmpm_jc_label.argtypes = [p, i, fp, ll, fp]
    L.kmpm_set_surrogate.argtypes = [p, p, d]
    L.kmpm_surrogate_stats.argtypes = [p, ctypes.POINTER(ll)]
    L.kmpm_tuning.argtypes = [p]
    L.kmpm_download_particles_async.argtypes = [p, i, i, fp]
    L.kmpm_sync_downloads.argtypes = [p]
    L.kmpm_wait_download.argtypes = [p, ctypes.c_void_p]
    L.kmpm_tuning.restype = ctypes.c_char_p
    L.kmpm_add_contact.argtypes = [p, i, i, i, d]
    L.kmpm_contact_force.argtypes = [p, i, dp]
    L.kmpm_set_scalars.argtypes = [p, d, d, ll]
    L.kmpm_set_np_per_cell.argtypes = [p, i, i]
    L.kmpm_state_size.argtypes = [p, ctypes.POINTER(ull)]
    L.kmpm_save_state.argtypes = [p, ctypes.c_void_p, ull]
    L.kmpm_load_state.argtypes = [p, ctypes.c_void_p, ull]
    _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class GpuBackend:
    """Runs a Scenario on the GPU through the C ABI."""

    def __init__(self, s: sc.Scenario, precision: int = 0, track_strain: bool = True, independent: bool = False,
                 autotune: bool = True):
        L = load()
        self.L, self.s = L, s
        prm = KmpmParams()
        prm.method, prm.scheme, prm.basis, prm.dim = s.method, s.scheme, s.basis, s.dim
        prm.pic_flip, prm.thermal = s.pic_flip, int(s.thermal)
        prm.dt, prm.dt_factor, prm.dt_constant = s.dt, s.dt_factor, int(s.dt_constant)
        for k in range(3):
            prm.boxlo[k], prm.boxhi[k] = float(s.boxlo[k]), float(s.boxhi[k])
        prm.precision = precision
        prm.track_strain = int(track_strain)
        prm.independent = int(independent)
        prm.autotune = int(autotune)
        prm.transfer = int(getattr(s, "transfer", 0))
        prm.axisymmetric = int(getattr(s, "axisymmetric", False))
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
            si = self._ck(L.kmpm_add_solid(h, sol.grid, sol.mat, sol.np, _dp(x0), _dp(x0), _dp(v), _dp(m), _dp(vo),
                                           sol.T0), allow_id=True)
            if getattr(sol, "ppc", 0):
                self._ck(L.kmpm_set_np_per_cell(h, si, int(sol.ppc)))
        for f in s.fixes:
            self.add_fix(f)
        for c in s.contacts:
            self.add_contact(c)

    def _ck(self, r, allow_id=False):
        if r < 0 or (r != KMPM_OK and not allow_id):
            raise KmpmError(r, self.L.kmpm_last_error(self.h).decode())
        return r

    def close(self):
        """Free the context and its device memory now (kmpm_destroy), not
        whenever the garbage collector reaches this object."""
        if getattr(self, "h", None):
            self.L.kmpm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_fix(self, f: sc.FixSpec):
        mask = np.ascontiguousarray(f.node_mask, np.uint8)
        st = (ctypes.c_int * 3)(*f.set)
        coef = np.ascontiguousarray(f.coef, float).ravel()
        self._ck(self.L.kmpm_add_fix(self.h, f.kind, f.grid, mask.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)),
                                     st, _dp(coef)), allow_id=True)

    def add_contact(self, c: sc.ContactSpec) -> int:
        return self._ck(self.L.kmpm_add_contact(self.h, c.kind, c.solid1, c.solid2, c.mu), allow_id=True)

    def contact_force(self, k: int):
        out = np.zeros(3)
        self._ck(self.L.kmpm_contact_force(self.h, int(k), _dp(out)))
        return out

    def run(self, n: int):
        self._ck(self.L.kmpm_run(self.h, int(n)))

    def run_async(self, n: int):
        """Queue n steps and return (kmpm_run_async); :meth:`sync` waits for
        them and raises the first error they met."""
        self._ck(self.L.kmpm_run_async(self.h, int(n)))

    def sync(self):
        self._ck(self.L.kmpm_sync(self.h))

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
        return out.reshape(n, 3, 3) if w == 9 else (out.reshape(n, w) if w in (3, 6) else out)

    def particles_async(self, si: int, field: str, out):
        """Queue the download of one field into ``out``, a page-locked float64
        torch tensor of n*width values (torch.empty(..., pin_memory=True));
        valid after :meth:`sync_downloads`."""
        code, w = PARTICLE_FIELDS[field]
        assert out.dtype.is_floating_point and out.element_size() == 8 and out.is_pinned()
        assert out.numel() == self.s.solids[si].np * w
        self._ck(self.L.kmpm_download_particles_async(self.h, si, code, out.data_ptr()))

    def sync_downloads(self):
        self._ck(self.L.kmpm_sync_downloads(self.h))

    def wait_download(self, out):
        """Wait for the last download queued into ``out`` only."""
        self._ck(self.L.kmpm_wait_download(self.h, out.data_ptr()))

    def upload_velocity(self, si: int, v):
        v = np.ascontiguousarray(v, float)
        self._ck(self.L.kmpm_upload_particles(self.h, si, 2, _dp(v)))

    def upload(self, si: int, field: str, values):
        """Upload one particle field (the layout ``particles`` returns)."""
        code, w = PARTICLE_FIELDS[field]
        a = np.ascontiguousarray(values, float).reshape(-1)
        assert a.size == self.s.solids[si].np * w
        self._ck(self.L.kmpm_upload_particles(self.h, si, code, _dp(a)))

    def set_scalars(self, time: float, dt: float, ntimestep: int):
        self._ck(self.L.kmpm_set_scalars(self.h, float(time), float(dt), int(ntimestep)))

    # ---- restart (Solid::write_restart / read_restart, src/solid.cpp:2841-2957)
    def restart_state(self):
        """The per-particle state a restart file carries, as FP64 arrays per
        solid, with the clock (time, dt, ntimestep)."""
        names = RESTART_FIELDS_TL if self.s.method == sc.TLMPM else RESTART_FIELDS_UL
        extra = ("T",) if self.s.thermal else ()
        return {"scalars": self.scalars(),
                "solids": [{f: self.particles(si, f) for f in names + extra} for si in range(len(self.s.solids))]}

    def restore_state(self, st):
        """Restore ``restart_state`` into a context made by the same setup."""
        self.run(0)  # builds the context
        for si, fields in enumerate(st["solids"]):
            for f, a in fields.items():
                self.upload(si, f, a)
        t, dt, n = st["scalars"]
        self.set_scalars(t, dt, n)

    # ---- device snapshot (bit-exact checkpoint of the whole device state)
    def save_state(self) -> bytes:
        n = ctypes.c_ulonglong()
        self._ck(self.L.kmpm_state_size(self.h, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value)
        self._ck(self.L.kmpm_save_state(self.h, buf, n.value))
        return buf.raw

    def load_state(self, blob: bytes):
        buf = ctypes.create_string_buffer(blob, len(blob))
        self._ck(self.L.kmpm_load_state(self.h, buf, len(blob)))

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

    def tuning(self):
        """The autotuner's record (launch shapes tried, their ms, the choice)."""
        import json
        return json.loads(self.L.kmpm_tuning(self.h).decode())

    # ---- learned return map (training pairs, surrogate)
    def log_start(self, capacity: int, fraction: float, seed: int = 0):
        self._ck(self.L.kmpm_log_start(self.h, int(capacity), float(fraction), int(seed)))

    def log_stop(self):
        self._ck(self.L.kmpm_log_stop(self.h))

    def log_data(self):
        """The logged pairs as a CUDA tensor [n, 22] (a copy: inputs then outputs)."""
        import torch
        ptr, n = ctypes.c_void_p(), ctypes.c_longlong()
        self._ck(self.L.kmpm_log_data(self.h, ctypes.byref(ptr), ctypes.byref(n)))
        if n.value == 0:
            return torch.zeros((0, MLP_NIN + MLP_NOUT), dtype=torch.float32, device="cuda")
        return device_view(ptr.value, (n.value, MLP_NIN + MLP_NOUT)).clone()

    def jc_label(self, material: int, X):
        """Closed-form return map of one material on input rows X (CUDA
        float32 [n, 15]): [n, 8] = 7 outputs and the plastic flag."""
        import torch
        X = X.contiguous()
        Y = torch.empty((X.shape[0], MLP_NOUT + 1), dtype=torch.float32, device=X.device)
        torch.cuda.synchronize()
        self._ck(self.L.kmpm_jc_label(self.h, int(material), X.data_ptr(), X.shape[0], Y.data_ptr()))
        return Y

    def set_surrogate(self, mlp, tol: float = 1e-3):
        self._ck(self.L.kmpm_set_surrogate(self.h, mlp.h if mlp is not None else None, float(tol)))

    def surrogate_stats(self):
        out = (ctypes.c_longlong * 4)()
        self._ck(self.L.kmpm_surrogate_stats(self.h, out))
        return dict(plastic=out[0], network=out[1], outside=out[2], residual=out[3])

    def profile(self, nsteps: int):
        """Mean device time (ms) of every phase of a step, from CUDA events on
        the library's stream (eager launches, not the captured graph)."""
        out = np.zeros(32)
        n = ctypes.c_int(0)
        self._ck(self.L.kmpm_profile(self.h, int(nsteps), _dp(out), 32, ctypes.byref(n)))
        return {self.L.kmpm_profile_phase(self.h, k).decode(): float(out[k]) for k in range(n.value)}


class _CudaArray:
    def __init__(self, ptr, shape):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": "<f4", "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def device_view(ptr, shape):
    """A torch view (no copy) of a float32 device array owned by the library."""
    import torch
    return torch.as_tensor(_CudaArray(ptr, shape), device="cuda")


class Mlp:
    """The learned return map's network (kmpm_mlp_*): FP32 training on the
    GPU, FP32 and tensor-core inference.  X / Y are CUDA float32 tensors in
    physical units ([n, 15] / [n, 7])."""

    def __init__(self, batch: int = 8192, seed: int = 0):
        L = load()
        self.L = L
        h = ctypes.c_void_p()
        r = L.kmpm_mlp_create(int(batch), ctypes.byref(h))
        if r != KMPM_OK:
            raise KmpmError(r, "kmpm_mlp_create failed (no CUDA device?)")
        self.h = h
        self.batch = batch
        self._ck(L.kmpm_mlp_init(h, int(seed)))

    def _ck(self, r):
        if r != KMPM_OK:
            raise KmpmError(r, self.L.kmpm_mlp_last_error(self.h).decode())

    def __del__(self):
        if getattr(self, "h", None):
            self.L.kmpm_mlp_destroy(self.h)
            self.h = None

    @staticmethod
    def _f32(a):
        a = np.ascontiguousarray(a, np.float32)
        return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))

    def init(self, seed: int):
        self._ck(self.L.kmpm_mlp_init(self.h, int(seed)))

    @property
    def params(self):
        out = np.empty(MLP_NPARAMS, np.float32)
        self._ck(self.L.kmpm_mlp_get_params(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return out

    @params.setter
    def params(self, v):
        a, ptr = self._f32(v)
        assert a.size == MLP_NPARAMS
        self._ck(self.L.kmpm_mlp_set_params(self.h, ptr))

    @property
    def norm(self):
        out = np.empty(MLP_NNORM, np.float32)
        self._ck(self.L.kmpm_mlp_get_norm(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return out

    @norm.setter
    def norm(self, v):
        a, ptr = self._f32(v)
        assert a.size == MLP_NNORM
        self._ck(self.L.kmpm_mlp_set_norm(self.h, ptr))

    def loss_grad(self, X, Y):
        import torch
        X, Y = X.contiguous(), Y.contiguous()
        torch.cuda.synchronize()
        loss = ctypes.c_float()
        g = np.empty(MLP_NPARAMS, np.float32)
        self._ck(self.L.kmpm_mlp_loss_grad(self.h, X.data_ptr(), Y.data_ptr(), X.shape[0], ctypes.byref(loss),
                                           g.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return float(loss.value), g

    def train(self, X, Y, steps: int, batch: int = None, lr: float = 1e-3, lr_final_ratio: float = 0.01,
              seed: int = 0, report_every: int = 0) -> float:
        import torch
        X, Y = X.contiguous(), Y.contiguous()
        torch.cuda.synchronize()
        o = TrainOpts(batch=int(batch or self.batch), steps=int(steps), lr=float(lr),
                      lr_final_ratio=float(lr_final_ratio), seed=int(seed), report_every=int(report_every))
        loss = ctypes.c_float()
        self._ck(self.L.kmpm_mlp_train(self.h, X.data_ptr(), Y.data_ptr(), X.shape[0], ctypes.byref(o),
                                       ctypes.byref(loss)))
        return float(loss.value)

    def predict(self, X):
        import torch
        X = X.contiguous()
        Y = torch.empty((X.shape[0], MLP_NOUT), dtype=torch.float32, device=X.device)
        torch.cuda.synchronize()
        self._ck(self.L.kmpm_mlp_predict(self.h, X.data_ptr(), X.shape[0], Y.data_ptr()))
        return Y

    def predict_tc(self, X):
        """Tensor-core inference: (Y [n, 7], inside-envelope flags [n] int8)."""
        import torch
        X = X.contiguous()
        Y = torch.empty((X.shape[0], MLP_NOUT), dtype=torch.float32, device=X.device)
        ins = torch.empty((X.shape[0],), dtype=torch.int8, device=X.device)
        torch.cuda.synchronize()
        self._ck(self.L.kmpm_mlp_predict_tc(self.h, X.data_ptr(), X.shape[0], Y.data_ptr(), ins.data_ptr()))
        return Y, ins
