"""Plain-data description of one MPM problem, shared by every backend.

The script-command mirror (:mod:`karamelo_gb300.model`) fills a
:class:`Scenario` exactly the way Karamelo's host classes fill their state
(``Domain``, ``Grid::init``, ``Solid::populate``, ``Material``, ``Group``,
``Fix``); a backend then runs the time step on it.  Everything here is host
setup, not the hot path.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

# method / scheme / basis codes (src/update.h:78-90 names)
TLMPM, ULMPM = 0, 1
USL, MUSL, USF = 0, 1, 2
LINEAR, CUBIC, BERNSTEIN, QUADRATIC = 0, 1, 2, 3
BASIS_NAMES = {"linear": LINEAR, "cubic-spline": CUBIC, "Bernstein-quadratic": BERNSTEIN,
               "quadratic-spline": QUADRATIC}

# Mat::type (src/material.h:114-119) -- RIGID is not supported on the GPU path
MAT_LINEAR, MAT_NEO_HOOKEAN, MAT_EOS_STRENGTH = 0, 1, 2
EOS_LINEAR, EOS_SHOCK, EOS_FLUID = 0, 1, 2
STR_LINEAR, STR_PLASTIC, STR_JC, STR_SWIFT, STR_FLUID = 0, 1, 2, 3, 4
DAMAGE_NONE, DAMAGE_JC = -1, 0
TEMP_NONE, TEMP_PLASTIC_WORK = -1, 0

FIX_VELOCITY_NODES, FIX_BODY_FORCE = 0, 1
CONTACT_MIN_PENETRATION, CONTACT_HERTZ = 0, 1
CONTACT_STYLES = {"contact/minimize_penetration": CONTACT_MIN_PENETRATION, "contact/hertz": CONTACT_HERTZ}


class MaterialParams(ctypes.Structure):
    """C layout of one material (``kmpm_material`` in include/kmpm.h).

    Parameter vectors follow the argument order of the reference commands:
    eos linear (rho0, K), shock (rho0, K, c0, S, Gamma, cv, Tr, Q1, Q2),
    fluid (rho0, K, Gamma); strength linear (G), plastic (G, sigmay),
    johnson_cook (G, A, B, n, epsdot0, C, m, Tr, Tm), swift (G, A, B, C, n),
    fluid (mu); damage_johnson_cook (d1..d5, epsdot0, Tr, Tm);
    plastic_work (chi, cp, kappa, alpha, T0, Tm).
    """

    _fields_ = [
        ("type", ctypes.c_int),
        ("rho0", ctypes.c_double), ("E", ctypes.c_double), ("nu", ctypes.c_double),
        ("cp", ctypes.c_double), ("kappa", ctypes.c_double),
        ("eos", ctypes.c_int), ("eos_p", ctypes.c_double * 12),
        ("strength", ctypes.c_int), ("str_p", ctypes.c_double * 12),
        ("damage", ctypes.c_int), ("dam_p", ctypes.c_double * 8),
        ("temp", ctypes.c_int), ("temp_p", ctypes.c_double * 6),
    ]

    # Mat::Mat (src/material.cpp:720-769): derived moduli
    def moduli(self):
        if self.type == MAT_EOS_STRENGTH:
            rho0, K, G = self.eos_p[0], self.eos_p[1], self.str_p[0]
            lam = K - 2 * G / 3
            return dict(rho0=rho0, K=K, G=G, lam=lam, c=np.sqrt((lam + 2 * G) / rho0),
                        cp=self.temp_p[1] if self.temp >= 0 else 0.0)
        E, nu = self.E, self.nu
        G = E / (2 * (1 + nu))
        K = E / (3 * (1 - 2 * nu))
        return dict(rho0=self.rho0, K=K, G=G, lam=E * nu / ((1 + nu) * (1 - 2 * nu)),
                    c=np.sqrt(K / self.rho0), cp=self.cp)


@dataclass
class GridSpec:
    """One background grid (``Grid::init``, src/grid.cpp:68-413, one process)."""
    lo: np.ndarray            # boundlo: solid bounds (TL) or box (UL)
    cellsize: float           # Grid::cellsize
    h: float                  # node spacing (cellsize/2 for Bernstein)
    nx: int
    ny: int
    nz: int
    nxg: int                  # global counts, used by the boundary-modified cubic ntype
    nyg: int
    nzg: int
    hi: np.ndarray = None     # boundhi

    @property
    def nnodes(self) -> int:
        return self.nx * self.ny * self.nz

    def node_positions(self, dim: int) -> np.ndarray:
        """Node x0 in the reference order (i outer, k inner), src/grid.cpp:222-226."""
        i, j, k = np.meshgrid(np.arange(self.nx), np.arange(self.ny), np.arange(self.nz), indexing="ij")
        x = np.zeros((self.nnodes, 3))
        x[:, 0] = self.lo[0] + i.ravel() * self.h
        if dim >= 2:
            x[:, 1] = self.lo[1] + j.ravel() * self.h
        if dim == 3:
            x[:, 2] = self.lo[2] + k.ravel() * self.h
        return x


@dataclass
class SolidSpec:
    """Particles of one solid (``Solid::populate``, src/solid.cpp:1810-2336)."""
    name: str
    grid: int
    mat: int
    x0: np.ndarray            # (n, 3)
    v: np.ndarray             # (n, 3)
    mass: np.ndarray          # (n,)
    vol0: np.ndarray          # (n,)
    T0: float
    ptag: np.ndarray          # (n,) int64, 1-based global tags
    mask: np.ndarray = None   # (n,) group bitmask
    ppc: int = 0              # Solid::np_per_cell: particles per cell per direction

    @property
    def np(self) -> int:
        return int(self.x0.shape[0])


@dataclass
class FixSpec:
    """A fix lowered to the device.

    ``velocity_nodes``: per-axis v(t) = c0 + c1*t + c2*exp(c3*t), applied as in
    FixVelocityNodes (src/fix_velocity_nodes.cpp:130-271).
    ``body_force``: constant per-axis acceleration c0 (FixBodyforce,
    src/fix_body_force.cpp:106-179).
    """
    kind: int
    grid: int
    node_mask: np.ndarray     # (nnodes,) uint8
    set: tuple
    coef: np.ndarray          # (3, 4)
    name: str = ""


@dataclass
class ContactSpec:
    """A contact fix between two solids (``fix(ID, contact/minimize_penetration,
    solid1, solid2, mu)``, src/fix_contact_min_penetration.cpp:33-73, or
    ``fix(ID, contact/hertz, solid1, solid2)``, src/fix_contact_hertz.cpp:33-70)."""
    kind: int
    solid1: int
    solid2: int
    mu: float = 0.0
    name: str = ""


@dataclass
class Scenario:
    method: int = TLMPM
    scheme: int = MUSL
    basis: int = LINEAR
    dim: int = 3
    pic_flip: float = 0.99
    transfer: int = 0            # 0: PIC/FLIP blend, 1: APIC (kmpm_params.transfer)
    axisymmetric: bool = False   # Domain::axisymmetric: 2-D, x = r, y = z
    thermal: bool = False
    dt: float = 1e-16            # Update::Update, src/update.cpp:38
    dt_factor: float = 0.9
    dt_constant: bool = False
    boxlo: np.ndarray = field(default_factory=lambda: np.zeros(3))
    boxhi: np.ndarray = field(default_factory=lambda: np.zeros(3))
    materials: List[MaterialParams] = field(default_factory=list)
    grids: List[GridSpec] = field(default_factory=list)
    solids: List[SolidSpec] = field(default_factory=list)
    fixes: List[FixSpec] = field(default_factory=list)
    contacts: List[ContactSpec] = field(default_factory=list)

    @property
    def total_particles(self) -> int:
        return sum(s.np for s in self.solids)


def grid_geometry(dim: int, basis: int, boundlo, boundhi, boxhi, cellsize: float) -> GridSpec:
    """Node counts of ``Grid::init`` (src/grid.cpp:68-200) for one process.

    ``boxhi`` is the process sub-domain upper bound (the whole box here).
    """
    h = cellsize / 2 if basis == BERNSTEIN else cellsize
    boundlo = np.asarray(boundlo, float)
    boundhi = np.asarray(boundhi, float)
    L = [max(0.0, min(boxhi[d], boundhi[d]) - boundlo[d]) for d in range(3)]
    noffhi = [int(np.ceil(L[d] / h)) for d in range(3)]
    Lg = boundhi - boundlo
    nxg = int(Lg[0] / h) + 1
    while nxg * h <= Lg[0] + 0.5 * h:
        nxg += 1
    if dim >= 2:
        nyg = int(int(Lg[1]) / h) + 1           # src/grid.cpp:143 casts L before dividing
        while nyg * h <= Lg[1] + 0.5 * h:
            nyg += 1
    else:
        nyg = 1
    if dim == 3:
        nzg = int(int(Lg[2]) / h) + 1
        while nzg * h <= Lg[2] + 0.5 * h:
            nzg += 1
    else:
        nzg = 1
    n = [max(0, noffhi[0]), max(0, noffhi[1]) if dim >= 2 else 1, max(0, noffhi[2]) if dim >= 3 else 1]
    for d in range(3):
        while boundlo[d] + h * (n[d] - 0.5) < min(boxhi[d], boundhi[d]):
            n[d] += 1
    return GridSpec(lo=boundlo.copy(), cellsize=cellsize, h=h, nx=n[0], ny=n[1], nz=n[2],
                    nxg=nxg, nyg=nyg, nzg=nzg, hi=boundhi.copy())
