"""Host-side mirror of Karamelo's input-script commands for the GPU method.

A Karamelo input script such as::

    method(tlmpm, FLIP, cubic-spline, 0.99)
    dimension(3, -16.2, 16.2, -4, 4, -4, 4, 0.2)
    eos(eosl, linear, rho, K)
    strength(jc, johnson_cook, G, A, B, n, epsdot0, C, m, Tr, Tm)
    material(mat, eos-strength, eosl, jc)
    region(cyl, cylinder, x, 0, 0, R, -L, L)
    solid(s1, region, cyl, 2, mat, 0.2, Tr)
    fix(v0, initial_velocity_particles, g, 190, NULL, NULL)
    run(100)

becomes, with the GPU style keyword ``tlmpm/gpu``::

    sim = MPM()
    sim.method("tlmpm/gpu", "FLIP", "cubic-spline", 0.99)
    sim.dimension(3, -16.2, 16.2, -4, 4, -4, 4, 0.2)
    ...
    sim.run(100)

The commands fill a :class:`~karamelo_gb300.scenario.Scenario` the way the
reference's host classes fill their state (cited per command); ``run`` hands
it to the backend, which for the ``/gpu`` styles is the CUDA library behind
the C ABI in include/kmpm.h.  Errors raise :class:`KarameloError`, the
counterpart of the reference's ``error->all`` / ``error->one``.
"""
from __future__ import annotations

import functools
import inspect
import math
from typing import Callable, Dict, List, Optional

import numpy as np

from . import scenario as sc
from .regions import BIG, make_region


class KarameloError(RuntimeError):
    """Raised where the reference calls Error::all / Error::one (src/error.cpp:33-68)."""


class TimeFn:
    """Time-dependent fix value v(time) = c0 + c1*time + c2*exp(c3*time).

    The reference evaluates arbitrary expressions of ``time``
    (src/fix_velocity_nodes.cpp:66-108); the device path supports this family,
    which covers constants, ramps and ``1-exp(-time)`` loadings.
    """

    def __init__(self, c0=0.0, c1=0.0, c2=0.0, c3=0.0):
        self.c = np.array([c0, c1, c2, c3], float)

    def __call__(self, t):
        return self.c[0] + self.c[1] * t + self.c[2] * np.exp(self.c[3] * t)


def _coef(value) -> np.ndarray:
    if isinstance(value, TimeFn):
        return value.c.copy()
    return np.array([float(value), 0.0, 0.0, 0.0])


def exact_literal(x: float) -> str:
    """``x`` written in Karamelo's input language so that its parser yields
    exactly this double.  The parser reads each numeric literal with ``stof``
    (single precision, src/input.cpp:405-411) and then evaluates in double,
    so a literal such as 0.8 would arrive as 0.800000011920929.  Here x =
    M 2^E with an integer M < 2^53 is written as a sum of 24-bit pieces of M
    scaled by powers of two; every literal is exact in single precision and
    every operation is exact in double."""
    x = float(x)
    if not math.isfinite(x):
        raise ValueError(f"non-finite script literal {x}")
    if x == 0.0:
        return "0"
    if x == int(x) and abs(x) < 2 ** 24:
        return str(int(x)) if x > 0 else f"(0-{int(-x)})"
    m, e = math.frexp(abs(x))
    M, E = int(m * 2 ** 53), e - 53
    while M % 2 == 0:
        M //= 2
        E += 1
    a, rem = divmod(M, 2 ** 48)
    b, c = divmod(rem, 2 ** 24)
    terms = []
    if a:
        terms.append(f"{a}*{2 ** 48}")
    if b:
        terms.append(f"{b}*{2 ** 24}")
    if c:
        terms.append(str(c))
    body = "(" + "+".join(terms) + ")"
    # scale by 2^E in factors of at most 2^100 (each a power of two, exact in single precision)
    while E < 0:
        k = min(-E, 100)
        body = f"({body}/{2 ** k})"
        E += k
    while E > 0:
        k = min(E, 100)
        body = f"({body}*{2 ** k})"
        E -= k
    return body if x > 0 else f"(0-{body})"


def script_arg(v) -> str:
    """One command argument in Karamelo's input language."""
    if v is None:
        return "NULL"
    if isinstance(v, TimeFn):
        c0, c1, c2, c3 = (float(t) for t in v.c)
        return (f"{exact_literal(c0)}+{exact_literal(c1)}*time+"
                f"{exact_literal(c2)}*exp({exact_literal(c3)}*time)")
    if isinstance(v, (bool, np.bool_)):
        return "true" if v else "false"
    if isinstance(v, (int, np.integer, float, np.floating)):
        return exact_literal(float(v))
    if v in ("-INF", "+INF"):
        # the reference's block region takes INF for every bound (a lower
        # bound reads it as -BIG) but rejects -INF for zlo (src/region_block.cpp:102)
        return "INF"
    return str(v)


def _command(fn):
    """Marks a script command: besides running it, the call is recorded as a
    line of Karamelo's input language (``MPM.script``), so that the reference
    itself can run the same sequence of commands."""
    sig = inspect.signature(fn)

    @functools.wraps(fn)
    def wrapper(self, *args):
        bound = sig.bind(self, *args)
        vals = []
        for name, par in list(sig.parameters.items())[1:]:
            if par.kind == inspect.Parameter.VAR_POSITIONAL:
                vals.extend(bound.arguments.get(name, ()))
            elif name in bound.arguments:
                vals.append(bound.arguments[name])
            elif fn.__name__ == "solid" and name == "T0":
                vals.append(par.default)  # the reference's solid() takes T0 explicitly
        if fn.__name__ == "method" and vals and isinstance(vals[0], str) and vals[0].endswith("/gpu"):
            vals[0] = vals[0][:-4]
        self.script.append(f"{fn.__name__}({', '.join(script_arg(v) for v in vals)})")
        return fn(self, *args)

    return wrapper


_SUPPORTED_FIXES = ("velocity_nodes", "body_force", "initial_velocity_particles", "kinetic_energy", "strain_energy")


class MPM:
    """The script session (the ``MPM`` god-object of src/mpm.cpp, host side only)."""

    def __init__(self, backend_factory: Optional[Callable] = None):
        self.s = sc.Scenario()
        self._backend_factory = backend_factory
        self.backend = None
        self.regions: Dict[str, object] = {}
        self.eoses: Dict[str, tuple] = {}
        self.strengths: Dict[str, tuple] = {}
        self.damages: Dict[str, tuple] = {}
        self.temperatures: Dict[str, tuple] = {}
        self.material_ids: Dict[str, int] = {}
        self.solid_ids: Dict[str, int] = {}
        self.groups: Dict[str, dict] = {}
        self.energy_fixes: Dict[str, str] = {}
        self.contact_ids: Dict[str, int] = {}
        self.np_total = 0
        self.method_set = False
        self.dim_set = False
        self.ntimestep = 0
        # the commands so far, in Karamelo's input language (see _command)
        self.script: List[str] = []

    # ------------------------------------------------------------ method/scheme
    @_command
    def method(self, style: str, sub: str, basis: str = "linear", *rest):
        """``method()``: Update::create_method, src/update.cpp:108-196."""
        base = style[:-4] if style.endswith("/gpu") else style
        if base not in ("tlmpm", "ulmpm"):
            raise KarameloError(f"Illegal method style {style}: the GPU path provides tlmpm/gpu and ulmpm/gpu")
        if self._backend_factory is None and not style.endswith("/gpu"):
            raise KarameloError(f"method style {style} is the reference's CPU method; use {base}/gpu")
        self.s.method = sc.TLMPM if base == "tlmpm" else sc.ULMPM
        self.s.transfer = 0
        if sub == "PIC":
            self.s.pic_flip = 0.0
        elif sub == "FLIP":
            if not rest:
                raise KarameloError("Illegal method command: FLIP needs the PIC/FLIP ratio")
        elif sub in ("APIC", "MLS"):
            # APIC and MLS set PIC_FLIP = 0 (src/tlmpm.cpp:82-84, src/ulmpm.cpp:79-82)
            if sub == "MLS" and self.s.method != sc.ULMPM:
                raise KarameloError("MLS is a ULMPM method type")
            self.s.transfer = 1 if sub == "APIC" else 4
            self.s.pic_flip = 0.0
        elif sub in ("AFLIP", "ASFLIP"):
            if not rest:
                raise KarameloError(f"Illegal method command: {sub} needs the PIC/FLIP ratio")
            self.s.transfer = 2 if sub == "AFLIP" else 3
        else:
            raise KarameloError(f"method type {sub} not supported on the GPU path "
                                "(PIC, FLIP, APIC, AFLIP, ASFLIP or MLS)")
        if basis not in sc.BASIS_NAMES:
            raise KarameloError(f"shape function {basis} not supported: linear, cubic-spline, quadratic-spline, "
                                "Bernstein-quadratic")
        self.s.basis = sc.BASIS_NAMES[basis]
        if self.s.basis == sc.BERNSTEIN and self.s.method == sc.ULMPM:
            raise KarameloError("Bernstein-quadratic shape functions are only supported with TLMPM")
        affine = self.s.transfer == 1 or (self.s.method == sc.ULMPM and self.s.transfer >= 2)
        linear_tl = self.s.basis == sc.LINEAR and self.s.method == sc.TLMPM
        if affine and self.s.basis not in (sc.CUBIC, sc.QUADRATIC) and not linear_tl:
            # Solid::compute_inertia_tensor, src/solid.cpp:1447-1473
            raise KarameloError(f"{sub} runs with the cubic or quadratic spline (and, for tlmpm, linear)")
        rest = list(rest)
        if sub in ("FLIP", "AFLIP", "ASFLIP"):
            self.s.pic_flip = float(rest.pop(0))
        if rest:
            kw = rest.pop(0)
            if kw == "thermo-mechanical":
                self.s.thermal = True
            elif kw == "mechanical":
                self.s.thermal = False
            else:
                raise KarameloError(f"Illegal method keyword {kw}")
        if rest:
            raise KarameloError("Illegal method command: too many arguments")
        self.method_set = True

    @_command
    def scheme(self, style: str):
        """``scheme()``: Update::create_scheme, src/update.cpp:83-102 (default MUSL)."""
        base = style[:-4] if style.endswith("/gpu") else style
        if base == "usl":
            self.s.scheme = sc.USL
        elif base == "musl":
            self.s.scheme = sc.MUSL
        elif base == "usf":
            self.s.scheme = sc.USF
        else:
            raise KarameloError(f"Illegal scheme style {style}: usl, musl or usf")

    @_command
    def set_dt(self, dt):
        """Update::set_dt, src/update.cpp:58-65."""
        self.s.dt = float(dt)
        self.s.dt_constant = True

    @_command
    def dt_factor(self, f):
        """Update::set_dt_factor, src/update.cpp:51-56."""
        self.s.dt_factor = float(f)

    # ------------------------------------------------------------ domain/regions
    @_command
    def dimension(self, dim, *args):
        """Domain::set_dimension, src/domain.cpp:496-551."""
        if not self.method_set:
            raise KarameloError("a method must be defined before the dimension")
        dim = int(dim)
        need = {1: 3, 2: 5, 3: 7}[dim]
        if len(args) != need:
            raise KarameloError("dimension: wrong number of arguments")
        lo, hi = np.zeros(3), np.zeros(3)
        for d in range(dim):
            lo[d], hi[d] = float(args[2 * d]), float(args[2 * d + 1])
        self.s.dim = dim
        self.s.boxlo, self.s.boxhi = lo, hi
        self.sublo, self.subhi = lo.copy(), hi.copy()
        self.cellsize = float(args[-1])
        if self.s.method == sc.ULMPM:
            if self.cellsize < 0:
                raise KarameloError("cellsize negative")
            self.s.grids.append(sc.grid_geometry(dim, self.s.basis, lo, hi, self.subhi, self.cellsize))
        self.dim_set = True

    @_command
    def axisymmetric(self, flag):
        """``axisymmetric(true|false)``: Domain::set_axisymmetric,
        src/domain.cpp:558-570.  Solids created afterwards get masses and
        volumes multiplied by their radius x0_r (Solid::populate,
        src/solid.cpp:2292-2295).  The GPU path takes it in 2-D mechanical runs."""
        on = str(flag).lower() in ("true", "1")
        if str(flag).lower() not in ("true", "false", "1", "0"):
            raise KarameloError("axisymmetric(true) or axisymmetric(false)")
        if on and (self.s.dim != 2 or self.s.thermal):
            raise KarameloError("axisymmetric runs on the GPU path are 2-D and mechanical")
        self.s.axisymmetric = on

    @_command
    def region(self, name, kind, *args):
        """``region()``: Domain::add_region; block regions grow the box
        (src/region_block.cpp:45-120)."""
        if name in self.regions:
            raise KarameloError(f"reuse of region ID {name}")
        self.regions[name] = make_region(kind, args, self.s.dim, self.s.boxlo, self.s.boxhi, len(self.regions))

    # ------------------------------------------------------------ materials
    @_command
    def eos(self, name, kind, *p):
        """``eos()``: src/eos_linear.cpp, src/eos_shock.cpp, src/eos_fluid.cpp."""
        n = {"linear": 2, "shock": 9, "fluid": 3}
        if kind not in n:
            raise KarameloError(f"unknown eos {kind}")
        if len(p) < n[kind]:
            raise KarameloError(f"eos {kind}: too few arguments")
        self.eoses[name] = ({"linear": sc.EOS_LINEAR, "shock": sc.EOS_SHOCK, "fluid": sc.EOS_FLUID}[kind],
                            [float(x) for x in p[: n[kind]]])

    @_command
    def strength(self, name, kind, *p):
        """``strength()``: src/strength_*.cpp."""
        n = {"linear": 1, "plastic": 2, "johnson_cook": 9, "swift": 5, "fluid": 1}
        code = {"linear": sc.STR_LINEAR, "plastic": sc.STR_PLASTIC, "johnson_cook": sc.STR_JC,
                "swift": sc.STR_SWIFT, "fluid": sc.STR_FLUID}
        if kind not in n:
            raise KarameloError(f"unknown strength {kind}")
        if len(p) < n[kind]:
            raise KarameloError(f"strength {kind}: too few arguments")
        vals = [float(x) for x in p[: n[kind]]]
        if kind == "johnson_cook" and vals[7] == vals[8]:
            raise KarameloError("Error: reference temperature Tr equals melting temperature Tm")
        self.strengths[name] = (code[kind], vals)

    @_command
    def damage(self, name, kind, *p):
        """``damage()``: src/damage_jc.cpp:32-89."""
        if kind != "damage_johnson_cook":
            raise KarameloError(f"unknown damage {kind}")
        if len(p) < 8:
            raise KarameloError("damage_johnson_cook: too few arguments")
        self.damages[name] = (sc.DAMAGE_JC, [float(x) for x in p[:8]])

    @_command
    def temperature(self, name, kind, *p):
        """``temperature()``: src/temperature_plastic_work.cpp:20-57."""
        if kind != "plastic_work":
            raise KarameloError(f"unknown temperature {kind}")
        if len(p) != 6:
            raise KarameloError("plastic_work: wrong number of arguments")
        self.temperatures[name] = (sc.TEMP_PLASTIC_WORK, [float(x) for x in p])

    @_command
    def material(self, name, kind, *p):
        """Material::add_material, src/material.cpp:249-380."""
        if name in self.material_ids:
            raise KarameloError("Error: reuse of material ID.")
        m = sc.MaterialParams()
        m.damage, m.temp = sc.DAMAGE_NONE, sc.TEMP_NONE
        if kind in ("linear", "neo-hookean"):
            m.type = sc.MAT_LINEAR if kind == "linear" else sc.MAT_NEO_HOOKEAN
            m.rho0, m.E, m.nu = (float(x) for x in p[:3])
            if len(p) >= 5:
                m.cp, m.kappa = float(p[3]), float(p[4])
        elif kind == "rigid":
            raise KarameloError("rigid materials are not supported on the GPU path")
        elif kind == "eos-strength":
            m.type = sc.MAT_EOS_STRENGTH
            if p[0] not in self.eoses:
                raise KarameloError(f"Error: could not find EOS named: {p[0]}.")
            if p[1] not in self.strengths:
                raise KarameloError(f"Error: could not find strength named: {p[1]}.")
            m.eos, ep = self.eoses[p[0]]
            m.strength, spar = self.strengths[p[1]]
            for i, v in enumerate(ep):
                m.eos_p[i] = v
            for i, v in enumerate(spar):
                m.str_p[i] = v
            for extra in p[2:]:
                if extra in self.damages:
                    m.damage, dp = self.damages[extra]
                    for i, v in enumerate(dp):
                        m.dam_p[i] = v
                elif extra in self.temperatures:
                    m.temp, tp = self.temperatures[extra]
                    for i, v in enumerate(tp):
                        m.temp_p[i] = v
                else:
                    raise KarameloError(f"Error: could not find damage or temperature named: {extra}.")
        else:
            raise KarameloError(f"unknown material type {kind}")
        self.s.materials.append(m)
        self.material_ids[name] = len(self.s.materials) - 1

    # ------------------------------------------------------------ solids
    @_command
    def solid(self, name, kind, region, ppc, mat, cellsize, T0=0.0):
        """``solid(id, region, region_id, ppc1d, mat, cellsize, T0)``:
        Solid::Solid + Solid::populate, src/solid.cpp:59-163, 1810-2336."""
        if not self.dim_set:
            raise KarameloError("The domain must be created before any solids can")
        if kind != "region":
            raise KarameloError("only region-populated solids are supported on the GPU path")
        if region not in self.regions:
            raise KarameloError(f"Error: region ID {region} not does not exist.")
        if mat not in self.material_ids:
            raise KarameloError(f"Error: could not find material named {mat}")
        if name in self.solid_ids:
            raise KarameloError(f"Error: reuse of solid ID {name}")
        reg = self.regions[region]
        dim = self.s.dim
        cellsize = float(cellsize)
        lim = np.array(reg.limits(), float)
        solidlo, solidhi = lim[0::2].copy(), lim[1::2].copy()
        if self.s.method == sc.TLMPM:
            g = sc.grid_geometry(dim, self.s.basis, solidlo, solidhi, self.subhi, cellsize)
            self.s.grids.append(g)
            gid = len(self.s.grids) - 1
            boundlo, boundhi = solidlo, solidhi
        else:
            gid = 0
            if cellsize != self.s.grids[0].cellsize:
                # Grid::setup (src/grid.cpp:415-420) would overwrite the shared
                # UL grid's cellsize after its nodes were laid out
                raise KarameloError("ulmpm solids must use the cellsize given to dimension()")
            boundlo, boundhi = self.s.boxlo, self.s.boxhi
        delta = cellsize
        # populate lattice, src/solid.cpp:1871-2101
        nsub = []
        for d in range(3):
            Llo = max(0.0, self.sublo[d] - boundlo[d])
            Lhi = max(0.0, min(self.subhi[d], boundhi[d]) - boundlo[d])
            n0 = int(np.floor(Llo / delta))
            n1 = int(np.ceil(Lhi / delta))
            n = max(0, n1 - n0) if d < dim else 1
            while boundlo[d] + delta * (n0 + n - 0.5) < min(self.subhi[d], boundhi[d]):
                n += 1
            nsub.append((n0, n))
        ppc = int(ppc)
        if ppc == 1:
            pts = np.zeros((1, 3))
        elif ppc == 2:
            xi = 0.25
            pts = np.array([[-xi, -xi, -xi], [-xi, xi, -xi], [xi, -xi, -xi], [xi, xi, -xi],
                            [-xi, -xi, xi], [-xi, xi, xi], [xi, -xi, xi], [xi, xi, xi]])
        elif ppc == 3:
            xi = 0.7746 / 2
            v = [-xi, 0, xi]
            pts = np.array([[a, b, c] for c in v for a in v for b in v])
        else:
            dd = 1.0 / ppc
            pts = np.array([[(i + 0.5) * dd - 0.5, (j + 0.5) * dd - 0.5, (k + 0.5) * dd - 0.5]
                            for k in range(ppc) for i in range(ppc) for j in range(ppc)])
        nip = {1: ppc, 2: ppc * ppc, 3: ppc ** 3}[dim] if ppc != 1 else 1
        pts = pts[:nip]
        vol = delta ** dim
        mass = self.s.materials[self.material_ids[mat]].moduli()["rho0"] * vol / nip
        vol /= nip
        ii, jj, kk, pp = np.meshgrid(np.arange(nsub[0][1]), np.arange(nsub[1][1]), np.arange(nsub[2][1]),
                                     np.arange(nip), indexing="ij")
        ii, jj, kk, pp = ii.ravel(), jj.ravel(), kk.ravel(), pp.ravel()
        x = np.zeros((ii.size, 3))
        x[:, 0] = boundlo[0] + delta * (nsub[0][0] + ii + 0.5 + pts[pp, 0])
        x[:, 1] = boundlo[1] + delta * (nsub[1][0] + jj + 0.5 + pts[pp, 1])
        if dim == 3:
            x[:, 2] = boundlo[2] + delta * (nsub[2][0] + kk + 0.5 + pts[pp, 2])
        inside_sub = np.all((x >= self.sublo) & (x <= self.subhi), axis=1)
        keep = inside_sub & reg.inside(x)
        x = x[keep]
        n = x.shape[0]
        if n == 0:
            raise KarameloError("Error: solid does not have any particles.")
        ptag = np.arange(1, n + 1, dtype=np.int64) + self.np_total
        self.np_total += n
        masses, vols = np.full(n, mass), np.full(n, vol)
        if self.s.axisymmetric:
            # mass = mass_ x0_r, vol0 = mass / rho0 (src/solid.cpp:2292-2295)
            rho0 = self.s.materials[self.material_ids[mat]].moduli()["rho0"]
            masses = mass * x[:, 0]
            vols = masses / rho0
        self.s.solids.append(sc.SolidSpec(name=name, grid=gid, mat=self.material_ids[mat], x0=x,
                                          v=np.zeros((n, 3)), mass=masses, vol0=vols,
                                          T0=float(T0), ptag=ptag, mask=np.ones(n, np.int64), ppc=ppc))
        self.solid_ids[name] = len(self.s.solids) - 1

    # ------------------------------------------------------------ groups/fixes
    @_command
    def group(self, name, pon, kind, region, sel="all", *solids):
        """Group::assign, src/group.cpp:65-238 (region match on x0)."""
        if pon not in ("particles", "nodes"):
            raise KarameloError(f"Error: do not understand keyword {pon}")
        if kind != "region" or region not in self.regions:
            raise KarameloError(f"Error: could not find region {region}.")
        reg = self.regions[region]
        targets = list(range(len(self.s.solids))) if sel == "all" else [self.solid_ids[sn] for sn in solids]
        if sel not in ("all", "solid"):
            raise KarameloError(f"Error: unknown keyword in group command: {sel}")
        masks = {}
        for si in targets:
            if pon == "particles":
                masks[si] = reg.match(self.s.solids[si].x0)
            else:
                g = self.s.grids[self.s.solids[si].grid]
                masks[si] = reg.match(g.node_positions(self.s.dim))
        self.groups[name] = dict(pon=pon, solid=-1 if sel == "all" else targets[-1], masks=masks)

    @_command
    def fix(self, name, kind, group, *vals):
        """Modify::add_fix for the fixes the GPU method lowers; any other fix is an error
        (the GPU path has no CPU fallback)."""
        if kind in sc.CONTACT_STYLES:
            # fix(ID, contact/minimize_penetration, solid1, solid2, mu) and
            # fix(ID, contact/hertz, solid1, solid2): the third argument is a solid
            # (src/fix_contact_min_penetration.cpp:55-73, src/fix_contact_hertz.cpp:52-70)
            code = sc.CONTACT_STYLES[kind]
            args = [group] + list(vals)
            need = 3 if code == sc.CONTACT_MIN_PENETRATION else 2
            if len(args) < need:
                raise KarameloError("Error: not enough arguments.")
            ids = []
            for nm in args[:2]:
                if nm not in self.solid_ids:
                    raise KarameloError(f"Error: solid {nm} unknown.")
                ids.append(self.solid_ids[nm])
            mu = float(args[2]) if code == sc.CONTACT_MIN_PENETRATION else 0.0
            c = sc.ContactSpec(kind=code, solid1=ids[0], solid2=ids[1], mu=mu, name=name)
            self.s.contacts.append(c)
            self.contact_ids[name] = len(self.s.contacts) - 1
            if self.backend is not None:
                self.backend.add_contact(c)
            return
        if kind not in _SUPPORTED_FIXES:
            raise KarameloError(f"fix {kind} is not supported by the GPU method")
        if group != "all" and group not in self.groups:
            raise KarameloError(f"Error: could not find group {group}")
        if kind in ("kinetic_energy", "strain_energy"):
            self.energy_fixes[name] = kind
            return
        gr = self.groups.get(group)
        dim = self.s.dim
        vals = list(vals) + [None] * (3 - len(vals))
        set_ = tuple(int(v is not None and d < dim) for d, v in enumerate(vals[:3]))
        if kind == "initial_velocity_particles":
            # FixInitialVelocityParticles::initial_integrate, src/fix_initial_velocity_particles.cpp:99-163
            if gr is None or gr["pon"] != "particles":
                raise KarameloError("initial_velocity_particles needs a group of particles")
            if self.ntimestep != 0:
                return  # applies at step 1 only
            for si, m in gr["masks"].items():
                for d in range(3):
                    if set_[d]:
                        self.s.solids[si].v[m, d] = float(vals[d])
            return
        coef = np.zeros((3, 4))
        for d in range(3):
            if set_[d]:
                coef[d] = _coef(vals[d])
        code = sc.FIX_VELOCITY_NODES if kind == "velocity_nodes" else sc.FIX_BODY_FORCE
        if code == sc.FIX_BODY_FORCE and np.any(coef[:, 1:] != 0):
            raise KarameloError("body_force values must be constants on the GPU path")
        if group == "all":
            targets = [(si, np.ones(self.s.grids[s.grid].nnodes, bool)) for si, s in enumerate(self.s.solids)]
        else:
            if gr["pon"] != "nodes":
                raise KarameloError(f"{kind} needs to be given a group of nodes")
            targets = list(gr["masks"].items())
        # the reference loops over the solids of the group and applies the fix
        # to each solid's grid; on the shared UL grid this repeats it once per solid
        for si, m in targets:
            f = sc.FixSpec(kind=code, grid=self.s.solids[si].grid, node_mask=m.astype(np.uint8),
                           set=set_, coef=coef.copy(), name=name)
            self.s.fixes.append(f)
            if self.backend is not None:
                self.backend.add_fix(f)

    # ------------------------------------------------------------ run
    def _ensure_backend(self):
        if self.backend is None:
            if not self.s.solids:
                raise KarameloError("Error: no solid was defined")
            if self._backend_factory is not None:
                self.backend = self._backend_factory(self.s)
            else:
                from .gpu import GpuBackend
                self.backend = GpuBackend(self.s)
        return self.backend

    @_command
    def run(self, n):
        """Run::command, src/run.cpp:32-57."""
        b = self._ensure_backend()
        b.run(int(n))
        self.ntimestep += int(n)

    @_command
    def run_time(self, t):
        """RunTime::command, src/run_time.cpp:30-60."""
        b = self._ensure_backend()
        self.ntimestep += b.run_time(float(t))

    # ------------------------------------------------------------ outputs
    def particles(self, solid, field):
        return self._ensure_backend().particles(self.solid_ids[solid] if isinstance(solid, str) else solid, field)

    def energies(self):
        """(Ek, Es): FixKineticEnergy / ComputeStrainEnergy over all solids."""
        return self._ensure_backend().energies()

    def contact_force(self, name):
        """The contact fix's variables (ID_x, ID_y, ID_z) after the last step."""
        return self._ensure_backend().contact_force(self.contact_ids[name])

    @property
    def time(self):
        return self._ensure_backend().scalars()[0]

    @property
    def dt(self):
        return self._ensure_backend().scalars()[1]
