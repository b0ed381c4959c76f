"""Parity cases run by the reference itself (the golden fixtures) and by this
project's backends (the FP64 oracle and the CUDA path), from one definition.

Each case builds an input script through :class:`karamelo_gb300.model.MPM`
(the host mirror of Karamelo's commands) and follows a plan of runs, fixes
added between runs, and records:

* ``("run", n)``: ``run(n)``;
* ``("call", fn)``: ``fn(sim)`` issues more commands (e.g. the wall fix);
* ``("state", label)``: every solid's particles (x, v, the dumped stress, eps_p,
  damage, damage_init, T) at this point;
* ``("vars", label)``: the energy fixes' Ek_s and Es_s at this point;
* ``("loop", n, plan)``: the inner plan n times.

``reference_script`` turns a case into the reference's input language (the
commands the model recorded, with every number written exactly, plus the
harness directives ``#@state`` / ``#@vars``); ``tests/golden/make_ref_golden.py``
runs it through the reference (``oracle/_ref/ref_harness``) and stores the
records as ``tests/golden/ref_<case>.npz``.  ``run_plan`` runs the same plan on
one of this project's backends and returns records of the same form, and
``compare`` measures one against the other by ptag.

Large cases store a subset of particles (every k-th ptag) and the
root-sum-square of each field over all particles.
"""
from __future__ import annotations

import os
import struct

import numpy as np

from karamelo_gb300 import workloads as W

HERE = os.path.dirname(os.path.abspath(__file__))
STATE_COLS = 36          # ptag, x0 3, x 3, v 3, stress 9, F 9, eps_p, eps_p rate, damage, damage_init, T, J, vol, mass
SUBSET_TARGET = 5000     # particles kept per state record of a large case
SYM = ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))
FIELDS = ("x", "v", "sigma", "eps_p", "damage", "damage_init", "T")


class NullBackend:
    """Backend that runs nothing: a case builds its script with it."""

    def __init__(self, s):
        self.s = s

    def run(self, n):
        pass

    def run_time(self, t):
        return 0

    def add_fix(self, f):
        pass

    def add_contact(self, c):
        pass


def _wall(sim):
    W.taylor_bar_wall(sim)


def _block_wall(sim):
    sim.fix("wall", "velocity_nodes", "gw", 0, None, None)


def _every(n, plan):
    return ("loop", n, plan)


# name -> (builder(factory, method) -> MPM, CPU method keyword, plan, description)
CASES = {
    # 2-D ULMPM, USL, linear basis, two linear-elastic disks: the energy trace
    # of every step through 3000 steps and the particle state on the way
    "disks_ulmpm_usl_linear": (
        lambda f, m: W.two_disks(f, method=m), "ulmpm",
        [_every(100, [("run", 1), ("vars", "E")]), ("state", "s100"),
         _every(900, [("run", 1), ("vars", "E")]), ("state", "s1000"),
         _every(2000, [("run", 1), ("vars", "E")]), ("state", "s3000")],
        "two colliding disks, 416 particles, 3000 steps"),
    # the Taylor bar's physics at cellsize 0.8 mm: TLMPM MUSL cubic, Johnson-Cook + linear EOS
    "taylor_tlmpm_musl_cubic_jc_0.8": (
        lambda f, m: W.taylor_bar(f, cellsize=0.8, method=m), "tlmpm",
        [("run", 1), ("call", _wall), ("run", 10), ("state", "w10"), ("run", 90), ("state", "w100")],
        "Taylor bar at 0.8 mm (16,848 particles): step 1, wall, 100 steps"),
    # the Taylor bar at cellsize 0.2 mm, 1,045,872 particles
    "taylor_tlmpm_musl_cubic_jc_0.2": (
        lambda f, m: W.taylor_bar(f, cellsize=0.2, method=m), "tlmpm",
        [("run", 1), ("call", _wall), ("run", 10), ("state", "w10")],
        "Taylor bar at 0.2 mm (1,045,872 particles): step 1, wall, 10 steps"),
    # the dam break's physics at 50 mm: ULMPM MUSL cubic, Tait EOS + viscosity, gravity, slip walls
    "dam_ulmpm_musl_cubic_50mm": (
        lambda f, m: W.dam_break(f, cellsize=0.05, method=m), "ulmpm",
        [("run", 50), ("state", "s50"), ("run", 150), ("state", "s200")],
        "dam break at 50 mm (8,192 particles): 200 steps"),
    # the dam break at 10 mm: 1,024,000 particles
    "dam_ulmpm_musl_cubic_10mm": (
        lambda f, m: W.dam_break(f, cellsize=0.01, method=m), "ulmpm",
        [("run", 10), ("state", "s10")],
        "dam break at 10 mm (1,024,000 particles): 10 steps"),
    # the physics of the batch of bars: 2-D TLMPM MUSL cubic tensile bar, shock
    # EOS + Johnson-Cook strength + damage, ends pulled at 50 m/s
    "tensile_tlmpm_jc_damage": (
        lambda f, m: W.tensile_bar_2d(f, cellsize=0.8, vend=50.0, ramp=False, method=m), "tlmpm",
        [("run", 1500), ("state", "s1500"), ("run", 1500), ("state", "s3000")],
        "one 2-D tensile bar with Johnson-Cook damage, 3000 steps"),
    # Johnson-Cook with plastic-work heating (thermo-mechanical TLMPM)
    "block_tlmpm_jc_thermal": (
        lambda f, m: W.block_bar(f, m, "johnson_cook", thermal=True), "tlmpm",
        [("run", 1), ("call", _block_wall), ("run", 150), ("state", "s150")],
        "thermo-mechanical Johnson-Cook bar at a wall, 150 steps"),
}


def build(name, factory, gpu=False):
    builder, cpu_method, _plan, _ = CASES[name]
    return builder(factory, cpu_method + ("/gpu" if gpu else ""))


def _flatten(plan):
    for item in plan:
        if item[0] == "loop":
            for _ in range(item[1]):
                yield from _flatten(item[2])
        else:
            yield item


# ------------------------------------------------------------------ reference side
def reference_script(name):
    """The case in the reference's input language, with harness directives."""
    sim = build(name, NullBackend)
    lines = list(sim.script)
    for item in _flatten(CASES[name][2]):
        n0 = len(sim.script)
        if item[0] == "run":
            sim.run(item[1])
        elif item[0] == "call":
            item[1](sim)
        lines += sim.script[n0:]
        if item[0] == "state":
            lines.append(f"#@state {item[1]}")
        elif item[0] == "vars":
            lines.append(f"#@vars {item[1]} Ek_s Es_s")
    return "\n".join(lines) + "\n"


def read_harness(path):
    """Records of ref_harness's output file: a list of dicts."""
    b = open(path, "rb").read()
    o, out = 0, []
    while o < len(b):
        label = b[o:o + 32].rstrip(b"\0").decode()
        step, time, dt = struct.unpack_from("<qdd", b, o + 32)
        o += 56
        n = struct.unpack_from("<i", b, o)[0]
        o += 4
        rec = {"label": label, "step": step, "time": time, "dt": dt}
        if label.startswith("E"):
            rec["vals"] = np.frombuffer(b, "<f8", n, o).copy()
            o += 8 * n
        else:
            solids = []
            for _ in range(n):
                npart = struct.unpack_from("<q", b, o)[0]
                o += 8
                solids.append(np.frombuffer(b, "<f8", npart * STATE_COLS, o).reshape(npart, STATE_COLS).copy())
                o += 8 * npart * STATE_COLS
            rec["rows"] = np.concatenate(solids) if solids else np.zeros((0, STATE_COLS))
        out.append(rec)
    return out


def state_from_rows(rows):
    """Harness rows -> field arrays sorted by ptag."""
    rows = rows[np.argsort(rows[:, 0], kind="stable")]
    sig = rows[:, 10:19].reshape(-1, 3, 3)
    return {"ptag": rows[:, 0].astype(np.int64), "x": rows[:, 4:7], "v": rows[:, 7:10],
            "sigma": np.stack([sig[:, a, b] for a, b in SYM], 1), "eps_p": rows[:, 28], "damage": rows[:, 30],
            "damage_init": rows[:, 31], "T": rows[:, 32]}


def subset_mask(ptag):
    k = max(1, int(np.ceil(len(ptag) / SUBSET_TARGET)))
    return (ptag % k) == 0 if k > 1 else np.ones(len(ptag), bool)


def pack(records):
    """Harness records -> the arrays of a fixture file."""
    arrays = {}
    evals, esteps, etimes = [], [], []
    for r in records:
        if "vals" in r:
            evals.append(r["vals"])
            esteps.append(r["step"])
            etimes.append(r["time"])
            continue
        lab = r["label"]
        st = state_from_rows(r["rows"])
        keep = subset_mask(st["ptag"])
        arrays[f"{lab}__step"] = np.array(r["step"])
        arrays[f"{lab}__time"] = np.array(r["time"])
        arrays[f"{lab}__dt"] = np.array(r["dt"])
        arrays[f"{lab}__n"] = np.array(len(st["ptag"]))
        for f in ("ptag",) + FIELDS:
            arrays[f"{lab}__{f}"] = st[f][keep]
        for f in FIELDS:
            arrays[f"{lab}__rss_{f}"] = np.array(np.sqrt(np.sum(st[f] ** 2)))
    if evals:
        arrays["E__step"] = np.array(esteps)
        arrays["E__time"] = np.array(etimes)
        arrays["E__vals"] = np.array(evals)
    return arrays


def load(name):
    path = os.path.join(HERE, f"ref_{name}.npz")
    return dict(np.load(path)) if os.path.exists(path) else None


# ------------------------------------------------------------------ this project's side
def capture_state(sim):
    """Every solid's fields, in ptag order, from a backend (oracle or GPU)."""
    parts = {f: [] for f in ("ptag",) + FIELDS}
    for si, sol in enumerate(sim.s.solids):
        parts["ptag"].append(np.asarray(sol.ptag, np.int64))
        parts["x"].append(sim.particles(si, "x"))
        parts["v"].append(sim.particles(si, "v"))
        sg = sim.particles(si, "sigma")
        parts["sigma"].append(np.stack([sg[:, a, b] for a, b in SYM], 1))
        for f in ("eps_p", "damage", "damage_init", "T"):
            parts[f].append(sim.particles(si, f))
    st = {f: np.concatenate(v) for f, v in parts.items()}
    order = np.argsort(st["ptag"], kind="stable")
    return {f: v[order] for f, v in st.items()}


def run_plan(name, factory, gpu=False, prepare=None):
    """Runs a case on a backend; returns {label: state} and the energy trace
    (steps, time, (Ek, Es) rows).  ``prepare(sim)`` may alter the scenario
    before the backend is created."""
    sim = build(name, factory, gpu=gpu)
    if prepare:
        prepare(sim)
    sim._ensure_backend()
    states, E = {}, []
    for item in _flatten(CASES[name][2]):
        if item[0] == "run":
            sim.run(item[1])
        elif item[0] == "call":
            item[1](sim)
        elif item[0] == "state":
            st = capture_state(sim)
            st["step"], st["time"], st["dt"] = sim.ntimestep, sim.time, sim.dt
            states[item[1]] = st
        elif item[0] == "vars":
            E.append((sim.ntimestep, sim.time, *sim.energies()))
    return sim, states, np.array(E) if E else None


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def compare(fixture, label, state):
    """Relative L2 errors of a captured state against a fixture record, on
    the fixture's particle subset, and of the all-particle root-sum-squares."""
    pt = fixture[f"{label}__ptag"]
    idx = np.searchsorted(state["ptag"], pt)
    assert np.array_equal(state["ptag"][idx], pt), "particle tags differ from the reference's"
    assert len(state["ptag"]) == int(fixture[f"{label}__n"]), "particle count differs from the reference's"
    err = {}
    for f in FIELDS:
        ref = fixture[f"{label}__{f}"]
        if np.linalg.norm(ref) == 0.0 and np.linalg.norm(state[f][idx]) == 0.0:
            err[f] = 0.0
            continue
        err[f] = rel(state[f][idx], ref)
        rss = float(np.sqrt(np.sum(state[f] ** 2)))
        err[f"rss_{f}"] = abs(rss - float(fixture[f"{label}__rss_{f}"])) / max(float(fixture[f"{label}__rss_{f}"]), 1e-300)
    return err
