"""Parity with the reference itself.

The fixtures tests/golden/ref_<case>.npz hold particle states (and, for the
two disks, the energy trace of every step) written by the unmodified
reference (every src/*.cpp of the Karamelo tree compiled against
oracle/stubs, driven by oracle/ref_harness.cpp; made by
tests/golden/make_ref_golden.py from the cases in tests/golden/ref_cases.py).
Particles are matched by ptag; tolerances are relative L2 norms over the
stored particles (a subset of every k-th ptag for the cases above 5000
particles), stated per case.

* CPU: the FP64 oracle (oracle/mpm_oracle.cpp) against the reference.  Both
  compute in FP64 from the same inputs (the scripts write every number
  exactly), so they agree to round-off: bit for bit for the ULMPM cases,
  within 1e-12 where the polar decomposition and eigenvalues differ in
  rounding (the reference's Eigen routines against the oracle's).
* GPU: the CUDA path through the C ABI against the reference, at the
  tolerances of its FP32 arithmetic.
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import ref_cases as RC  # noqa: E402

SMALL = ["disks_ulmpm_usl_linear", "taylor_tlmpm_musl_cubic_jc_0.8", "dam_ulmpm_musl_cubic_50mm",
         "block_tlmpm_jc_thermal", "tensile_tlmpm_jc_damage"]
LARGE = ["taylor_tlmpm_musl_cubic_jc_0.2", "dam_ulmpm_musl_cubic_10mm"]


def _fixture(name):
    fx = RC.load(name)
    if fx is None:
        pytest.fail(f"missing fixture tests/golden/ref_{name}.npz (tests/golden/make_ref_golden.py)")
    return fx


def test_fixtures_present_and_consistent():
    for name in SMALL + LARGE:
        fx = _fixture(name)
        labels = sorted({k.split("__")[0] for k in fx if not k.startswith("E__")})
        assert labels, name
        for lab in labels:
            pt = fx[f"{lab}__ptag"]
            assert np.all(np.diff(pt) > 0) and len(pt) <= int(fx[f"{lab}__n"])
            for f in RC.FIELDS:
                assert np.all(np.isfinite(fx[f"{lab}__{f}"]))
    # the two disks' published sizes: 416 particles (208 per disk), 3000 steps logged
    fx = _fixture("disks_ulmpm_usl_linear")
    assert int(fx["s3000__n"]) == 416 and len(fx["E__step"]) == 3000
    # the Taylor bar at 0.2 mm: 1,045,872 particles; the dam break at 10 mm: 1,024,000
    assert int(_fixture("taylor_tlmpm_musl_cubic_jc_0.2")["w10__n"]) == 1045872
    assert int(_fixture("dam_ulmpm_musl_cubic_10mm")["s10__n"]) == 1024000


# ------------------------------------------------------------------ FP64 oracle
@pytest.mark.parametrize("name", SMALL)
def test_oracle_matches_reference(oracle_mod, name):
    fx = _fixture(name)
    sim, states, E = RC.run_plan(name, oracle_mod.OracleBackend)
    for lab, st in states.items():
        assert st["step"] == int(fx[f"{lab}__step"])
        assert abs(st["time"] - float(fx[f"{lab}__time"])) <= 1e-12 * abs(float(fx[f"{lab}__time"]))
        assert abs(st["dt"] / float(fx[f"{lab}__dt"]) - 1) < 1e-12
        for k, e in RC.compare(fx, lab, st).items():
            assert e < 1e-10, f"{name} {lab} {k}: rel L2 {e:.3e}"
    if E is not None:
        ref = fx["E__vals"]
        assert np.array_equal(E[:, 0], fx["E__step"])
        assert np.max(np.abs(E[:, 2:] - ref)) <= 1e-12 * np.max(np.abs(ref))


# ------------------------------------------------------------------ CUDA path
GPU_TOL = {
    # 3-D TLMPM MUSL cubic Johnson-Cook + linear EOS (FP32 bulk)
    "taylor_tlmpm_musl_cubic_jc_0.8": {"x": 1e-6, "v": 1e-4, "sigma": 1e-4, "eps_p": 1e-4},
    "taylor_tlmpm_musl_cubic_jc_0.2": {"x": 1e-6, "v": 1e-4, "sigma": 1e-4, "eps_p": 1e-4},
    # ULMPM fluid: the Tait pressure amplifies J's rounding by gamma = 7
    "dam_ulmpm_musl_cubic_50mm": {"x": 1e-6, "v": 1e-4, "sigma": 1e-3},
    "dam_ulmpm_musl_cubic_10mm": {"x": 1e-6, "v": 1e-4, "sigma": 1e-3},
    "block_tlmpm_jc_thermal": {"x": 1e-6, "v": 1e-3, "sigma": 1e-3, "eps_p": 1e-3, "T": 1e-5},
    "tensile_tlmpm_jc_damage": {"x": 1e-6, "v": 1e-3, "sigma": 1e-3, "eps_p": 1e-3, "damage_init": 1e-3},
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(GPU_TOL))
def test_gpu_matches_reference(gpu_lib, name):
    from karamelo_gb300.gpu import GpuBackend
    fx = _fixture(name)
    sim, states, _ = RC.run_plan(name, None, gpu=True)
    assert isinstance(sim.backend, GpuBackend)
    for lab, st in states.items():
        assert st["step"] == int(fx[f"{lab}__step"])
        assert abs(st["dt"] / float(fx[f"{lab}__dt"]) - 1) < 1e-5
        assert abs(st["time"] / float(fx[f"{lab}__time"]) - 1) < 1e-5
        err = RC.compare(fx, lab, st)
        print(f"\n{name} {lab}: " + ", ".join(f"{f} {err[f]:.2e}" for f in GPU_TOL[name]))
        for f, tol in GPU_TOL[name].items():
            assert err[f] < tol, f"{name} {lab} {f}: rel L2 {err[f]:.3e} >= {tol}"
            assert err[f"rss_{f}"] < tol, f"{name} {lab} rss {f}: {err['rss_' + f]:.3e} >= {tol}"


# The two disks (2-D ULMPM, USL, linear basis, 3000 steps).  The disks fly rigidly until
# their particles reach the nodes (step ~125); there the near-empty nodes of
# the linear basis amplify rounding, and FP32 and FP64 runs part.  The
# oracle's own sensitivity floor, measured by running it from the initial
# state rounded to FP32 (relative L2 against the reference): x 2.2e-8 and
# v 1.5e-8 at step 100; x 8.6e-6, v 5.5e-4, sigma 3.3e-3 at step 1000;
# x 1.9e-4, v 9.2e-3, sigma 0.33 at step 3000; Ek + Es within 8.8e-4 of the
# largest total energy over the 3000 steps (rounding the whole particle state
# to FP32 after every step gives the same floor: 7.3e-4 on the energy).  That
# floor perturbs inputs and storage only; the GPU also divides p by m in FP32
# at the near-empty nodes, and lands at 1.6-9.3 times the floor on the states
# and 16 times on Ek + Es (the strain energy of the collision), 7 times with
# the FP64 islands.  The GPU is held to 20 times the floor.
C1_FLOOR = {"s1000": {"x": 8.6e-6, "v": 5.5e-4, "sigma": 3.3e-3},
            "s3000": {"x": 1.9e-4, "v": 9.2e-3, "sigma": 0.33}}
C1_ENERGY_FLOOR = 8.8e-4
C1_FACTOR = 20.0


@pytest.mark.gpu
def test_gpu_two_disks_3000_steps(gpu_lib):
    name = "disks_ulmpm_usl_linear"
    fx = _fixture(name)
    sim, states, E = RC.run_plan(name, None, gpu=True)
    # before the particles reach the nodes: FP32 rounding only
    err = RC.compare(fx, "s100", states["s100"])
    assert err["x"] < 1e-6 and err["v"] < 1e-5
    assert np.max(np.abs(states["s100"]["sigma"])) < 1e-2  # Pa; the collision stresses are ~100 Pa
    for lab, fl in C1_FLOOR.items():
        err = RC.compare(fx, lab, states[lab])
        print(f"\n{name} {lab}: " + ", ".join(f"{f} {err[f]:.2e}" for f in fl))
        for f, floor in fl.items():
            assert err[f] < C1_FACTOR * floor, f"{lab} {f}: {err[f]:.3e} >= {C1_FACTOR} x floor {floor:.1e}"
    ref = fx["E__vals"]
    assert np.array_equal(E[:, 0], fx["E__step"])
    dev = np.max(np.abs(E[:, 2:].sum(1) - ref.sum(1))) / np.max(ref.sum(1))
    print(f"\n{name} Ek + Es over 3000 steps: {dev:.2e} of the largest total")
    assert dev < C1_FACTOR * C1_ENERGY_FLOOR, f"Ek + Es: {dev:.3e}"
