"""The Karamelo-side boundary: the tlmpm/gpu and ulmpm/gpu method styles and
the GPU scheme (karamelo_gb300/styles) compiled with the unmodified Karamelo
sources and linked with libkmpm.so (karamelo_gb300/styles/Makefile), then run
on input scripts through Karamelo's own Input parser.

These tests need the Karamelo tree (located when oracle/_ref was built; they
are skipped elsewhere).  Where no CUDA device is visible, a run of a GPU
style stops at kmpm_create with Karamelo's error report; every check that
precedes the device (the style registry, the scheme hand-over, the
materials' and fixes' lowering) has run by then."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
REF_SRC_FILE = os.path.join(ROOT, "oracle", "_ref", "ref_src.txt")
STYLES = os.path.join(ROOT, "karamelo_gb300", "styles")
BIN = os.path.join(STYLES, "_build", "karamelo_gpu")


def _tree():
    if not os.path.exists(REF_SRC_FILE):
        return None
    src = open(REF_SRC_FILE).read().strip()
    return src if os.path.isdir(src) else None


pytestmark = pytest.mark.skipif(_tree() is None, reason="the Karamelo source tree is not available")


@pytest.fixture(scope="module")
def karamelo_gpu():
    from karamelo_gb300 import build
    build.build()
    subprocess.check_call(["make", "-s", "-j8", "-C", STYLES, f"REF_SRC={_tree()}"])
    assert os.path.exists(BIN)
    return BIN


def _run(exe, script, tmp_path):
    p = tmp_path / "in.mpm"
    p.write_text(script)
    r = subprocess.run([exe, "-i", str(p)], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    return r.returncode, r.stdout + r.stderr


def _has_device():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def _script(name, method, scheme):
    import ref_cases as RC
    s = RC.reference_script(name)
    return s.replace(f"method({method},", f"method({method}/gpu,").replace(f"scheme({scheme})", f"scheme({scheme}/gpu)")


@pytest.mark.parametrize("name,method,scheme", [("taylor_tlmpm_musl_cubic_jc_0.8", "tlmpm", "musl"),
                                                ("disks_ulmpm_usl_linear", "ulmpm", "usl"),
                                                ("dam_ulmpm_musl_cubic_50mm", "ulmpm", "musl"),
                                                ("tensile_tlmpm_jc_damage", "tlmpm", "musl")])
def test_gpu_styles_run_the_script_to_the_device(karamelo_gpu, tmp_path, name, method, scheme):
    rc, out = _run(karamelo_gpu, _script(name, method, scheme), tmp_path)
    if _has_device():
        assert rc == 0, out[-2000:]
    else:
        assert rc != 0 and "kmpm_create: CUDA runtime failure or no CUDA device" in out, out[-2000:]


def test_cpu_scheme_after_gpu_method_is_refused(karamelo_gpu, tmp_path):
    import ref_cases as RC
    s = RC.reference_script("taylor_tlmpm_musl_cubic_jc_0.8").replace("method(tlmpm,", "method(tlmpm/gpu,")
    rc, out = _run(karamelo_gpu, s, tmp_path)  # scheme(musl) follows method(): a CPU scheme
    assert rc != 0 and "installed a CPU scheme" in out


def test_unsupported_fix_is_refused_before_the_device(karamelo_gpu, tmp_path):
    s = _script("taylor_tlmpm_musl_cubic_jc_0.8", "tlmpm", "musl")
    s = s.replace("run(1)\n", "fix(fvp, velocity_particles, gBall1, 1, NULL, NULL)\nrun(1)\n", 1)
    rc, out = _run(karamelo_gpu, s, tmp_path)
    assert rc != 0 and "fix style velocity_particles is not supported on the GPU" in out


def test_time_dependent_body_force_is_refused(karamelo_gpu, tmp_path):
    # (a time-dependent velocity_nodes value cannot be given to the reference
    # at all: its constructor rewrites "time" as "time - dt" until no "time"
    # is left, src/fix_velocity_nodes.cpp:69-75, which never ends)
    s = _script("taylor_tlmpm_musl_cubic_jc_0.8", "tlmpm", "musl")
    s = s.replace("run(1)\n", "fix(fb, body_force, all, 2*time, NULL, NULL)\nrun(1)\n", 1)
    rc, out = _run(karamelo_gpu, s, tmp_path)
    assert rc != 0 and "must be constant" in out


def test_gpu_scheme_needs_a_gpu_method(karamelo_gpu, tmp_path):
    import ref_cases as RC
    s = RC.reference_script("taylor_tlmpm_musl_cubic_jc_0.8").replace("scheme(musl)", "scheme(musl/gpu)")
    rc, out = _run(karamelo_gpu, s, tmp_path)
    assert rc != 0 and "needs the tlmpm/gpu or ulmpm/gpu method" in out
