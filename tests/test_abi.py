"""The C ABI library loads and exports every symbol include/kmpm.h declares (CPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "kmpm.h")).read()
    return sorted(set(re.findall(r"\b(kmpm_[a-z_0-9]+)\s*\(", txt)))


def test_header_and_binding_agree():
    from karamelo_gb300 import gpu
    assert sorted(gpu.EXPORTED) == declared_symbols()


def test_library_exports_all_symbols(gpu_lib):
    for name in declared_symbols():
        assert hasattr(gpu_lib, name), name


def test_struct_layout_matches_header(gpu_lib, tmp_path):
    """The ctypes mirrors have the sizes a C compiler gives the header's structs."""
    import subprocess
    from karamelo_gb300.gpu import KmpmParams, TrainOpts
    from karamelo_gb300.scenario import MaterialParams
    src = tmp_path / "sz.c"
    src.write_text('#include "kmpm.h"\n#include <stdio.h>\n'
                   'int main(void){printf("%zu %zu %zu %d %d %d %d\\n", sizeof(kmpm_params), sizeof(kmpm_material),'
                   ' sizeof(kmpm_train_opts), KMPM_MLP_NIN, KMPM_MLP_NOUT, KMPM_MLP_NPARAMS, KMPM_MLP_NNORM);'
                   'return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.check_call(["gcc", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    p, m, t, nin, nout, npar, nnorm = map(int, subprocess.check_output([str(exe)]).split())
    assert ctypes.sizeof(KmpmParams) == p
    assert ctypes.sizeof(MaterialParams) == m
    assert ctypes.sizeof(TrainOpts) == t
    from karamelo_gb300 import gpu
    assert (gpu.MLP_NIN, gpu.MLP_NOUT, gpu.MLP_NPARAMS, gpu.MLP_NNORM) == (nin, nout, npar, nnorm)


def test_create_without_device_fails_loudly(gpu_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from karamelo_gb300.gpu import KmpmError, KmpmParams
    p = KmpmParams()
    p.method, p.scheme, p.basis, p.dim = 0, 1, 1, 3
    h = ctypes.c_void_p()
    assert gpu_lib.kmpm_create(ctypes.byref(p), ctypes.byref(h)) == -2  # KMPM_ERR_CUDA
    from karamelo_gb300 import workloads as W
    sim = W.two_disks()
    with pytest.raises(KmpmError):
        sim.run(1)
