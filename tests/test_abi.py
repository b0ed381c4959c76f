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


def test_struct_layout_matches_header(gpu_lib):
    from karamelo_gb300.gpu import KmpmParams
    from karamelo_gb300.scenario import MaterialParams
    # kmpm_params: 4 ints, double, int, 2 doubles, int, 6 doubles, 3 ints
    assert ctypes.sizeof(KmpmParams) == 120
    assert ctypes.sizeof(MaterialParams) == 8 * (1 + 5 + 1 + 12 + 1 + 12 + 1 + 8 + 1 + 6)


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
