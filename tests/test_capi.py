"""CPU tests of the boundary: the C-ABI library loads, exports every symbol
include/fastem_gpu.h declares, and refuses work without a GPU instead of
falling back to the CPU."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "fastem_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fem_[a-z0-9_]+)\s*\(", txt)))


def test_header_and_binding_agree():
    from fastem_gb300 import _capi
    assert declared_symbols() == sorted(_capi.EXPORTS)


def test_library_exports_every_declared_symbol(gpu_lib):
    for name in declared_symbols():
        assert hasattr(gpu_lib, name), name


def test_api_version(gpu_lib):
    assert gpu_lib.fem_api_version() == 1


def test_no_cpu_fallback_without_gpu(gpu_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from fastem_gb300 import _capi as C
    cfg = C.EmConfig()
    gpu_lib.fem_em_config_default(ctypes.byref(cfg))
    h = ctypes.c_void_p()
    for prec in ("fp64", "fp32"):
        cfg.precision = C.PREC[prec]
        st = gpu_lib.fem_em_create(8, 1000, 4, ctypes.byref(cfg), ctypes.byref(h))
        assert st == C.FEM_ERR_NO_DEVICE and not h.value
    kc = C.KmConfig()
    gpu_lib.fem_km_config_default(ctypes.byref(kc))
    kc.precision = C.PREC["fp32"]
    st = gpu_lib.fem_km_create(8, 1000, 4, ctypes.byref(kc), ctypes.byref(h))
    assert st == C.FEM_ERR_NO_DEVICE


def test_bad_arguments_rejected(gpu_lib):
    from fastem_gb300 import _capi as C
    h = ctypes.c_void_p()
    assert gpu_lib.fem_em_create(0, 10, 2, None, ctypes.byref(h)) == C.FEM_ERR_BAD_ARG
    assert gpu_lib.fem_em_create(4, 10, 0, None, ctypes.byref(h)) == C.FEM_ERR_BAD_ARG
    assert gpu_lib.fem_em_create(4, 0, 2, None, ctypes.byref(h)) == C.FEM_ERR_BAD_ARG
    assert gpu_lib.fem_em_set_params(None, None, None, None) == C.FEM_ERR_BAD_ARG
    assert gpu_lib.fem_km_compute_mse_and_correct(None, None, None, None) == C.FEM_ERR_BAD_ARG
    assert "null" in C.last_error()


def test_km_repair_modes_and_rng_state_arguments(gpu_lib):
    """The k-means repair modes are checked before any device work, and the
    repair-generator state calls refuse a missing handle."""
    from fastem_gb300 import _capi as C
    kc = C.KmConfig()
    gpu_lib.fem_km_config_default(ctypes.byref(kc))
    assert kc.repair == 1                                   # FEM_KM_REPAIR_RANDOM
    kc.precision, kc.repair = C.PREC["fp32"], 3
    h = ctypes.c_void_p()
    assert gpu_lib.fem_km_create(8, 1000, 4, ctypes.byref(kc), ctypes.byref(h)) == C.FEM_ERR_BAD_ARG
    assert "repair" in C.last_error() and not h.value
    assert gpu_lib.fem_km_set_rng_state(None, b"1 2 3") == C.FEM_ERR_BAD_ARG
    buf = ctypes.create_string_buffer(16)
    assert gpu_lib.fem_km_get_rng_state(None, buf, 16) == C.FEM_ERR_BAD_ARG


def test_python_binding_raises_when_library_missing(monkeypatch, tmp_path):
    from fastem_gb300 import _capi
    monkeypatch.setattr(_capi, "_LIB", None)
    monkeypatch.setattr(_capi, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(ImportError):
        _capi.lib()
