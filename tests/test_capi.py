"""CPU tests of the boundary: the C-ABI library loads, exports every symbol
include/fastem_gpu.h declares, and refuses work without a GPU instead of
falling back to the CPU."""
import ctypes
import os
import re

import numpy as np
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


def test_batch_tuning_defaults_and_bad_sizes_rejected(gpu_lib):
    """the default work-item sizes, and sizes outside [256, 16384] or not
    multiples of 128 refused before any device call"""
    import ctypes
    from fastem_gb300 import _capi as C
    t = C.BatchTuning()
    C.lib().fem_em_batch_tuning_default(ctypes.byref(t))
    assert list(t.means_chunk) == [2048] * 4 and list(t.cov_chunk) == [4096] * 4
    d = np.array([8], dtype=np.int32)
    n = np.array([1000], dtype=np.int64)
    k = np.array([3], dtype=np.int32)
    cfg = C.EmConfig()
    C.lib().fem_em_config_default(ctypes.byref(cfg))
    cfg.precision = C.PREC["fp32"]
    for bad in (100, 200, 32768, 1000):
        t.means_chunk[2] = bad
        h = ctypes.c_void_p()
        st = C.lib().fem_em_batch_create_tuned(1, C.ptr(d), C.ptr(n), C.ptr(k), ctypes.byref(cfg), ctypes.byref(t),
                                               ctypes.byref(h))
        assert st == C.FEM_ERR_BAD_ARG and not h.value
        assert b"multiples of 128" in C.lib().fem_last_error()
    t.means_chunk[2] = 2048


def test_batch_tuning_table_is_valid():
    """the autotuner's committed table holds item sizes the engine accepts"""
    from fastem_gb300.batch import TUNING_TABLE, load_tuning
    import os
    if not os.path.exists(TUNING_TABLE):
        pytest.skip("no autotuner table")
    t = load_tuning()
    for key in ("means_chunk", "cov_chunk"):
        assert len(t[key]) == 4
        assert all(256 <= v <= 16384 and v % 128 == 0 for v in t[key])
