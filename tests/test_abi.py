"""C ABI of libislbm_gb300.so: every symbol declared in include/*.h is exported, argument checks
return status codes, and sizes are computed without a device."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    inc = os.path.join(ROOT, "include")
    src = "".join(open(os.path.join(inc, f)).read() for f in sorted(os.listdir(inc)) if f.endswith(".h"))
    return sorted(set(re.findall(r"ISLBM_API\s+(?:const\s+)?\w+\s*\*?\s*(islbm_\w+)\s*\(", src)))


def test_all_declared_symbols_exported(islbm_lib):
    lib = ctypes.CDLL(islbm_lib.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n


def test_invalid_parameters_rejected(islbm_lib):
    L = islbm_lib.load()
    for bad in [dict(NX=0), dict(NZ=4), dict(Re=-1.0), dict(precision=9), dict(NDTFRC=0), dict(bfl_mode=3)]:
        p = islbm_lib.default_params(**bad)
        n = ctypes.c_size_t()
        assert L.islbm_required_bytes(ctypes.byref(p), ctypes.byref(n)) == 1, bad
        h = ctypes.c_void_p()
        assert L.islbm_init(ctypes.byref(p), ctypes.byref(h)) == 1, bad
        assert not h.value


def test_null_handle_is_error(islbm_lib):
    L = islbm_lib.load()
    assert L.islbm_step(None, 1) == 1
    assert L.islbm_destroy(None) == 1
    assert L.islbm_sync(None) == 1


def test_required_bytes_scales_with_precision(islbm_lib):
    sizes = {}
    for prec in ["fp64", "fp32", "fp16", "bf16"]:
        p = islbm_lib.benchmark_params("hill256", precision=prec)
        sizes[prec] = islbm_lib.required_bytes(p)
    n = 128 * 256 * 192
    assert sizes["fp32"] >= 2 * 19 * n * 4
    assert sizes["fp16"] < sizes["fp32"] < sizes["fp64"]
    assert sizes["fp16"] == sizes["bf16"]


def test_hbm_budget_refusal(islbm_lib):
    p = islbm_lib.benchmark_params("hill256", precision="fp32", hbm_budget_bytes=1 << 20)
    with pytest.raises(islbm_lib.IslbmError) as e:
        islbm_lib.Solver(p)
    assert e.value.status == 4


def test_status_strings(islbm_lib):
    L = islbm_lib.load()
    for s in range(8):
        assert L.islbm_status_string(s)


def test_server_argument_checks(islbm_lib):
    L = islbm_lib.load()
    s = ctypes.c_void_p()
    assert L.islbm_server_create(0, 0, 0, ctypes.byref(s)) == 1      # steps_per_chunk < 1
    assert L.islbm_server_pump(None, None, None) == 1
    assert L.islbm_server_destroy(None) == 1
    assert L.islbm_server_submit(None, None, 1, 0.0, 0, None) == 1
