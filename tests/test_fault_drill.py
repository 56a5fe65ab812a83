"""Failure detection without a GPU fault: the tiled kernel's bounded pipeline wait runs out
(the copies of one plane are never started), the kernel completes, islbm_sync reports the
fault, and the device context stays usable for the next solve."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_timed_out_wait_is_reported_and_context_survives(islbm_lib):
    islbm = islbm_lib
    L = islbm.load()
    kw = dict(NX=32, NY=64, NZ=48, Re=58.9, Uref=0.05, precision="fp32", kernel=islbm.KERNEL_TILED)
    with islbm.Solver(islbm.default_params(**kw)) as s:
        assert L.islbm_fault_drill(s._h, 10) == 0
        s.step(1)
        st = L.islbm_sync(s._h)
        assert st == 2   # ISLBM_ERR_CUDA
        assert b"timed out" in L.islbm_status_string(st)
    # a new solve on the same device works
    with islbm.Solver(islbm.default_params(**kw)) as s:
        s.step(5)
        s.sync()
        assert s.healthy()


def test_drill_arguments(islbm_lib):
    islbm = islbm_lib
    L = islbm.load()
    with islbm.Solver(islbm.default_params(NX=32, NY=64, NZ=48, Re=58.9, precision="fp32")) as s:
        assert L.islbm_fault_drill(s._h, 48) == 1
        assert L.islbm_fault_drill(s._h, -2) == 1
        assert L.islbm_fault_drill(s._h, -1) == 0
    assert L.islbm_fault_drill(ctypes.c_void_p(), 3) == 1
