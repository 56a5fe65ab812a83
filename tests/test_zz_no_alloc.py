"""islbm_diagnostics_noalloc (fixed device scratch, no allocation) against islbm_diagnostics
(per-call scratch) through the C ABI, on two calls in a row. This file sorts last so that it
also runs after every other test in the same process."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def diag(lib, fn, h):
    out = (ctypes.c_double * 4)()
    st = getattr(lib, fn)(h, out)
    assert st == 0, lib.islbm_status_string(st).decode()
    return np.array(out[:])


@pytest.mark.parametrize("precision", ["fp32", "fp16", "fp64"])
def test_noalloc_matches_allocating_entry_point(islbm_lib, precision):
    islbm = islbm_lib
    L = islbm.load()
    L.islbm_diagnostics_noalloc.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
    L.islbm_diagnostics_noalloc.restype = ctypes.c_int
    # 98,304 nodes: 48 reduction blocks, the last one full; a second grid with a partial block
    for nx, ny, nz in ((32, 64, 48), (8, 16, 17)):
        p = islbm.default_params(NX=nx, NY=ny, NZ=nz, Re=60.0, Uref=0.05, precision=precision, init_mode=1, seed=11)
        with islbm.Solver(p) as s:
            for _ in range(2):   # two steps apart, two calls of each in a row
                s.step(5)
                ref1 = diag(L, "islbm_diagnostics", s._h)
                got1 = diag(L, "islbm_diagnostics_noalloc", s._h)
                got2 = diag(L, "islbm_diagnostics_noalloc", s._h)
                ref2 = diag(L, "islbm_diagnostics", s._h)
                for got, ref in ((got1, ref1), (got2, ref2)):
                    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0)
                assert np.all(np.isfinite(got1)) and abs(got1[0] - nx * ny * nz) < 1e-2 * nx * ny * nz


def test_noalloc_refuses_grids_above_its_scratch(islbm_lib):
    """A grid one plane above the fixed scratch's 33,554,432-node limit (384 x 288 x 304 =
    33,619,968 nodes, FP16 storage, 2.6 GB) is refused with a message naming the limit, while the
    allocating entry point serves it; nothing is launched for the refused call."""
    islbm = islbm_lib
    L = islbm.load()
    p = islbm.default_params(NX=384, NY=288, NZ=304, Re=60.0, Uref=0.05, precision="fp16", init_mode=0)
    with islbm.Solver(p) as s:
        out = (ctypes.c_double * 4)()
        st = L.islbm_diagnostics_noalloc(s._h, out)
        assert st == 6   # ISLBM_ERR_NOT_SUPPORTED
        msg = L.islbm_status_string(st).decode()
        assert "33554432" in msg and "islbm_diagnostics" in msg, msg
        ref = diag(L, "islbm_diagnostics", s._h)
        # the rest state held as FP16 deviations: the mass to FP16 rounding of the deviations
        assert abs(ref[0] - 384 * 288 * 304) < 1e-4 * 384 * 288 * 304
