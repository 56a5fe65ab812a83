"""Checkpoint / restart in the reference's file format (OutputData / InitialUsingBkpData,
C/fileIO.h:52-67, 262-266, 298-354): exact resume, and files laid out as the reference writes
them (here produced from the oracle's padded arrays) read back into the GPU solver."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_resume_is_exact(islbm_lib, tmp_path, precision):
    islbm = islbm_lib
    kw = dict(NX=32, NY=64, NZ=48, Re=58.9, Uref=0.05, NDTFRC=20, precision=precision, init_mode=1, seed=4,
              mass_interval=9)
    with islbm.Solver(islbm.default_params(**kw)) as a:
        a.step(37)
        a.checkpoint_write(str(tmp_path))
        a.step(30)
        fa, force_a = a.populations(), a.force
    names = sorted(os.listdir(tmp_path))
    assert "0_force.dat" in names and "f18_0.bin" in names and "rho_0.bin" in names
    assert os.path.getsize(tmp_path / "f0_0.bin") == 8 * (32 + 7) * (64 + 7) * (48 + 6)
    with islbm.Solver(islbm.default_params(**kw)) as b:
        b.checkpoint_read(str(tmp_path))
        assert b.scalars()["steps"] == 37
        b.step(30)
        np.testing.assert_array_equal(b.populations(), fa)
        assert b.force == force_a


def test_reads_reference_files(islbm_lib, oracle_mod, tmp_path):
    islbm = islbm_lib
    nx, ny, nz = 8, 16, 16
    o = oracle_mod.Oracle(nx, ny, nz, re=700.0, ub=0.05, ndtfrc=10, init_mode=1, seed=1234)
    o.step(12)
    # the reference's OutputData: raw doubles of the padded (NYD6, NZ6, NX6) arrays
    for q in range(19):
        np.ascontiguousarray(o.get("f", q), dtype=np.float64).tofile(tmp_path / ("f%d_0.bin" % q))
    for m in ("rho", "u", "v", "w"):
        np.ascontiguousarray(o.get(m), dtype=np.float64).tofile(tmp_path / ("%s_0.bin" % m))
    (tmp_path / "0_force.dat").write_text("%.15f" % o.force)
    p = islbm.default_params(NX=nx, NY=ny, NZ=nz, Re=700.0, Uref=0.05, NDTFRC=10, precision="fp64")
    with islbm.Solver(p) as s:
        s.checkpoint_read(str(tmp_path))
        f = s.populations()
        for q in range(19):
            np.testing.assert_array_equal(f[q], o.unique(o.get("f", q)))
        np.testing.assert_array_equal(s.fields()["v"], o.unique(o.get("v")))
        assert s.force == float("%.15f" % o.force)
