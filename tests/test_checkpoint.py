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


@pytest.mark.parametrize("gradients", [False, True])
def test_statistics_resume_is_exact(islbm_lib, tmp_path, gradients):
    """A run that checkpoints with statistics running and resumes gives the same time means as the
    run that never stopped; the statistics files are the reference's (Launch_OutputTB /
    InitialTBUsingBkpData, C/fileIO.h:356-500): accu.dat and <NAME>/<NAME>_<rank>.bin of
    NZ x (NY+1) x (NX+1) doubles."""
    islbm = islbm_lib
    kw = dict(NX=32, NY=64, NZ=48, Re=58.9, Uref=0.05, NDTFRC=20, precision="fp64", init_mode=1, seed=5)
    names = islbm.STATS if gradients else islbm.STATS[:24]

    def sample(s, n):
        for _ in range(n):
            s.step(3)
            s.stats_accumulate()

    with islbm.Solver(islbm.default_params(**kw)) as a:
        if gradients:
            a.stats_gradients(True)
        a.stats_reset()
        sample(a, 4)
        a.checkpoint_write(str(tmp_path))
        sample(a, 5)
        ref = {n: a.stats_mean(n) for n in names}
        assert a.stats_samples() == 9
    st = tmp_path / "statistics"
    assert (st / "accu.dat").read_text().strip() == "4"
    assert os.path.getsize(st / "U" / "U_0.bin") == 8 * 48 * 65 * 33
    assert (st / "DUDX2" / "DUDX2_0.bin").exists() == gradients
    # the duplicated periodic end nodes hold copies of the first ones
    u = np.fromfile(st / "U" / "U_0.bin").reshape(48, 65, 33)
    np.testing.assert_array_equal(u[:, 64, :], u[:, 0, :])
    np.testing.assert_array_equal(u[:, :, 32], u[:, :, 0])
    with islbm.Solver(islbm.default_params(**kw)) as b:
        if gradients:
            b.stats_gradients(True)
        b.checkpoint_read(str(tmp_path))
        assert b.stats_samples() == 4
        sample(b, 5)
        assert b.stats_samples() == 9
        for n in names:
            np.testing.assert_array_equal(b.stats_mean(n), ref[n], err_msg=n)
