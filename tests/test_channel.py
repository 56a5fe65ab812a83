"""Flat-channel mode (ChannelFunction, C/model.h:70-73): GPU FP64 against the oracle, and the
plane Poiseuille profile the reference checks in fileIO.h:250-258,
v_exact = Force/(2 niu) z (LZ - z), at steady state under a fixed body force."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_channel_matches_oracle(islbm_lib, oracle_mod):
    islbm = islbm_lib
    nx, ny, nz = 8, 16, 16
    p = islbm.default_params(NX=nx, NY=ny, NZ=nz, Re=20.0, Uref=0.05, NDTFRC=10, precision="fp64", init_mode=1,
                             seed=3, geometry=1)
    with islbm.Solver(p) as s:
        s.step(40)
        g = s.fields()
        force = s.force
    o = oracle_mod.Oracle(nx, ny, nz, re=20.0, ub=0.05, ndtfrc=10, init_mode=1, seed=3, geometry=1)
    o.step(40)
    assert rel_l2(g["rho"], o.unique(o.get("rho"))) <= 1e-12
    # the velocity vector (the spanwise component alone is at the noise level of the start)
    vel = lambda d: np.stack([d[c] for c in "uvw"])
    assert rel_l2(vel(g), vel({c: o.unique(o.get(c)) for c in "uvw"})) <= 1e-12
    assert abs(force - o.force) <= 1e-12 * abs(o.force)
    # the same wall rows as the oracle (the flat wall still gets BFL rows where a departure
    # point falls below it)
    for n in ("BFL3", "BFL4", "BFL15", "BFL16"):
        np.testing.assert_array_equal(islbm.host_table_int(p, n), o.get_int(n))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_poiseuille(islbm_lib, precision):
    islbm = islbm_lib
    nx, ny, nz = 8, 16, 16
    min_size = (3.036 - 1.0) / nz * 0.6
    tau = 1.0
    re = 3 * 0.05 / ((tau - 0.5) * min_size)
    # controller off (period longer than the run): the force stays at its initial value
    p = islbm.default_params(NX=nx, NY=ny, NZ=nz, Re=re, Uref=0.05, NDTFRC=10**9, precision=precision, init_mode=0,
                             geometry=1)
    with islbm.Solver(p) as s:
        s.step(12000)
        v = s.fields()["v"]
        force = s.force
        niu = s.constants()["niu"]
    z = islbm.host_table(p, "z").reshape(ny + 7, nz + 6)[3, 3:nz + 3]
    exact = force / (2.0 * niu) * z * (3.036 - z)
    prof = v.mean(axis=(1, 2))
    assert np.abs(v - prof[:, None, None]).max() <= 1e-6 * np.abs(prof).max()   # uniform in x and y
    assert np.abs(prof - exact).max() <= 0.03 * exact.max()
