"""The oracle's flat-channel mode (ChannelFunction, C/model.h:70-73) against the plane Poiseuille
profile the reference checks in fileIO.h:250-258, v_exact = Force/(2 niu) z (LZ - z): a known
answer for the step without the hill or curved-wall rows."""
import numpy as np


def test_oracle_poiseuille(oracle_mod):
    nx, ny, nz = 8, 16, 16
    min_size = (3.036 - 1.0) / nz * 0.6
    re = 3 * 0.05 / (0.5 * min_size)   # tau = 1
    # controller off (period longer than the run): the body force keeps its initial value
    o = oracle_mod.Oracle(nx, ny, nz, re=re, ub=0.05, ndtfrc=10**9, init_mode=0, geometry=1, threads=4)
    o.step(12000)
    v = o.unique(o.get("v"))
    prof = v.mean(axis=(1, 2))
    assert np.abs(v - prof[:, None, None]).max() <= 1e-9 * np.abs(prof).max()   # uniform in x and y
    z = o.get("z").reshape(ny + 7, nz + 6)[3, 3:nz + 3]
    exact = o.force / (2.0 * o.scalar("niu")) * z * (3.036 - z)
    assert np.abs(prof - exact).max() <= 0.03 * exact.max()
