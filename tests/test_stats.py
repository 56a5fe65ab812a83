"""Time-averaged statistics (MeanVars, C/statistics.h:122-174) against the same sums taken on the
host from islbm_fields after each sampled step, for FP64 and FP32 fields."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def host_quantities(f):
    u, v, w = f["u"], f["v"], f["w"]
    p = 1.0 / 3.0 * f["rho"] - 1.0 / 3.0
    return {"U": u, "V": v, "W": w, "P": p, "UU": u * u, "UV": u * v, "UW": u * w, "VV": v * v, "VW": v * w,
            "WW": w * w, "PU": p * u, "PV": p * v, "PW": p * w, "PP": p * p, "KT": 0.5 * (u * u + v * v + w * w),
            "UUU": u * u * u, "UUV": u * u * v, "UUW": u * u * w, "VVU": v * v * u, "VVV": v * v * v,
            "VVW": v * v * w, "WWU": w * w * u, "WWV": w * w * v, "WWW": w * w * w}


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_stats_match_host_sums(islbm_lib, precision):
    islbm = islbm_lib
    p = islbm.default_params(NX=32, NY=64, NZ=48, Re=58.9, Uref=0.05, precision=precision, init_mode=1, seed=21)
    with islbm.Solver(p) as s:
        acc = None
        s.stats_reset()
        for k in range(5):
            s.step(7)
            s.stats_accumulate()
            q = host_quantities(s.fields())
            acc = q if acc is None else {n: acc[n] + q[n] for n in q}
        assert s.stats_samples() == 5
        for name in islbm.STATS[:24]:   # the MeanVars quantities (gradients not enabled)
            got = s.stats_mean(name)
            ref = acc[name] / 5
            scale = np.abs(ref).max()
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-14 * scale, err_msg=name)
        prof = s.stats_profile("V", 10)
        np.testing.assert_allclose(prof, (acc["V"] / 5)[:, 10, :].mean(axis=1), rtol=1e-12)
        ref_layout = s.stats_mean("U", layout=islbm.LAYOUT_REFERENCE)
        assert ref_layout.shape == (p.NY + 7, p.NZ + 6, p.NX + 7)
        np.testing.assert_array_equal(ref_layout[3:-4, 3:-3, 3:-4].transpose(1, 0, 2), s.stats_mean("U"))
        s.stats_reset()
        assert s.stats_samples() == 0


def test_wall_shear_of_poiseuille(islbm_lib):
    """Flat channel at steady state: the force balance gives nu dv/dz = F LZ / 2 at the wall, so
    cf = F LZ / Ub^2 on every row."""
    islbm = islbm_lib
    nx, ny, nz = 8, 16, 16
    re = 3 * 0.05 / (0.5 * (3.036 - 1.0) / nz * 0.6)   # tau = 1
    p = islbm.default_params(NX=nx, NY=ny, NZ=nz, Re=re, Uref=0.05, NDTFRC=10**9, precision="fp64", init_mode=0,
                             geometry=1)
    with islbm.Solver(p) as s:
        s.step(12000)
        s.stats_reset()
        s.stats_accumulate()
        cf = s.stats_wall_shear()
        force = s.force
    exact = force * 3.036 / 0.05 ** 2
    assert cf.shape == (ny,)
    assert np.abs(cf - exact).max() <= 0.03 * exact


def lagrange_slope(zn, m, t):
    s = 0.0
    for l in range(5):
        if l == m:
            continue
        p = 1.0 / (zn[m] - zn[l])
        for i in range(5):
            if i != m and i != l:
                p *= (t - zn[i]) / (zn[m] - zn[i])
        s += p
    return s


def host_gradients(islbm, p, f):
    """MeanDerivatives' nine squared gradients (C/statistics.h:176-222) from the fields."""
    nx, ny, nz = p.NX, p.NY, p.NZ
    dx, dy = p.LX / nx, p.LY / ny
    z = islbm.host_table(p, "z").reshape(ny + 7, nz + 6)[3:ny + 3, 3:nz + 3]   # (y, z)
    out = {}
    for c, a in (("U", f["u"]), ("V", f["v"]), ("W", f["w"])):
        gx = (8 * (np.roll(a, -1, 2) - np.roll(a, 1, 2)) - (np.roll(a, -2, 2) - np.roll(a, 2, 2))) / 12 / dx
        gy = (8 * (np.roll(a, -1, 1) - np.roll(a, 1, 1)) - (np.roll(a, -2, 1) - np.roll(a, 2, 1))) / 12 / dy
        gz = np.zeros_like(a)
        for k in range(nz):
            nb = min(max(k - 2, 0), nz - 5)
            for y in range(ny):
                zn = z[y, nb:nb + 5]
                w = [lagrange_slope(zn, m, z[y, k]) for m in range(5)]
                gz[k, y, :] = sum(w[m] * a[nb + m, y, :] for m in range(5))
        out["D%sDX2" % c], out["D%sDY2" % c], out["D%sDZ2" % c] = gx * gx, gy * gy, gz * gz
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gradient_stats(islbm_lib, precision):
    islbm = islbm_lib
    p = islbm.default_params(NX=32, NY=64, NZ=48, Re=58.9, Uref=0.05, precision=precision, init_mode=1, seed=8)
    with islbm.Solver(p) as s:
        s.stats_gradients(True)
        s.stats_reset()
        acc = None
        for _ in range(3):
            s.step(5)
            s.stats_accumulate()
            g = host_gradients(islbm, p, s.fields())
            acc = g if acc is None else {n: acc[n] + g[n] for n in g}
        for name, ref in acc.items():
            np.testing.assert_allclose(s.stats_mean(name), ref / 3, rtol=1e-9, atol=1e-12 * np.abs(ref).max(),
                                       err_msg=name)
        np.testing.assert_allclose(s.stats_mean("V"), s.stats_mean("V"))   # the base quantities stay
