"""islbm_diagnostics: FP64 whole-field reduction (total mass, mean streamwise momentum, kinetic
energy, maximum speed) against the same quantities computed on the host from the populations."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# D3Q19 velocity components in the reference's ordering (moments of C/evolution.h:600-607)
EX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
EY = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1])
EZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1])


def host_diagnostics(f):
    rho = f.sum(axis=0)
    j = [np.tensordot(e, f, axes=(0, 0)) for e in (EX, EY, EZ)]
    u2 = (j[0] ** 2 + j[1] ** 2 + j[2] ** 2) / rho ** 2
    return np.array([rho.sum(), j[1].sum() / rho.size, 0.5 * (rho * u2).sum(), np.sqrt(u2.max())])


@pytest.mark.parametrize("precision", ["fp64", "fp32", "fp16", "bf16"])
def test_diagnostics_match_host(islbm_lib, precision):
    islbm = islbm_lib
    # 4100 nodes per plane: the last reduction block is partial
    p = islbm.default_params(NX=32, NY=64, NZ=48, Re=60.0, Uref=0.05, precision=precision, init_mode=1, seed=3)
    with islbm.Solver(p) as s:
        n = p.NX * p.NY * p.NZ
        d0 = s.diagnostics()
        assert abs(d0["mass"] - n) <= 1e-3 * n
        s.step(40)
        d = s.diagnostics()
        f = s.populations()
        ref = host_diagnostics(f)
        got = np.array([d["mass"], d["momentum_y"], d["kinetic_energy"], d["max_speed"]])
        # same values in FP64, only the summation order differs
        np.testing.assert_allclose(got, ref, rtol=1e-11, atol=0)
        assert s.diagnostics() == d   # deterministic: block partials are added in block order


def test_diagnostics_odd_size(islbm_lib):
    islbm = islbm_lib
    p = islbm.default_params(NX=8, NY=16, NZ=17, Re=60.0, Uref=0.05, precision="fp32", init_mode=1, seed=5)
    with islbm.Solver(p) as s:
        s.step(3)
        d = s.diagnostics()
        ref = host_diagnostics(s.populations())
        np.testing.assert_allclose([d["mass"], d["momentum_y"], d["kinetic_energy"], d["max_speed"]], ref, rtol=1e-11)
