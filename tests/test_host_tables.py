"""Host precompute of the CUDA library against the oracle (no GPU needed).

Mesh, Lagrange weights, xi weights, wall distances Q and the BFL weight tables must equal the
oracle's (and so the reference's) bit for bit; the integer BFL flags and the z stencil bases
exactly.
"""
import numpy as np
import pytest

FLOAT_TABLES = ["x", "y", "z", "xi", "Q3", "Q4", "Q15", "Q16"]
WEIGHT_TABLES = ["XPara0", "XPara2", "YPara0", "YPara2", "XiF3", "XiF4", "XiF5", "XiF6", "XiF15", "XiF16",
                 "XiF17", "XiF18", "XBFL37", "XBFL38", "YBFL378", "XiBFL378", "XBFL49", "XBFL410", "YBFL4910",
                 "XiBFL4910", "YBFL15", "XiBFL15", "YBFL16", "XiBFL16"]


@pytest.mark.parametrize("grid,geometry", [((8, 16, 16), 0), ((32, 64, 48), 0), ((16, 48, 24), 0), ((8, 16, 16), 1)])
def test_tables_bit_exact(islbm_lib, oracle_mod, grid, geometry):
    nx, ny, nz = grid
    p = islbm_lib.default_params(NX=nx, NY=ny, NZ=nz, Re=700.0, Uref=0.05, NDTFRC=100, geometry=geometry)
    O = oracle_mod.Oracle(nx, ny, nz, geometry=geometry)
    for nm in FLOAT_TABLES:
        assert np.array_equal(islbm_lib.host_table(p, nm), O.get(nm)), nm
    for nm in WEIGHT_TABLES:
        for a in range(7):
            assert np.array_equal(islbm_lib.host_table(p, nm, a), O.get(nm, a)), (nm, a)
    for nm in ["BFL3", "BFL4", "BFL15", "BFL16"]:
        assert np.array_equal(islbm_lib.host_table_int(p, nm), O.get_int(nm)), nm


def test_steepness_alpha_one_is_reference(islbm_lib):
    p1 = islbm_lib.default_params(NX=8, NY=16, NZ=16, alpha=1.0)
    z1 = islbm_lib.host_table(p1, "z")
    p2 = islbm_lib.default_params(NX=8, NY=16, NZ=16, alpha=1.3)
    z2 = islbm_lib.host_table(p2, "z")
    assert not np.array_equal(z1, z2)
    # steeper footprint keeps the crest height (z at k = 2 is the wall)
    assert abs(z2.reshape(23, 22)[3, 2] - z1.reshape(23, 22)[3, 2]) < 1e-12


def test_lagrange_weights_partition_of_unity(islbm_lib):
    p = islbm_lib.default_params(NX=32, NY=64, NZ=48)
    for nm in ["XPara0", "XPara2", "YPara0", "YPara2"]:
        w = np.stack([islbm_lib.host_table(p, nm, a) for a in range(7)])[:, 3:-3]
        np.testing.assert_allclose(w.sum(axis=0), 1.0, atol=1e-13)
    xi = np.stack([islbm_lib.host_table(p, "XiF5", a) for a in range(7)]).reshape(7, 71, 54)[:, 3:-3, 3:-3]
    np.testing.assert_allclose(xi.sum(axis=0), 1.0, atol=1e-12)


def test_first_wall_spacing_is_min_size(islbm_lib):
    p = islbm_lib.default_params(NX=32, NY=64, NZ=48)
    z = islbm_lib.host_table(p, "z").reshape(71, 54)
    min_size = (3.036 - 1.0) / 48 * 0.6
    # the tanh factor is solved on the crest column (y = 0); first spacing there is minSize
    assert abs((z[3, 4] - z[3, 3]) - min_size) < 1e-12
    # the first node sits half a cell above the hill, the top node half a cell below LZ
    np.testing.assert_allclose(z[3:-3, 3] - z[3:-3, 2], min_size / 2, atol=1e-12)


def test_hill_profile_known_values(islbm_lib):
    p = islbm_lib.default_params(NX=8, NY=64, NZ=16)
    z = islbm_lib.host_table(p, "z").reshape(71, 22)
    hill = z[:, 2]
    assert abs(hill[3] - 1.0) < 1e-12           # crest at y = 0
    assert abs(hill[3 + 32]) < 1e-15            # flat floor at mid-channel
    assert np.all(hill >= -1e-15) and np.all(hill <= 1.0 + 1e-12)
