"""Bit-exact check of the oracle against the reference compiled for host cores.

Runs only where oracle/_ref holds a reference build (this needs the reference sources;
build one with `python oracle/ref_build.py --nx 8 --ny 16 --nz 16 --ndtfrc 10`).
"""
import numpy as np
import pytest

from oracle.oracle import Reference, reference_library


@pytest.mark.parametrize("massk", [0, 5])
def test_bit_exact_against_reference(oracle_mod, massk):
    path = reference_library(8, 16, 16, 700.0, 10, massk)
    if path is None:
        pytest.skip("reference build not present (needs the reference sources)")
    R = Reference(path, mode=1, seed=1234)
    O = oracle_mod.Oracle(8, 16, 16, ndtfrc=10, mass_interval=massk)
    for q in range(19):
        assert np.array_equal(R.get("f", q), O.get("f", q))
    for s in range(30):
        R.step(1)
        O.step(1)
        assert R.force == O.force
        for q in range(19):
            assert np.array_equal(R.get("f", q), O.get("f", q)), (s, q)
        for nm in ("rho", "u", "v", "w"):
            assert np.array_equal(R.get(nm), O.get(nm)), (s, nm)
