"""The serving request stream (serving.py, no GPU): seeded and reproducible, Poisson arrivals
with the stated mean gap, every request inside its grid's stable relaxation-time range and the
stable hill-steepness interval, with its grid's step cap, and parameters that carry the request
through to islbm_params."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def serving(islbm_lib):
    import serving as mod
    return mod


def test_stream_is_reproducible_and_poisson(serving):
    a = serving.make_requests(64, seed=2024, mean_gap=0.5)
    b = serving.make_requests(64, seed=2024, mean_gap=0.5)
    assert a == b
    assert serving.make_requests(64, seed=2025, mean_gap=0.5) != a
    t = np.array([r["arrival"] for r in a])
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert np.all(gaps > 0)
    # exponential gaps: sample mean of 64 within four standard errors of 0.5 s
    assert abs(gaps.mean() - 0.5) < 4 * 0.5 / np.sqrt(64)
    # a long stream: the mean converges, and the coefficient of variation is that of an exponential
    g = np.diff([r["arrival"] for r in serving.make_requests(4000, seed=7, mean_gap=0.5)])
    assert abs(g.mean() - 0.5) < 0.03 and abs(g.std() / g.mean() - 1.0) < 0.08


def test_requests_stay_in_the_stable_ranges(serving):
    reqs = serving.make_requests(500, seed=11)
    grids = {g: (cap, tau) for g, cap, tau in serving.GRIDS}
    seen = set()
    for r in reqs:
        g = (r["NY"], r["NX"], r["NZ"])
        assert g in grids
        seen.add(g)
        cap, (tlo, thi) = grids[g]
        tau = 0.5 + 3.0 * r["Uref"] / (r["Re"] * serving.min_size(r["NZ"]))
        assert tlo - 1e-12 <= tau <= thi + 1e-12
        assert serving.ALPHA_RANGE[0] <= r["alpha"] <= serving.ALPHA_RANGE[1]
        assert r["max_steps"] == cap
        assert r["precision"] in ("fp32", "fp16")
        assert r["tol"] == serving.TOL
    assert seen == set(grids)   # every grid of the mix occurs


def test_params_carry_the_request(serving, islbm_lib):
    r = serving.make_requests(3, seed=5)[2]
    p = serving.params_of(r)
    assert (p.NX, p.NY, p.NZ) == (r["NX"], r["NY"], r["NZ"])
    assert p.Re == pytest.approx(r["Re"]) and p.Uref == pytest.approx(r["Uref"])
    assert p.alpha == pytest.approx(r["alpha"]) and p.seed == r["seed"]
    assert p.precision == {"fp32": islbm_lib.FP32, "fp16": islbm_lib.FP16_DEV}[r["precision"]]
    q = serving.params_of(r, precision="fp64")
    assert q.precision == islbm_lib.FP64
