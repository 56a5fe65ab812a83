"""Serving loop (include/islbm_serve.h): a solve gives the same result alone and inside a mixed
batch, retirement on convergence / cap / divergence, and admission under the device budget."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def stable(islbm, NX=32, NY=64, NZ=48, tau=0.6, **kw):
    """Parameters with relaxation time `tau` (the reference scheme is stable near 0.6)."""
    p = islbm.default_params(NX=NX, NY=NY, NZ=NZ, Uref=0.05, NDTFRC=50, init_mode=1, seed=7, perturb=0.01, **kw)
    min_size = (p.LZ - 1.0) / NZ * p.CFL
    p.Re = 3.0 * p.Uref / ((tau - 0.5) * min_size)
    return p


def alone(islbm, p, steps):
    with islbm.Solver(p) as s:
        s.step(steps)
        return s.fields(), s.force


# (precision, NX, les, tau): batched groups (FP32 / FP16, two widths, LES on/off) plus an FP64
# solve that runs on its own kernel inside the same pump
MIX = [("fp32", 32, 0.0, 0.60), ("fp32", 32, 0.0, 0.65), ("fp32", 64, 0.0, 0.90),
       ("fp16", 32, 0.0, 0.62), ("fp32", 32, 0.1, 0.60), ("fp64", 32, 0.0, 0.60)]
TOL = {"fp64": 1e-12, "fp32": 1e-6, "fp16": 1e-4}


def test_same_alone_and_in_mix(islbm_lib):
    islbm = islbm_lib
    steps = 230   # not a multiple of the chunk: the last chunk is shorter
    # grids of the hill family (NY, NX, NZ) = (2, 1, 3/2) * NX; the reference scheme needs a
    # larger tau on the finer grid (it diverges on 64 x 128 x 96 at tau = 0.6 and 0.7)
    params = [stable(islbm, NX=nx, NY=2 * nx, NZ=3 * nx // 2, tau=tau, precision=prec, les_cs=cs)
              for prec, nx, cs, tau in MIX]
    with islbm.Server(steps_per_chunk=100) as srv:
        ids = [srv.submit(p, max_steps=steps, tol=0.0, keep_fields=True) for p in params]
        srv.drain()
        for (prec, nx, cs, tau), p, rid in zip(MIX, params, ids):
            info = srv.info(rid)
            assert info["status"] == "capped", (prec, nx, info)
            assert info["steps"] == steps
            got = srv.fields(rid)
            ref, force = alone(islbm, p, steps)
            for m in ("rho", "u", "v", "w"):
                assert np.all(np.isfinite(got[m]))
            err_rho = rel_l2(got["rho"], ref["rho"])
            vel = lambda d: np.stack([d["u"], d["v"], d["w"]])
            err_u = rel_l2(vel(got), vel(ref))
            assert err_rho <= TOL[prec] and err_u <= 10 * TOL[prec], (prec, nx, cs, err_rho, err_u)
            assert abs(info["force"] - force) <= 1e-6 * abs(force) + 1e-12


def test_retirement_and_admission(islbm_lib):
    islbm = islbm_lib
    p = stable(islbm, precision="fp32")
    need = islbm.required_bytes(p) + 3 * 4 * p.NX * p.NY * p.NZ
    # room for one solve at a time: the second request waits for the first to retire
    with islbm.Server(hbm_budget_bytes=int(1.5 * need), steps_per_chunk=50) as srv:
        a = srv.submit(p, max_steps=120, tol=0.0)
        b = srv.submit(p, max_steps=10_000, tol=10.0)          # converges at its first check
        big = stable(islbm, NX=128, NY=256, NZ=64, precision="fp32")
        c = srv.submit(big, max_steps=10, tol=0.0)              # larger than the whole budget
        srv.drain()
        ia, ib, ic = srv.info(a), srv.info(b), srv.info(c)
        assert ia["status"] == "capped" and ia["steps"] == 120
        assert ib["status"] == "converged" and ib["steps"] == 50 and 0.0 <= ib["delta"] < 10.0
        assert ic["status"] == "rejected" and ic["steps"] == 0
        assert ib["t_admit"] >= ia["t_done"]
        st = srv.stats()
        assert st["bytes_in_use"] == 0
        assert st["updates"] == 170 * p.NX * p.NY * p.NZ


def test_divergent_solve_retires(islbm_lib):
    islbm = islbm_lib
    # tau close to 1/2 at this resolution diverges within a few hundred steps
    bad = stable(islbm, tau=0.5005, precision="fp32")
    good = stable(islbm, precision="fp32")
    with islbm.Server(steps_per_chunk=100) as srv:
        rb = srv.submit(bad, max_steps=3000, tol=0.0)
        rg = srv.submit(good, max_steps=300, tol=0.0, keep_fields=True)
        srv.drain()
        assert srv.info(rb)["status"] == "diverged"
        assert srv.info(rg)["status"] == "capped"
        ref, _ = alone(islbm, good, 300)
        assert rel_l2(srv.fields(rg)["rho"], ref["rho"]) <= 1e-6


def test_continuous_batching_admits_mid_flight(islbm_lib):
    """Requests submitted between pumps while others are part-way through their solve: one joins
    a running batch (new composition, new graph), one of a new width forms a new batch (graph
    capture and tuning), one arrives after a retirement, and an FP64 solve runs alongside. Each
    result equals the same parameters run alone, to the tolerances of the mixed test."""
    islbm = islbm_lib
    chunk = 50
    spec = {   # name: (precision, NX, les_cs, tau, steps cap)
        "a": ("fp32", 32, 0.0, 0.60, 300), "b": ("fp16", 32, 0.0, 0.62, 250), "c": ("fp32", 32, 0.1, 0.61, 200),
        "d": ("fp32", 64, 0.0, 0.90, 150), "e": ("fp32", 32, 0.0, 0.64, 100), "f": ("fp32", 32, 0.0, 0.66, 150),
        "g": ("fp64", 32, 0.0, 0.60, 100),
    }
    params = {}
    for i, (k, (prec, nx, cs, tau, cap)) in enumerate(spec.items()):
        params[k] = stable(islbm, NX=nx, NY=2 * nx, NZ=3 * nx // 2, tau=tau, precision=prec, les_cs=cs)
        params[k].seed = 11 + i
    ids = {}
    with islbm.Server(steps_per_chunk=chunk) as srv:
        def submit(*names):
            for k in names:
                ids[k] = srv.submit(params[k], max_steps=spec[k][4], tol=0.0, keep_fields=True)

        submit("a", "e")
        srv.pump()                        # a, e at one chunk
        submit("b", "c")                  # join while a and e are part-way
        srv.pump()
        assert srv.info(ids["a"])["status"] == "active" and srv.info(ids["b"])["status"] == "active"
        submit("d", "g")                  # a new width: its own batch, captured and tuned now
        srv.pump()
        while srv.info(ids["e"])["status"] == "active":
            srv.pump()                    # e reaches its cap and retires
        assert srv.info(ids["a"])["status"] == "active"
        submit("f")                       # admitted after that retirement, into the running batch
        srv.drain()
        vel = lambda d: np.stack([d["u"], d["v"], d["w"]])
        assert srv.info(ids["f"])["t_admit"] >= srv.info(ids["e"])["t_done"]
        for k, (prec, nx, cs, tau, cap) in spec.items():
            info = srv.info(ids[k])
            assert info["status"] == "capped" and info["steps"] == cap, (k, info)
            got = srv.fields(ids[k])
            ref, force = alone(islbm, params[k], cap)
            err_rho, err_u = rel_l2(got["rho"], ref["rho"]), rel_l2(vel(got), vel(ref))
            assert err_rho <= TOL[prec] and err_u <= 10 * TOL[prec], (k, err_rho, err_u)
            assert abs(info["force"] - force) <= 1e-6 * abs(force) + 1e-12, k


def test_checks_span_full_chunks(islbm_lib):
    """Every convergence check of a solve spans exactly steps_per_chunk of its own steps: the
    autotuner's timed steps count toward the chunk, a solve that arrives while another is at
    its cap still gets a full first interval, and a solve whose cap comes before its first full
    interval retires as capped even with a tolerance it would meet on a shorter interval."""
    islbm = islbm_lib
    chunk = 50
    p = stable(islbm, precision="fp32")
    with islbm.Server(steps_per_chunk=chunk) as srv:
        a = srv.submit(p, max_steps=120, tol=0.0)            # tuned on its first chunk
        srv.pump()
        assert srv.info(a)["steps"] == chunk
        b = srv.submit(p, max_steps=10_000, tol=10.0)        # new composition: tuned again
        c = srv.submit(p, max_steps=30, tol=10.0)            # capped before any check
        srv.drain()
        ia, ib, ic = srv.info(a), srv.info(b), srv.info(c)
        assert ia["status"] == "capped" and ia["steps"] == 120
        assert ib["status"] == "converged" and ib["steps"] == chunk, ib
        assert ic["status"] == "capped" and ic["steps"] == 30 and ic["delta"] == -1.0, ic
