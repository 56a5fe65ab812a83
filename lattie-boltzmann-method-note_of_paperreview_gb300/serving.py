"""Request stream for the serving loop: seeded periodic-hill solve requests with Poisson
arrivals, driven through islbm.Server (continuous batching) or one after another through
islbm.Solver (sequential plain solves), with completion latency per request.

A request is drawn from its seed: the grid (three sizes of the hill family, named streamwise x
spanwise x wall-normal), the relaxation time (hence Re_h on that grid), the hill steepness
alpha and the storage format. Relaxation times are drawn from a range in which the reference
step is stable on that grid: [0.6, 0.68] on 64x32x48, [0.9, 1.0] on 128x64x96, [1.0, 1.1] on
256x128x192 (the scheme needs a larger tau on finer grids; Re_h in the thousands, tau near 1/2,
diverges on all three). The steepness is drawn uniformly from ALPHA_RANGE: the reference step
diverges within a thousand steps for many hill shapes, in narrow bands scattered over
[0.5, 1.5] (scans in steps of 0.05, then 0.01 near the stable values, over the three grids and
their tau ranges); [0.71, 0.76] is the widest interval stable at every scanned point of every
grid and tau of the stream.

Convergence: a solve retires when delta = sqrt(mean |u - u_prev|^2)/U_b over CHUNK = 1000
steps falls below TOL, or at its grid's step cap. From a seeded perturbed start the flow keeps
a slow transient with controller-driven oscillations: delta falls to a few 1e-2 within
10-20 thousand steps on the two smaller grids and stays above 1e-2 over 40 thousand steps, so
TOL is 5e-2 (a tolerance of 1e-5 is not reached within any practical cap).
"""
import time

import numpy as np

import islbm

# (streamwise NY, spanwise NX, wall-normal NZ), the step cap and the stable tau range of each grid
GRIDS = [((64, 32, 48), 20000, (0.6, 0.68)), ((128, 64, 96), 16000, (0.9, 1.0)), ((256, 128, 192), 2000, (1.0, 1.1))]
ALPHA_RANGE = (0.71, 0.76)
CHUNK = 1000
TOL = 5e-2


def min_size(NZ, LZ=3.036, CFL=0.6):
    return (LZ - 1.0) / NZ * CFL


def make_requests(n, seed=2024, mean_gap=0.5, precisions=("fp32", "fp16"), tol=TOL, cap_scale=1.0,
                  alpha_range=ALPHA_RANGE):
    """n requests with exponential inter-arrival gaps (mean `mean_gap` seconds)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(mean_gap)
        (ny, nx, nz), cap, (tlo, thi) = GRIDS[rng.integers(len(GRIDS))]
        tau = rng.uniform(tlo, thi)
        alpha = float(rng.uniform(*alpha_range))
        prec = precisions[rng.integers(len(precisions))]
        ub = 0.05
        re = 3.0 * ub / ((tau - 0.5) * min_size(nz))
        out.append(dict(arrival=t, NX=nx, NY=ny, NZ=nz, Re=re, Uref=ub, alpha=alpha, precision=prec,
                        seed=int(rng.integers(1, 2**31)), max_steps=max(1, int(cap * cap_scale)), tol=tol))
    return out


def params_of(req, **override):
    kw = dict(NX=req["NX"], NY=req["NY"], NZ=req["NZ"], Re=req["Re"], Uref=req["Uref"], alpha=req["alpha"],
              precision=req["precision"], seed=req["seed"], init_mode=1, perturb=0.01, NDTFRC=100)
    kw.update(override)
    return islbm.default_params(**kw)


def _stats(lat):
    lat = np.sort(np.asarray(lat))
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "max_s": float(lat.max())}


def run_server(reqs, steps_per_chunk=CHUNK, hbm_budget_bytes=150 << 30, device=0, keep=()):
    """Submit each request at its arrival time, pump until all retired. Returns a summary and the
    per-request info (fields of the request indices in `keep` are kept)."""
    with islbm.Server(device=device, hbm_budget_bytes=hbm_budget_bytes, steps_per_chunk=steps_per_chunk) as srv:
        t0 = time.monotonic()
        pending = list(range(len(reqs)))
        ids, lag = {}, {}
        infos, fields = {}, {}
        while True:
            now = time.monotonic() - t0
            while pending and reqs[pending[0]]["arrival"] <= now:
                i = pending.pop(0)
                r = reqs[i]
                ids[i] = srv.submit(params_of(r), r["max_steps"], r["tol"], keep_fields=i in keep)
                lag[i] = (time.monotonic() - t0) - r["arrival"]
            active, queued = srv.pump()
            if active == 0 and queued == 0:
                if not pending:
                    break
                time.sleep(max(0.0, reqs[pending[0]]["arrival"] - (time.monotonic() - t0)))
        wall = time.monotonic() - t0
        lat = []
        for i, rid in ids.items():
            inf = srv.info(rid)
            infos[i] = inf
            lat.append(inf["t_done"] - inf["t_submit"] + lag[i])
            if i in keep:
                fields[i] = srv.fields(rid)
        st = srv.stats()
    first = min(r["arrival"] for r in reqs)
    return {"updates": st["updates"], "wall_s": wall, "busy_s": st["busy_seconds"],
            "mlups": st["updates"] / max(wall - first, 1e-9) / 1e6, "latency": _stats(lat),
            "status": {s: sum(1 for v in infos.values() if v["status"] == s) for s in islbm.SOLVE_STATUS.values()}}, \
        infos, fields


def run_sequential(reqs, steps_per_check=CHUNK, device=0):
    """The same requests as plain solves, one at a time in arrival order (each starts at its arrival or
    when the previous one ends), with the same convergence check every `steps_per_check` steps."""
    t0 = time.monotonic()
    lat, updates = [], 0
    per_grid = {}
    for r in reqs:
        now = time.monotonic() - t0
        if now < r["arrival"]:
            time.sleep(r["arrival"] - now)
        t_start = time.monotonic()
        with islbm.Solver(params_of(r, device=device)) as s:
            n = r["NX"] * r["NY"] * r["NZ"]
            f = s.fields()   # initial state, as the server's first snapshot
            prev = np.stack([f["u"], f["v"], f["w"]])
            steps = 0
            while steps < r["max_steps"]:
                k = min(steps_per_check, r["max_steps"] - steps)
                s.step(k)
                steps += k
                f = s.fields()
                u = np.stack([f["u"], f["v"], f["w"]])
                delta = np.sqrt(np.sum((u - prev) ** 2) / n) / r["Uref"]
                # the server's retirement rules: converged, or diverged (non-finite or delta > 1000)
                if delta < r["tol"] or not (delta <= 1e3):
                    break
                prev = u
            updates += steps * n
        g = per_grid.setdefault("%dx%dx%d" % (r["NY"], r["NX"], r["NZ"]), {"requests": 0, "updates": 0, "seconds": 0.0})
        g["requests"] += 1
        g["updates"] += steps * n
        g["seconds"] += time.monotonic() - t_start
        lat.append(time.monotonic() - t0 - r["arrival"])
    wall = time.monotonic() - t0
    first = min(r["arrival"] for r in reqs)
    for g in per_grid.values():   # each grid's requests run alone: their own rate, set-up included
        g["mlups_alone"] = g["updates"] / max(g["seconds"], 1e-9) / 1e6
    return {"updates": updates, "wall_s": wall, "mlups": updates / max(wall - first, 1e-9) / 1e6,
            "latency": _stats(lat), "per_grid": per_grid}
