"""Benchmark of the ISLBM periodic-hill step on GB300 (one JSON line on rank 0).

Workload: the 256x128x192 hill case (streamwise NY = 256, spanwise NX = 128, wall-normal
NZ = 192; 6.29 M nodes), Re_h = 2800, Smagorinsky C_s = 0.1, U_b = 0.05, seeded perturbed
equilibrium start, forcing controller on. One step = one fused kernel launch over all nodes.
  value      MLUPS of the plain FP32 step, populations resident in HBM (the two FP32
             population buffers, 2 x 478 MB, exceed the 129 MB L2, so no flush is needed)
  e2e        MLUPS through the C ABI from host buffers: the initial populations are uploaded
             from host memory, and every 100 steps rho, u, v, w are read back (the reference
             main loop's mass-check cadence), all inside the timed region
  roofline   achieved HBM GB/s of the step kernel from the algorithmic bytes (2 x 19 x 4 B
             per node) over the CUDA-event time per launch, against the measured copy peak
  mixed      the same for FP16 / BF16 deviation storage (2 x 19 x 2 B per node)
  cpu_baseline  the CPU oracle (a restatement of the reference's step) on a bounded sample
  serve      a seeded request stream (Poisson arrivals) over three hill grids through the
             serving loop (continuous batching, one batched launch per step, CUDA graphs),
             against the same requests as sequential plain solves: aggregate MLUPS, p50/p99
             completion latency, and the error of sampled results against plain FP64 solves
--impl reference times that CPU path alone (all host threads) on the same workload.
Multi-GPU: replicas only (each rank runs its own solve; value is the sum over ranks).
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "lattie-boltzmann-method-note_of_paperreview_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "ISLBM MLUPS & %HBM peak, mixed vs plain FP32 at stated err; serve p50/p99"
# DRAM bytes of one launch of the FP32 step on this workload, from an ncu capture of the same
# kernel (dram__bytes_read.sum + dram__bytes_write.sum: 590.6 MB + 433.0 MB)
NCU_TRAFFIC_BYTES = 1023.6e6
CASE = dict(NX=128, NY=256, NZ=192, Re=2800.0, Uref=0.05, NDTFRC=100, les_cs=0.1)
WORKLOAD = "periodic hill 256x128x192 (streamwise x spanwise x wall-normal), Re_h 2800, LES Cs 0.1, Ub 0.05"


def measured_peak_gbs():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 20 ms; the summary keeps the samples taken
    between mark_start() and mark_end() (the timed region), by their timestamps."""
    QUERY = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.t0 = self.t1 = None
        fd, self.path = tempfile.mkstemp(prefix="islbm_clocks_", suffix=".csv")
        os.close(fd)

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "20"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
            # wait (at most 5 s) until the sampler is running, so the timed region is covered
            deadline = time.time() + 5.0
            while time.time() < deadline and os.path.getsize(self.path) == 0:
                time.sleep(0.05)
        except Exception:
            self.proc = None
        return self

    def mark_start(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def __del__(self):
        try:
            os.unlink(self.path)
        except Exception:
            pass

    def summary(self):
        import datetime
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 10:
                    try:
                        t = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                    except ValueError:
                        t = None
                    rows.append((t, parts[1:]))
        except Exception:
            pass
        window = "timed region"
        if self.t0 is not None and self.t1 is not None:
            inside = [r for t, r in rows if t is not None and self.t0 <= t <= self.t1]
            if not inside:   # shorter than the sampling interval: the samples next to it
                window = "within 50 ms of the timed region"
                inside = [r for t, r in rows if t is not None and self.t0 - 0.05 <= t <= self.t1 + 0.05]
            rows = inside
        else:
            rows = [r for _, r in rows]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "").isdigit())
        mx = max((float(r[2]) for r in rows if r[2].replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows), "window": window}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def time_steps(islbm, torch, solver, steps):
    """CUDA-event time of `steps` launches on the solver's own stream (ms)."""
    stream = torch.cuda.ExternalStream(solver.stream_handle())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    solver.step(steps)
    ev1.record(stream)
    ev1.synchronize()
    return ev0.elapsed_time(ev1)


def device_run(islbm, torch, precision, steps, warmup, device, clk=None):
    p = islbm.default_params(precision=precision, device=device, **CASE)
    with islbm.Solver(p) as s:
        s.step(warmup)
        s.sync()
        if clk is not None:
            clk.mark_start()
        ms = time_steps(islbm, torch, s, steps)
        if clk is not None:
            clk.mark_end()
        ok = s.healthy()
        fields = s.fields()
    n = CASE["NX"] * CASE["NY"] * CASE["NZ"]
    return {"ms": ms, "mlups": n * steps / (ms * 1e-3) / 1e6, "healthy": ok, "fields": fields}


LARGE = dict(NX=384, NY=768, NZ=512, Re=10595.0, Uref=0.04, NDTFRC=100, les_cs=0.1)


def large_run(islbm, torch, device, steps=10, warmup=3):
    """The large single solve (768x384x512, 151M nodes, Re_h 10595, LES): FP32 and FP16-deviation
    storage on the tiled kernel, MLUPS and HBM fraction, and the xi weight-table bytes stored per
    (y, z) against per node."""
    n = LARGE["NX"] * LARGE["NY"] * LARGE["NZ"]
    peak, _ = measured_peak_gbs()
    out = {"grid": "NY768 NX384 NZ512", "nodes": n, "steps": steps}
    for prec, eb in (("fp32", 4), ("fp16", 2)):
        p = islbm.default_params(precision=prec, device=device, **LARGE)
        with islbm.Solver(p) as s:
            s.step(warmup)
            s.sync()
            ms = time_steps(islbm, torch, s, steps)
            if prec == "fp32":
                wt = s.weight_table_bytes()
                out["weight_table_bytes"] = {"per_y_z": wt["stored"], "per_node": wt["per_node"]}
        mlups = n * steps / (ms * 1e-3) / 1e6
        gbs = 2 * 19 * eb * n / (ms * 1e-3 / steps) / 1e9
        out[prec] = {"mlups": mlups, "hbm_gbs": gbs, "frac": gbs / peak, "ms_per_step": ms / steps}
    return out


def large_accuracy_run(islbm, device, steps=800, samples=10, tau=1.1, k64=20):
    """Storage-format accuracy of the large grid (768x384x512): time-averaged u, v, w profiles of
    the FP16-deviation run against the FP32 run of the same case, at x/h = 0.5, 2, 4, 6, 8 (the
    stations of C/fileIO.h:118-249), and the instantaneous velocity of both after the first k64
    steps against an FP64 run of the same grid (the FP64 step runs at a fraction of a GLUPS, so it
    covers the first steps only). The case is the one relaxation time at which the reference
    scheme holds on this grid (tau = 1.1; it diverges within a few hundred steps at 0.6-1.0 and
    1.2-2.5). The comparison the configuration names, against an FP64 run of 256x128x192 at the
    same Reynolds number, has no common stable case: the same viscosity puts the coarse grid at
    tau = 0.725, where it grows without bound within 300 steps (the coarse grid holds only from
    tau = 1.0 up, which puts the fine grid at 1.83)."""
    import numpy as np
    case = dict(NX=384, NY=768, NZ=512, Uref=0.04, NDTFRC=100, les_cs=0.1)
    ms_f = (3.036 - 1.0) / case["NZ"] * 0.6
    re = 3.0 * case["Uref"] / ((tau - 0.5) * ms_f)
    rows = [int(round(st * case["NY"] / 9.0)) % case["NY"] for st in (0.5, 2.0, 4.0, 6.0, 8.0)]
    out = {"case": "768x384x512, %d steps, tau %.2f (Re_h %.1f), LES Cs 0.1, Ub 0.04" % (steps, tau, re),
           "samples": samples, "stations_x_over_h": [0.5, 2, 4, 6, 8]}
    prof, vel = {}, {}
    chunk = steps // samples
    for prec in ("fp32", "fp16", "fp64"):
        p = islbm.default_params(precision=prec, device=device, Re=re, **case)
        t0 = time.perf_counter()
        with islbm.Solver(p) as s:
            s.step(k64)
            f = s.fields()
            vel[prec] = np.stack([f["u"], f["v"], f["w"]])
            del f
            if prec == "fp64":
                out[prec] = {"healthy": s.healthy(), "seconds": time.perf_counter() - t0, "steps": k64}
                continue
            s.stats_reset()
            s.step(chunk - k64)
            s.stats_accumulate()
            for _ in range(samples - 1):
                s.step(chunk)
                s.stats_accumulate()
            prof[prec] = np.stack([[s.stats_profile(q, y) for y in rows] for q in ("U", "V", "W")])
            out[prec] = {"healthy": s.healthy(), "seconds": time.perf_counter() - t0,
                         "max_abs_profile_over_ub": float(np.abs(prof[prec]).max() / case["Uref"])}
    err = float(np.abs(prof["fp16"] - prof["fp32"]).max() / case["Uref"])
    out["fp16"]["time_avg_profiles_max_abs_err_vs_fp32_over_ub"] = err if np.isfinite(err) else None
    for prec in ("fp32", "fp16"):
        out[prec]["vs_fp64_after_%d_steps" % k64] = {
            "rel_l2_u": rel_l2(vel[prec], vel["fp64"]),
            "max_abs_u_over_ub": float(np.abs(vel[prec] - vel["fp64"]).max() / case["Uref"])}
    return out


def e2e_run(islbm, precision, steps, device, f_host):
    """Through the C ABI with host buffers: upload the state from pinned host memory, step, and
    read the fields into pinned host memory every 100 steps (the reference main loop's cadence)."""
    import ctypes
    import numpy as np
    import torch
    n = CASE["NX"] * CASE["NY"] * CASE["NZ"]
    f_pin = torch.from_numpy(np.ascontiguousarray(f_host, dtype=np.float64).reshape(-1)).pin_memory()
    outs = [torch.empty(n, dtype=torch.float64).pin_memory() for _ in range(4)]
    vp = ctypes.c_void_p
    p = islbm.default_params(precision=precision, device=device, **CASE)
    with islbm.Solver(p) as s:
        L, h = s._L, s._h
        s.sync()
        t0 = time.perf_counter()
        islbm.check(L.islbm_set_populations(h, vp(f_pin.data_ptr()), islbm.LAYOUT_UNIQUE))
        done, reads = 0, 0
        while done < steps:
            chunk = min(100, steps - done)
            s.step(chunk)
            done += chunk
            islbm.check(L.islbm_fields(h, *[vp(o.data_ptr()) for o in outs], islbm.LAYOUT_UNIQUE))
            reads += 1
        s.sync()
        dt = time.perf_counter() - t0
    h2d = 19 * n * np.dtype(np.float64).itemsize
    d2h = reads * 4 * n * 8
    return {"value": n * steps / dt / 1e6, "unit": "MLUPS", "h2d_bytes_per_step": h2d / steps,
            "d2h_bytes_per_step": d2h / steps, "note": "FP64 pinned host buffers through islbm_set_populations / "
                                                       "islbm_step / islbm_fields"}


def cpu_oracle_run(steps, threads, warmup=1):
    """The CPU oracle (reference restatement) on the same workload: `warmup` untimed steps, then
    `steps` timed steps; returns (MLUPS, seconds of the timed steps)."""
    from oracle.oracle import Oracle
    o = Oracle(CASE["NX"], CASE["NY"], CASE["NZ"], re=CASE["Re"], ub=CASE["Uref"], ndtfrc=CASE["NDTFRC"],
               les_cs=CASE["les_cs"], threads=threads)
    if warmup > 0:
        o.step(warmup)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    o.close()
    n = CASE["NX"] * CASE["NY"] * CASE["NZ"]
    return n * steps / dt / 1e6, dt


def accuracy_run(islbm, device, steps=1000):
    """Storage-format errors on the benchmark grid at a relaxation time where the reference
    scheme is stable (tau = 1.0; at Re_h 2800 it diverges): FP32 / FP16 / BF16 against FP64
    after `steps` steps from the same seeded state, and the total-mass drift of each."""
    import numpy as np
    min_size = (3.036 - 1.0) / CASE["NZ"] * 0.6
    kw = dict(CASE)
    kw["Re"] = 3.0 * CASE["Uref"] / (0.5 * min_size)
    # streamwise stations x/h = 0.5, 2, 4, 6, 8 of the profiles (rows of the uniform y mesh)
    rows = [int(round(st * CASE["NY"] / 9.0)) % CASE["NY"] for st in (0.5, 2.0, 4.0, 6.0, 8.0)]
    out, ref, ref_prof, ref_cf = {}, None, None, None
    for prec in ("fp64", "fp32", "fp16", "bf16"):
        with islbm.Solver(islbm.default_params(precision=prec, device=device, **kw)) as s:
            m0 = s.diagnostics()["mass"]
            s.stats_reset()
            for _ in range(steps // 10):   # time averages over the run, one sample every 10 steps
                s.step(10)
                s.stats_accumulate()
            f = s.fields()
            m1 = s.diagnostics()["mass"]
            prof = np.stack([[s.stats_profile(q, y) for y in rows] for q in ("U", "V", "W")])
            cf = s.stats_wall_shear()
        u = np.stack([f[c] for c in "uvw"])
        if ref is None:
            ref, ref_prof, ref_cf = u, prof, cf
        out[prec] = {"rel_l2_u_vs_fp64": rel_l2(u, ref), "max_abs_u_over_ub": float(np.abs(u - ref).max() / CASE["Uref"]),
                     "time_avg_profiles_max_abs_err_over_ub": float(np.abs(prof - ref_prof).max() / CASE["Uref"]),
                     "wall_cf_max_abs_err": float(np.abs(cf - ref_cf).max()), "wall_cf_max": float(np.abs(ref_cf).max()),
                     "mass_drift_rel": (m1 - m0) / m0}
    return {"case": "256x128x192, LES Cs 0.1, tau 1.0 (Re_h %.2f)" % kw["Re"], "steps": steps,
            "profiles": "spanwise-averaged time means of u, v, w at x/h = 0.5, 2, 4, 6, 8 (%d samples)" % (steps // 10),
            "errors": out}


def serve_run(islbm, nreq, device, mean_gap=0.5, n_err=8):
    """The specified request stream (Poisson arrivals) through the serving loop and as sequential
    plain solves, with per-grid accounting; then the error against plain FP64 solves for n_err
    requests of the stream (the two smaller grids; the FP64 step runs at a fraction of a GLUPS),
    each served in one batch for 1000 steps and solved alone in FP64 for the same steps."""
    import numpy as np
    import serving
    reqs = serving.make_requests(nreq, seed=2024, mean_gap=mean_gap)
    srv, infos, _ = serving.run_server(reqs, device=device)
    seq = serving.run_sequential(reqs, device=device)
    # capacity: the same requests all submitted at once, against the same plain solves back to
    # back (their summed solve time, set-up included)
    sat, _, _ = serving.run_server([dict(r, arrival=0.0) for r in reqs], device=device)
    seq_busy = sum(g["seconds"] for g in seq["per_grid"].values())
    capacity = {"server_mlups": sat["mlups"], "server_wall_s": sat["wall_s"], "server_updates": sat["updates"],
                "sequential_mlups": seq["updates"] / max(seq_busy, 1e-9) / 1e6, "sequential_busy_s": seq_busy,
                "speedup_mlups": sat["mlups"] / max(seq["updates"] / max(seq_busy, 1e-9) / 1e6, 1e-9),
                "status": sat["status"]}
    grids = {}
    for i, r in enumerate(reqs):
        g = grids.setdefault("%dx%dx%d" % (r["NY"], r["NX"], r["NZ"]), {"requests": 0, "updates": 0, "converged": 0,
                                                                         "steps": []})
        g["requests"] += 1
        g["updates"] += infos[i]["steps"] * r["NX"] * r["NY"] * r["NZ"]
        g["converged"] += infos[i]["status"] == "converged"
        g["steps"].append(infos[i]["steps"])
    total = sum(g["updates"] for g in grids.values())
    for g in grids.values():
        g["share_of_updates"] = g["updates"] / max(total, 1)
        st = g.pop("steps")
        g["steps_median"] = float(np.median(st))
    sample = [i for i, r in enumerate(reqs) if r["NZ"] == 48][:n_err // 2] + \
             [i for i, r in enumerate(reqs) if r["NZ"] == 96][:n_err - n_err // 2]
    errs = []
    steps = 1000
    with islbm.Server(device=device, steps_per_chunk=steps) as s_err:
        ids = {i: s_err.submit(serving.params_of(reqs[i]), steps, 0.0, keep_fields=True) for i in sample}
        s_err.drain()
        got = {i: s_err.fields(ids[i]) for i in sample}
    for i in sample:
        r = reqs[i]
        with islbm.Solver(serving.params_of(r, precision="fp64", device=device)) as s:
            s.step(steps)
            ref = s.fields()
        g = got[i]
        errs.append({"request": i, "grid": "%dx%dx%d" % (r["NY"], r["NX"], r["NZ"]), "precision": r["precision"],
                     "alpha": r["alpha"], "steps": steps,
                     "rel_l2_u_vs_fp64": rel_l2(np.stack([g[c] for c in "uvw"]), np.stack([ref[c] for c in "uvw"])),
                     "max_abs_u_over_ub": float(max(np.abs(g[c] - ref[c]).max() for c in "uvw") / r["Uref"])})
    return {"requests": nreq, "mean_gap_s": mean_gap, "grids": "64x32x48 / 128x64x96 / 256x128x192 (NY x NX x NZ)",
            "steps_cap": {"x".join(map(str, g)): c for g, c, _ in serving.GRIDS},
            "tau_range": {"x".join(map(str, g)): list(t) for g, _, t in serving.GRIDS},
            "alpha_range": list(serving.ALPHA_RANGE), "tol": serving.TOL, "chunk": serving.CHUNK,
            "convergence": "delta = sqrt(mean |u - u_prev|^2)/Ub over each chunk < tol",
            "server": srv, "sequential": seq, "speedup_mlups": srv["mlups"] / seq["mlups"], "capacity": capacity,
            "per_grid": grids, "error_vs_fp64": errs}


def slowest_rank_ms(ms, world, device):
    """Replicas: every rank ran the same workload; the job's time is the slowest rank's."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rel_l2(a, b):
    import numpy as np
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-large", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=64)
    args = ap.parse_args()
    rank, world, local = dist_env()
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return 0
        from oracle import build as ob
        ob.build()
        # every step is a full step of the workload (about 0.7 s on 16 host cores): at most 100
        # timed steps and 10 warm-up steps, and the line reports the counts actually run
        cpu_steps = max(1, min(args.steps, 100))
        cpu_warm = max(0, min(args.warmup, 10))
        mlups, dt = cpu_oracle_run(cpu_steps, threads, warmup=cpu_warm)
        line = {"metric": METRIC, "value": mlups, "unit": "MLUPS", "impl": "reference", "n_gpus": args.gpus,
                "steps": cpu_steps, "warmup": cpu_warm, "ms_per_step": dt / cpu_steps * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": {"workload": WORKLOAD, "grid": "NY256 NX128 NZ192", "precision": "fp64"},
                "cpu_baseline": {"value": mlups, "unit": "MLUPS", "cores": threads, "kind": "port",
                                 "steps": cpu_steps, "warmup": cpu_warm, "seconds": dt,
                                 "sample": f"{cpu_steps} full steps of the 256x128x192 grid after {cpu_warm} warm-up "
                                           f"steps, FP64, LES, OpenMP over {threads} host threads"},
                "e2e": {"value": mlups, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        if cpu_steps != args.steps or cpu_warm != args.warmup:
            line["requested"] = {"steps": args.steps, "warmup": args.warmup}
        print(json.dumps(line))
        return 0

    import numpy as np
    import torch
    import islbm
    import islbm_build
    islbm_build.build()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    peak, peak_kind = measured_peak_gbs()
    n = CASE["NX"] * CASE["NY"] * CASE["NZ"]

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    # plain FP32, device resident
    barrier()
    with ClockSampler(local) as clk:
        r32 = device_run(islbm, torch, "fp32", args.steps, args.warmup, local, clk)
    barrier()
    ms = slowest_rank_ms(r32["ms"], world, "cuda")
    value = n * args.steps * world / (ms * 1e-3) / 1e6
    bytes_per_launch = 2 * 19 * 4 * n
    achieved = bytes_per_launch / (ms * 1e-3 / args.steps) / 1e9
    line = {"metric": METRIC, "value": value, "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded perturbed equilibrium)",
            "config": {"workload": WORKLOAD, "grid": "NY256 NX128 NZ192", "precision": "fp32",
                       "l2": "inputs larger than L2 (2 x 478 MB population buffers), no flush",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "gpu_launches": args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": NCU_TRAFFIC_BYTES, "traffic_unit": "bytes per launch (ncu)",
                         "traffic_vs_algorithmic": NCU_TRAFFIC_BYTES / bytes_per_launch, "peak_kind": peak_kind,
                         "bytes_model": "2 x 19 x 4 B per node per step (read + write each population once)"},
            "clocks": clk.summary()}
    if rank == 0 and not args.no_mixed:
        mixed = {}
        for prec in ("fp16", "bf16"):
            r = device_run(islbm, torch, prec, args.steps, args.warmup, local)
            ach = 2 * 19 * 2 * n / (r["ms"] * 1e-3 / args.steps) / 1e9
            mixed[prec] = {"mlups": r["mlups"], "speedup_vs_fp32": r["mlups"] / r32["mlups"],
                           "hbm_gbs": ach, "frac": ach / peak, "steps": args.steps + args.warmup}
        # the FP64 step on the same workload (config side by side with FP32): the one-thread-per-node
        # kernel, bound by the FP64 pipe of GB300 rather than by memory
        steps64 = max(1, min(args.steps, 20))
        r = device_run(islbm, torch, "fp64", steps64, 2, local)
        ach = 2 * 19 * 8 * n / (r["ms"] * 1e-3 / steps64) / 1e9
        mixed["fp64"] = {"mlups": r["mlups"], "speedup_vs_fp32": r["mlups"] / r32["mlups"], "hbm_gbs": ach,
                         "frac": ach / peak, "steps": steps64, "kernel": "one thread per node (FP64 parity path)"}
        line["mixed"] = mixed
        line["accuracy"] = accuracy_run(islbm, local)
    if rank == 0 and not args.no_e2e:
        p = islbm.default_params(precision="fp32", device=local, **CASE)
        with islbm.Solver(p) as s:
            f_host = s.populations()
        line["e2e"] = e2e_run(islbm, "fp32", args.steps, local, f_host)
    if rank == 0 and not args.no_cpu:
        from oracle import build as ob
        ob.build()
        mlups, dt = cpu_oracle_run(args.cpu_steps, threads)
        line["cpu_baseline"] = {"value": mlups, "unit": "MLUPS", "cores": threads, "kind": "port",
                                "steps": args.cpu_steps, "warmup": 1, "seconds": dt,
                                "sample": f"{args.cpu_steps} full steps of the 256x128x192 grid after 1 warm-up step, "
                                          f"FP64, LES, OpenMP over {threads} host threads"}
    if rank == 0 and not args.no_large:
        line["large"] = large_run(islbm, torch, local)
        line["large"]["accuracy"] = large_accuracy_run(islbm, local)
    if rank == 0 and not args.no_serve:
        line["serve"] = serve_run(islbm, args.serve_requests, local)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
