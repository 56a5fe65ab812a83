"""Python mirror of the ISLBM C ABI (include/islbm.h) over ctypes.

`Solver` plays the role of the reference's main loop around its step path:
  Solver(params)            AllocateMemory + mesh/weights/BFL precompute + initial state
  solver.step(n)            n x Launch_CollisionStreaming (+ AccumulateUbulk and
                            Launch_ModifyForcingTerm every NDTFRC steps)
  solver.fields()           SendDataToCPU for rho, u, v, w
(reference: 筆記：金的code/0.可更改的code/evolution.h:842-1042, initialization.h, memory.h).

The compute path is the CUDA library only; if libislbm_gb300.so cannot be loaded this module
raises instead of falling back to anything else.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libislbm_gb300.so")

FP64, FP32, FP16_DEV, BF16_DEV = 0, 1, 2, 3
PRECISIONS = {"fp64": FP64, "fp32": FP32, "fp16": FP16_DEV, "bf16": BF16_DEV}
LAYOUT_UNIQUE, LAYOUT_REFERENCE = 0, 1
KERNEL_AUTO, KERNEL_GATHER, KERNEL_TILED, KERNEL_TILED_SINGLE = 0, 1, 2, 3

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory", 4: "HBM budget exceeded",
          5: "non-finite state", 6: "not supported", 7: "no CUDA device"}


class IslbmError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"islbm status {status}: {msg}")
        self.status = status


class Params(ctypes.Structure):
    """islbm_params; names follow the reference's variables.h."""
    _fields_ = [
        ("NX", ctypes.c_int), ("NY", ctypes.c_int), ("NZ", ctypes.c_int),
        ("LX", ctypes.c_double), ("LY", ctypes.c_double), ("LZ", ctypes.c_double),
        ("CFL", ctypes.c_double), ("LXi", ctypes.c_double),
        ("Re", ctypes.c_double), ("Uref", ctypes.c_double),
        ("NDTFRC", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("les_cs", ctypes.c_double),
        ("alpha", ctypes.c_double),
        ("init_mode", ctypes.c_int),
        ("seed", ctypes.c_ulonglong),
        ("perturb", ctypes.c_double),
        ("mass_interval", ctypes.c_int),
        ("bfl_mode", ctypes.c_int),
        ("device", ctypes.c_int),
        ("kernel", ctypes.c_int),
        ("hbm_budget_bytes", ctypes.c_size_t),
        ("geometry", ctypes.c_int),
    ]


class SolveInfo(ctypes.Structure):
    """islbm_solve_info (include/islbm_serve.h)."""
    _fields_ = [("id", ctypes.c_longlong), ("status", ctypes.c_int), ("steps", ctypes.c_longlong),
                ("nodes", ctypes.c_longlong), ("delta", ctypes.c_double), ("force", ctypes.c_double),
                ("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double), ("t_done", ctypes.c_double)]


# time-averaged quantities of islbm_stats_* (islbm_stat order)
STATS = ["U", "V", "W", "P", "UU", "UV", "UW", "VV", "VW", "WW", "PU", "PV", "PW", "PP", "KT",
         "UUU", "UUV", "UUW", "VVU", "VVV", "VVW", "WWU", "WWV", "WWW",
         "DUDX2", "DUDY2", "DUDZ2", "DVDX2", "DVDY2", "DVDZ2", "DWDX2", "DWDY2", "DWDZ2"]

SOLVE_STATUS = {0: "queued", 1: "active", 2: "converged", 3: "capped", 4: "diverged", 5: "rejected"}

_lib = None


def load():
    """Load libislbm_gb300.so (building it first if the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise IslbmError(-1, f"CUDA library not built: {LIB_PATH} (run build.py)")
    L = ctypes.CDLL(LIB_PATH)
    vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)
    P = ctypes.POINTER(Params)
    sig = {
        "islbm_default_params": [P],
        "islbm_required_bytes": [P, ctypes.POINTER(ctypes.c_size_t)],
        "islbm_init": [P, ctypes.POINTER(vp)],
        "islbm_step": [vp, ip],
        "islbm_fields": [vp, vp, vp, vp, vp, ip],
        "islbm_get_population": [vp, ip, vp, ip],
        "islbm_set_populations": [vp, vp, ip],
        "islbm_get_scalars": [vp, dp, dp, ctypes.POINTER(ctypes.c_longlong)],
        "islbm_set_force": [vp, ctypes.c_double],
        "islbm_get_constants": [vp, dp, dp, dp, dp],
        "islbm_weight_table_bytes": [vp, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)],
        "islbm_get_stream": [vp, ctypes.POINTER(vp)],
        "islbm_sync": [vp],
        "islbm_check_finite": [vp, ctypes.POINTER(ctypes.c_longlong)],
        "islbm_destroy": [vp],
        "islbm_diagnostics": [vp, dp],
        "islbm_fault_drill": [vp, ip],
        "islbm_diagnostics_noalloc": [vp, dp],
        "islbm_write_tecplot_ascii": [vp, ctypes.c_char_p],
        "islbm_write_tecplot_plt": [vp, ctypes.c_char_p],
        "islbm_write_monitor": [vp, ctypes.c_char_p, ip],
        "islbm_checkpoint_write": [vp, ctypes.c_char_p, ip],
        "islbm_checkpoint_read": [vp, ctypes.c_char_p, ip],
        "islbm_stats_reset": [vp],
        "islbm_stats_gradients": [vp, ip],
        "islbm_stats_accumulate": [vp],
        "islbm_stats_samples": [vp, ctypes.POINTER(ctypes.c_longlong)],
        "islbm_stats_mean": [vp, ip, vp, ip],
        "islbm_stats_profile": [vp, ip, ip, vp],
        "islbm_stats_wall_shear": [vp, vp],
        "islbm_stats_write": [vp, ctypes.c_char_p, ip],
        "islbm_stats_read": [vp, ctypes.c_char_p, ip],
        "islbm_host_table": [P, ctypes.c_char_p, ip, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)],
        "islbm_host_table_int": [P, ctypes.c_char_p, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)],
        "islbm_server_create": [ip, ctypes.c_size_t, ip, ctypes.POINTER(vp)],
        "islbm_server_submit": [vp, P, ctypes.c_longlong, ctypes.c_double, ip, ctypes.POINTER(ctypes.c_longlong)],
        "islbm_server_pump": [vp, ctypes.POINTER(ip), ctypes.POINTER(ip)],
        "islbm_server_info": [vp, ctypes.c_longlong, ctypes.POINTER(SolveInfo)],
        "islbm_server_fields": [vp, ctypes.c_longlong, vp, vp, vp, vp],
        "islbm_server_stats": [vp, ctypes.POINTER(ctypes.c_longlong), dp, ctypes.POINTER(ctypes.c_size_t)],
        "islbm_server_destroy": [vp],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    L.islbm_status_string.argtypes = [ctypes.c_int]
    L.islbm_status_string.restype = ctypes.c_char_p
    _lib = L
    return L


def check(status):
    if status != 0:
        msg = load().islbm_status_string(status).decode()
        raise IslbmError(status, msg)


def default_params(**overrides):
    p = Params()
    check(load().islbm_default_params(ctypes.byref(p)))
    for k, v in overrides.items():
        if k == "precision" and isinstance(v, str):
            v = PRECISIONS[v]
        setattr(p, k, v)
    return p


def benchmark_params(case, **overrides):
    """Parameter sets of the benchmark cases (grid given streamwise x spanwise x wall-normal
    in the benchmark's naming, i.e. NY x NX x NZ here)."""
    cases = {
        "hill64": dict(NX=32, NY=64, NZ=48, Re=700.0, Uref=0.05, NDTFRC=100, les_cs=0.0),
        "hill256": dict(NX=128, NY=256, NZ=192, Re=2800.0, Uref=0.05, NDTFRC=100, les_cs=0.1),
        "hill768": dict(NX=384, NY=768, NZ=512, Re=10595.0, Uref=0.04, NDTFRC=100, les_cs=0.1),
    }
    kw = dict(cases[case])
    kw.update(overrides)
    return default_params(**kw)


def required_bytes(params):
    n = ctypes.c_size_t()
    check(load().islbm_required_bytes(ctypes.byref(params), ctypes.byref(n)))
    return n.value


def host_table(params, name, idx=0):
    """FP64 host precompute table (reference layout indexing); no GPU needed."""
    L = load()
    cnt = ctypes.c_size_t()
    check(L.islbm_host_table(ctypes.byref(params), name.encode(), int(idx), None, 0, ctypes.byref(cnt)))
    out = np.zeros(cnt.value, dtype=np.float64)
    check(L.islbm_host_table(ctypes.byref(params), name.encode(), int(idx), out.ctypes.data_as(ctypes.c_void_p),
                             out.size, ctypes.byref(cnt)))
    return out


def host_table_int(params, name):
    L = load()
    cnt = ctypes.c_size_t()
    check(L.islbm_host_table_int(ctypes.byref(params), name.encode(), None, 0, ctypes.byref(cnt)))
    out = np.zeros(cnt.value, dtype=np.int32)
    check(L.islbm_host_table_int(ctypes.byref(params), name.encode(), out.ctypes.data_as(ctypes.c_void_p),
                                 out.size, ctypes.byref(cnt)))
    return out


class Solver:
    """One periodic-hill solve resident on the GPU."""

    def __init__(self, params):
        self.params = params
        self._L = load()
        h = ctypes.c_void_p()
        check(self._L.islbm_init(ctypes.byref(params), ctypes.byref(h)))
        self._h = h
        self.NX, self.NY, self.NZ = params.NX, params.NY, params.NZ
        self.N = self.NX * self.NY * self.NZ

    def close(self):
        if getattr(self, "_h", None):
            self._L.islbm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def step(self, n=1):
        check(self._L.islbm_step(self._h, int(n)))

    def sync(self):
        check(self._L.islbm_sync(self._h))

    def _shape(self, layout):
        if layout == LAYOUT_REFERENCE:
            return (self.NY + 7, self.NZ + 6, self.NX + 7)
        return (self.NZ, self.NY, self.NX)

    def fields(self, layout=LAYOUT_UNIQUE):
        shp = self._shape(layout)
        outs = [np.zeros(shp, dtype=np.float64) for _ in range(4)]
        check(self._L.islbm_fields(self._h, *[o.ctypes.data_as(ctypes.c_void_p) for o in outs], int(layout)))
        return dict(zip(("rho", "u", "v", "w"), outs))

    def population(self, q, layout=LAYOUT_UNIQUE):
        out = np.zeros(self._shape(layout), dtype=np.float64)
        check(self._L.islbm_get_population(self._h, int(q), out.ctypes.data_as(ctypes.c_void_p), int(layout)))
        return out

    def populations(self, layout=LAYOUT_UNIQUE):
        return np.stack([self.population(q, layout) for q in range(19)])

    def set_populations(self, f19, layout=LAYOUT_UNIQUE):
        a = np.ascontiguousarray(f19, dtype=np.float64)
        assert a.size == 19 * int(np.prod(self._shape(layout)))
        check(self._L.islbm_set_populations(self._h, a.ctypes.data_as(ctypes.c_void_p), int(layout)))

    def scalars(self):
        f, r, s = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        check(self._L.islbm_get_scalars(self._h, ctypes.byref(f), ctypes.byref(r), ctypes.byref(s)))
        return {"force": f.value, "rho_modify": r.value, "steps": s.value}

    @property
    def force(self):
        return self.scalars()["force"]

    @force.setter
    def force(self, value):
        check(self._L.islbm_set_force(self._h, float(value)))

    def constants(self):
        vals = [ctypes.c_double() for _ in range(4)]
        check(self._L.islbm_get_constants(self._h, *[ctypes.byref(v) for v in vals]))
        return dict(zip(("tau", "niu", "Uref", "minSize"), [v.value for v in vals]))

    def weight_table_bytes(self):
        a, b = ctypes.c_size_t(), ctypes.c_size_t()
        check(self._L.islbm_weight_table_bytes(self._h, ctypes.byref(a), ctypes.byref(b)))
        return {"stored": a.value, "per_node": b.value}

    def stream_handle(self):
        s = ctypes.c_void_p()
        check(self._L.islbm_get_stream(self._h, ctypes.byref(s)))
        return s.value or 0

    def diagnostics(self):
        """Total mass, mean streamwise momentum, kinetic energy and maximum speed (FP64)."""
        out = (ctypes.c_double * 4)()
        check(self._L.islbm_diagnostics(self._h, out))
        return {"mass": out[0], "momentum_y": out[1], "kinetic_energy": out[2], "max_speed": out[3]}

    def write_tecplot_ascii(self, path):
        check(self._L.islbm_write_tecplot_ascii(self._h, os.fsencode(path)))

    def write_tecplot_plt(self, path):
        check(self._L.islbm_write_tecplot_plt(self._h, os.fsencode(path)))

    def write_monitor(self, path, step):
        check(self._L.islbm_write_monitor(self._h, os.fsencode(path), int(step)))

    def checkpoint_write(self, directory, rank=0):
        check(self._L.islbm_checkpoint_write(self._h, os.fsencode(directory), int(rank)))

    def checkpoint_read(self, directory, rank=0):
        check(self._L.islbm_checkpoint_read(self._h, os.fsencode(directory), int(rank)))

    def stats_write(self, directory, rank=0):
        """The running sums and sample count in the reference's statistics files (Launch_OutputTB)."""
        check(self._L.islbm_stats_write(self._h, str(directory).encode(), rank))

    def stats_read(self, directory, rank=0):
        """Replace the running sums and sample count from statistics files (InitialTBUsingBkpData)."""
        check(self._L.islbm_stats_read(self._h, str(directory).encode(), rank))

    def stats_reset(self):
        check(self._L.islbm_stats_reset(self._h))

    def stats_gradients(self, on=True):
        """Also accumulate the squared velocity gradients (from the next reset on)."""
        check(self._L.islbm_stats_gradients(self._h, int(bool(on))))

    def stats_accumulate(self):
        check(self._L.islbm_stats_accumulate(self._h))

    def stats_samples(self):
        n = ctypes.c_longlong()
        check(self._L.islbm_stats_samples(self._h, ctypes.byref(n)))
        return n.value

    def stats_mean(self, quantity, layout=LAYOUT_UNIQUE):
        """Time mean of one quantity (name from STATS or index)."""
        q = STATS.index(quantity) if isinstance(quantity, str) else int(quantity)
        out = np.zeros(self._shape(layout), dtype=np.float64)
        check(self._L.islbm_stats_mean(self._h, q, out.ctypes.data_as(ctypes.c_void_p), int(layout)))
        return out

    def stats_profile(self, quantity, y):
        """Spanwise-averaged time mean at streamwise row y: NZ values from the hill surface up."""
        q = STATS.index(quantity) if isinstance(quantity, str) else int(quantity)
        out = np.zeros(self.params.NZ, dtype=np.float64)
        check(self._L.islbm_stats_profile(self._h, q, int(y), out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def stats_wall_shear(self):
        """Skin friction coefficient along the lower wall (NY values) from the time means."""
        out = np.zeros(self.params.NY, dtype=np.float64)
        check(self._L.islbm_stats_wall_shear(self._h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def healthy(self):
        bad = ctypes.c_longlong()
        st = self._L.islbm_check_finite(self._h, ctypes.byref(bad))
        if st not in (0, 5):
            check(st)
        return bad.value == 0


class Server:
    """Continuous-batching server over many solves on one GPU (include/islbm_serve.h)."""

    def __init__(self, device=0, hbm_budget_bytes=0, steps_per_chunk=500):
        self._L = load()
        self._s = ctypes.c_void_p()
        self._dims = {}
        check(self._L.islbm_server_create(device, hbm_budget_bytes, steps_per_chunk, ctypes.byref(self._s)))

    def close(self):
        if self._s:
            self._L.islbm_server_destroy(self._s)
            self._s = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, params, max_steps, tol=0.0, keep_fields=False):
        rid = ctypes.c_longlong()
        check(self._L.islbm_server_submit(self._s, ctypes.byref(params), int(max_steps), float(tol), int(keep_fields),
                                          ctypes.byref(rid)))
        self._dims[rid.value] = (params.NZ, params.NY, params.NX)
        return rid.value

    def pump(self):
        a, q = ctypes.c_int(), ctypes.c_int()
        check(self._L.islbm_server_pump(self._s, ctypes.byref(a), ctypes.byref(q)))
        return a.value, q.value

    def info(self, rid):
        i = SolveInfo()
        check(self._L.islbm_server_info(self._s, rid, ctypes.byref(i)))
        return {"id": i.id, "status": SOLVE_STATUS.get(i.status, i.status), "steps": i.steps, "nodes": i.nodes,
                "delta": i.delta, "force": i.force, "t_submit": i.t_submit, "t_admit": i.t_admit, "t_done": i.t_done}

    def fields(self, rid):
        """rho, u, v, w of a request, each shaped (NZ, NY, NX) (unique-node layout)."""
        out = {k: np.empty(self._dims[rid]) for k in ("rho", "u", "v", "w")}
        check(self._L.islbm_server_fields(self._s, rid, *[o.ctypes.data for o in out.values()]))
        return out

    def stats(self):
        u, b, m = ctypes.c_longlong(), ctypes.c_double(), ctypes.c_size_t()
        check(self._L.islbm_server_stats(self._s, ctypes.byref(u), ctypes.byref(b), ctypes.byref(m)))
        return {"updates": u.value, "busy_seconds": b.value, "bytes_in_use": m.value}

    def drain(self, max_pumps=1_000_000):
        """Pump until nothing is active or queued."""
        for _ in range(max_pumps):
            a, q = self.pump()
            if a == 0 and q == 0:
                return
        raise IslbmError(-1, "server did not drain")
