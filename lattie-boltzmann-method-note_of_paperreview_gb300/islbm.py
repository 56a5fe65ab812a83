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
KERNEL_AUTO, KERNEL_GATHER, KERNEL_TILED = 0, 1, 2

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
    ]


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
        "islbm_host_table": [P, ctypes.c_char_p, ip, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)],
        "islbm_host_table_int": [P, ctypes.c_char_p, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)],
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


def baseline_params(case, **overrides):
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

    def healthy(self):
        bad = ctypes.c_longlong()
        st = self._L.islbm_check_finite(self._h, ctypes.byref(bad))
        if st not in (0, 5):
            check(st)
        return bad.value == 0
