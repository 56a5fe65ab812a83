"""ctypes front-end of the CPU oracle (test infrastructure only).

Loads oracle/_build/libislbm_oracle.so (built by oracle/build.py) and, when present, the
reference compiled for host cores (oracle/_ref/*.so, built by oracle/ref_build.py in a
container that has the reference sources). Arrays come back in the reference's storage
layout (NYD6, NZ6, NX6); `unique()` cuts out the NY x NZ x NX unique nodes.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class OraParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("lx", ctypes.c_double), ("ly", ctypes.c_double), ("lz", ctypes.c_double),
        ("cfl", ctypes.c_double), ("lxi", ctypes.c_double),
        ("re", ctypes.c_double), ("ub", ctypes.c_double),
        ("ndtfrc", ctypes.c_int),
        ("init_mode", ctypes.c_int),
        ("seed", ctypes.c_ulonglong),
        ("amp", ctypes.c_double),
        ("mass_interval", ctypes.c_int),
        ("bfl_mode", ctypes.c_int),
        ("les_cs", ctypes.c_double),
        ("alpha", ctypes.c_double),
        ("threads", ctypes.c_int),
        ("geometry", ctypes.c_int),
    ]


def make_params(nx, ny, nz, re=700.0, ub=0.05, ndtfrc=100, init_mode=1, seed=1234, amp=0.01,
                mass_interval=0, bfl_mode=0, les_cs=0.0, alpha=1.0, threads=0, geometry=0):
    return OraParams(nx, ny, nz, 4.5, 9.0, 3.036, 0.6, 10.0, float(re), float(ub), int(ndtfrc),
                     int(init_mode), int(seed), float(amp), int(mass_interval), int(bfl_mode),
                     float(les_cs), float(alpha), int(threads), int(geometry))


_lib = None


def lib():
    global _lib
    if _lib is None:
        from oracle import build as _b  # noqa: WPS433 (local import keeps the module light)
        path = _b.build()
        L = ctypes.CDLL(path)
        L.ora_create.restype = ctypes.c_void_p
        L.ora_create.argtypes = [ctypes.POINTER(OraParams)]
        L.ora_destroy.argtypes = [ctypes.c_void_p]
        L.ora_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.ora_dims.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.ora_force.restype = ctypes.c_double
        L.ora_force.argtypes = [ctypes.c_void_p]
        L.ora_set_force.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.ora_scalar.restype = ctypes.c_double
        L.ora_scalar.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        L.ora_get.restype = ctypes.c_long
        L.ora_get.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p]
        L.ora_get_int.restype = ctypes.c_long
        L.ora_get_int.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
        L.ora_set_f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        _lib = L
    return _lib


class Oracle:
    """One oracle solve. Mirrors the reference's globals as named arrays."""

    def __init__(self, nx, ny, nz, **kw):
        self.params = make_params(nx, ny, nz, **kw)
        self._h = lib().ora_create(ctypes.byref(self.params))
        if not self._h:
            raise ValueError("oracle rejected the parameters")
        d = (ctypes.c_int * 6)()
        lib().ora_dims(self._h, d)
        self.NX6, self.NYD6, self.NZ6, self.NX, self.NY, self.NZ = list(d)

    def close(self):
        if self._h:
            lib().ora_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def step(self, n=1):
        if lib().ora_step(self._h, int(n)) != 0:
            raise RuntimeError("oracle step failed")

    @property
    def force(self):
        return lib().ora_force(self._h)

    @force.setter
    def force(self, value):
        lib().ora_set_force(self._h, float(value))

    def scalar(self, name):
        return lib().ora_scalar(self._h, name.encode())

    def get(self, name, idx=0):
        n3 = self.NX6 * self.NYD6 * self.NZ6
        buf = np.zeros(max(n3, 19), dtype=np.float64)
        cnt = lib().ora_get(self._h, name.encode(), int(idx), buf.ctypes.data_as(ctypes.c_void_p))
        if cnt < 0:
            raise KeyError(name)
        out = buf[:cnt].copy()
        return out.reshape(self.NYD6, self.NZ6, self.NX6) if cnt == n3 else out

    def get_int(self, name):
        buf = np.zeros(2 * self.NYD6, dtype=np.int32)
        cnt = lib().ora_get_int(self._h, name.encode(), buf.ctypes.data_as(ctypes.c_void_p))
        if cnt < 0:
            raise KeyError(name)
        return buf

    def set_f(self, q, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(-1)
        assert a.size == self.NX6 * self.NYD6 * self.NZ6
        lib().ora_set_f(self._h, int(q), a.ctypes.data_as(ctypes.c_void_p))

    def unique(self, a):
        """(NYD6, NZ6, NX6) reference layout -> (NZ, NY, NX) unique nodes, z-major."""
        u = a[3:3 + self.NY, 3:3 + self.NZ, 3:3 + self.NX]
        return np.ascontiguousarray(np.transpose(u, (1, 0, 2)))


class Reference:
    """The reference's own step compiled for host cores (available where it was built)."""

    def __init__(self, path, mode=1, seed=1234, amp=0.01, ub=0.05):
        self.L = ctypes.CDLL(path)
        self.L.ref_init.argtypes = [ctypes.c_int, ctypes.c_ulonglong, ctypes.c_double, ctypes.c_double]
        self.L.ref_force.restype = ctypes.c_double
        self.L.ref_get.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p]
        self.L.ref_get_int.argtypes = [ctypes.c_char_p, ctypes.c_void_p]
        d = (ctypes.c_int * 6)()
        self.L.ref_dims(d)
        self.NX6, self.NYD6, self.NZ6, self.NX, self.NY, self.NZ = list(d)
        self.L.ref_init(int(mode), int(seed), float(amp), float(ub))

    def step(self, n=1):
        self.L.ref_step(int(n))

    @property
    def force(self):
        return self.L.ref_force()

    def get(self, name, idx=0):
        n3 = self.NX6 * self.NYD6 * self.NZ6
        buf = np.zeros(n3, dtype=np.float64)
        cnt = self.L.ref_get(name.encode(), int(idx), buf.ctypes.data_as(ctypes.c_void_p))
        if cnt < 0:
            raise KeyError(name)
        out = buf[:cnt].copy()
        return out.reshape(self.NYD6, self.NZ6, self.NX6) if cnt == n3 else out

    def get_int(self, name):
        buf = np.zeros(2 * self.NYD6, dtype=np.int32)
        self.L.ref_get_int(name.encode(), buf.ctypes.data_as(ctypes.c_void_p))
        return buf


def reference_library(nx, ny, nz, re=700.0, ndtfrc=100, massk=0):
    path = os.path.join(HERE, "_ref", f"libislbm_ref_{nx}x{ny}x{nz}_re{re:g}_nd{ndtfrc}_m{massk}.so")
    return path if os.path.exists(path) else None
