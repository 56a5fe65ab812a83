"""The C ABI from C: tests/islbm_host.c is compiled with gcc as C11 against include/islbm.h only
and linked to libislbm_gb300.so.

* (CPU) The struct layouts the C compiler sees (sizeof and every member offset of islbm_params
  and islbm_solve_info) equal the ctypes mirror of islbm.py that the Python tests use.
* (GPU) The reference main loop of the integration notes, run as a C program: a 64x32x48 hill
  solve from the seeded perturbed start (v = Uref + 1 % noise), 100 steps in the FP64 path with islbm_fields in the reference layout
  (C/communication.h:260-273), against the oracle at relative L2 1e-12 on rho and the velocity and
  on the body force (the call sequence of C/evolution.h:842 and :1003).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, rel_l2


@pytest.fixture(scope="module")
def host_exe(islbm_lib, tmp_path_factory):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    out = str(tmp_path_factory.mktemp("c_host") / "islbm_host")
    libdir = os.path.dirname(islbm_lib.LIB_PATH)
    cmd = ["gcc", "-std=c11", "-O2", "-Wall", "-Wextra", "-Werror", os.path.join(ROOT, "tests", "islbm_host.c"),
           "-I", os.path.join(ROOT, "include"), "-L", libdir, "-lislbm_gb300", "-Wl,-rpath," + libdir, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_struct_layouts_match_ctypes_mirror(islbm_lib, host_exe):
    r = subprocess.run([host_exe, "layout"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    seen = dict(line.split() for line in r.stdout.strip().splitlines())
    for cname, cls in (("islbm_params", islbm_lib.Params), ("islbm_solve_info", islbm_lib.SolveInfo)):
        import ctypes
        assert int(seen[cname]) == ctypes.sizeof(cls), cname
        for field, _ in cls._fields_:
            assert int(seen[f"{cname}.{field}"]) == getattr(cls, field).offset, (cname, field)
        # every member the C compiler knows is mirrored
        assert {k.split(".", 1)[1] for k in seen if k.startswith(cname + ".")} == {f for f, _ in cls._fields_}


@pytest.mark.gpu
def test_c_main_loop_matches_oracle(host_exe, oracle_mod, tmp_path):
    steps, nx, ny, nz = 100, 32, 64, 48
    min_size = (3.036 - 1.0) / nz * 0.6
    re = 3.0 * 0.05 / ((0.6 - 0.5) * min_size)    # tau = 0.6, where the reference scheme is stable
    out = str(tmp_path / "fields.bin")
    r = subprocess.run([host_exe, "run", out, str(steps), "0", repr(re)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    o = oracle_mod.Oracle(nx, ny, nz, re=re, ndtfrc=100, init_mode=1, seed=1234, amp=0.01)
    o.step(steps)
    nref = o.NX6 * o.NYD6 * o.NZ6
    data = np.fromfile(out, dtype=np.float64)
    assert data.size == 4 * nref + 1
    shape = (o.NYD6, o.NZ6, o.NX6)
    got = {n: o.unique(data[m * nref:(m + 1) * nref].reshape(shape)) for m, n in enumerate(("rho", "u", "v", "w"))}
    ref = {n: o.unique(o.get(n)) for n in ("rho", "u", "v", "w")}
    vel = lambda d: np.stack([d["u"], d["v"], d["w"]])
    assert rel_l2(got["rho"], ref["rho"]) <= 1e-12
    assert rel_l2(vel(got), vel(ref)) <= 1e-12
    assert abs(data[-1] - o.force) <= 1e-12 * abs(o.force)
