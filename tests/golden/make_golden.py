"""Generate the golden fixtures in this directory from the reference's own step.

The reference (its headers under 筆記：金的code/0.可更改的code/) is compiled for host cores by
oracle/ref_build.py and run here; this script saves its tables and fields so that tests can
pin the oracle without the reference sources (the GPU machine does not have them).

Cases (grid NX x NY x NZ = 8 x 16 x 16, Re = 700, Ub = 0.05, perturbed start, seed 1234):
  hill_8x16x16_nd10.npz   forcing controller every 10 steps, no mass correction, 25 steps
  hill_8x16x16_nd10_m5.npz same with the mass correction every 5 steps, 25 steps
Run: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref_build  # noqa: E402
from oracle.oracle import Reference  # noqa: E402

TABLES = ["XPara0", "XPara2", "YPara0", "YPara2", "XiF3", "XiF4", "XiF5", "XiF6", "XiF15", "XiF16", "XiF17",
          "XiF18", "XBFL37", "XBFL38", "YBFL378", "XiBFL378", "XBFL49", "XBFL410", "YBFL4910", "XiBFL4910",
          "YBFL15", "XiBFL15", "YBFL16", "XiBFL16"]


def unique(R, a):
    u = a[3:3 + R.NY, 3:3 + R.NZ, 3:3 + R.NX]
    return np.ascontiguousarray(np.transpose(u, (1, 0, 2)))


def make(nx, ny, nz, nd, massk, steps, snaps, keep_f, out):
    lib = ref_build.build(nx, ny, nz, 700.0, 0.05, nd, massk)
    R = Reference(lib, mode=1, seed=1234, amp=0.01, ub=0.05)
    data = {"dims": np.array([nx, ny, nz, nd, massk, steps])}
    for nm in ["x", "y", "z", "xi", "Q3", "Q4", "Q15", "Q16"]:
        data["t_" + nm] = R.get(nm)
    for nm in TABLES:
        data["t_" + nm] = np.stack([R.get(nm, a) for a in range(7)])
    for nm in ["BFL3", "BFL4", "BFL15", "BFL16"]:
        data["i_" + nm] = R.get_int(nm)
    data["f0"] = np.stack([unique(R, R.get("f", q)) for q in range(19)])
    force = [R.force]
    for s in range(1, steps + 1):
        R.step(1)
        force.append(R.force)
        if s in snaps:
            for nm in ["rho", "u", "v", "w"]:
                data[f"s{s}_{nm}"] = unique(R, R.get(nm))
    if keep_f:
        data[f"f{steps}"] = np.stack([unique(R, R.get("f", q)) for q in range(19)])
    data["force"] = np.array(force)
    np.savez_compressed(os.path.join(HERE, out), **data)
    print("wrote", out)


if __name__ == "__main__":
    make(8, 16, 16, 10, 0, 25, (1, 10, 25), True, "hill_8x16x16_nd10.npz")
    make(8, 16, 16, 10, 5, 25, (5, 25), False, "hill_8x16x16_nd10_m5.npz")
