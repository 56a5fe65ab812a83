"""Compile the CPU oracle (oracle/islbm_oracle.c) into oracle/_build/libislbm_oracle.so.

Test infrastructure only. Flags keep IEEE operation order (-ffp-contract=off, no
fast-math) so that results do not depend on FMA contraction of the host compiler.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libislbm_oracle.so")


def build(force=False, cc="gcc"):
    src = os.path.join(HERE, "islbm_oracle.c")
    hdr = os.path.join(HERE, "islbm_oracle.h")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr)):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [cc, "-std=c11", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-Wall", "-Wno-unused-function", "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
