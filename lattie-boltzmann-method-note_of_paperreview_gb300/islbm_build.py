"""Build libislbm_gb300.so in-tree (`_build/`) for sm_103a with nvcc.

Every translation unit is compiled in parallel with one -gencode (compute_103a/sm_103a),
then linked into a shared library that exports only the C ABI of include/islbm.h.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libislbm_gb300.so")
SOURCES = ["abi.cu", "geometry.cpp", "step_gather.cu", "step_tiled.cu", "step_pair.cu", "serve.cu", "diagnostics.cu", "stats.cu", "checkpoint.cu", "writers.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _compile(src, verbose):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", f) for f in ("islbm.h", "islbm_serve.h", "islbm_testing.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj, ""
    flags = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
             "-Xcompiler", "-fvisibility=hidden"] + ARCH
    if src.endswith(".cu"):
        flags += ["--expt-relaxed-constexpr", "-Xptxas", "-v"] if verbose else ["--expt-relaxed-constexpr"]
    cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", obj] + flags
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr[-8000:]))
    return obj, r.stderr


def build(verbose=False, jobs=None):
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=jobs or len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
