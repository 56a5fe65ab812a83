"""Build the reference's own ISLBM step for host cores (test infrastructure, not product).

The reference (ChenPengChung/Lattie-Boltzmann-Method-Note_of_PaperReView, directory
``筆記：金的code/0.可更改的code/``) is an annotated copy of a CUDA+MPI solver with no main.cu
and no build system, and its headers do not compile as published. This recipe reads the
headers where they lie, applies only mechanical repairs in memory, splices them into
``ref_driver.inc`` (the host driver that plays main.cu for one process), and pipes the
single translation unit to ``g++`` on stdin. No reference source is written anywhere; the
only output is ``oracle/_ref/libislbm_ref_<NX>x<NY>x<NZ>[...].so``.

Mechanical repairs (each one named after the defect it removes):
  1. interpolationHillISLBM.h: ``//`` annotations pasted inside macro bodies are stripped,
     comment-only lines inside macros are dropped and the lost ``\\`` continuations
     restored (C/interpolationHillISLBM.h:10,14,23,42,69,138,151); the annotated
     parameter lists of F6_Intrpl7 (:64) and X_Y_XI_Intrpl7 (:68) get their plain
     parameter names back (the annotations in parentheses are removed).
  2. evolution.h: the ``}`` that closes ``if ( BFLReqF3_d[idx_xi] == 1 ){`` in
     stream_collide (lost at C/evolution.h:531) is inserted; only lines 1-840 (kernels)
     and 1003-1042 (Launch_ModifyForcingTerm) are compiled, the launcher (:842-1001)
     is CUDA launch syntax and is emulated by the driver with the same argument lists.
  3. MRT_Matrix.h is included before MRT_Process.h with ``#undef m_matrix`` in between,
     so the complete m_matrix of C/MRT_Process.h:4-62 is used instead of the truncated
     redefinition at C/MRT_Matrix.h:74-80.
  4. CUDA runtime / MPI calls are mapped to host equivalents (memcpy, calloc, jp = 1).

Grid and flow constants replace the compile-time ones of variables.h:
  NX, NY, NZ, jp = 1, tau = 0.5 + 3*Ub/(Re*minSize) (so that Uref = Re*niu = Ub),
  Re, NDTFRC; every derived macro (NX6, NYD6, NZ6, minSize, dt, niu, Uref) is the
  reference's own.

Usage: python oracle/ref_build.py --nx 32 --ny 64 --nz 48 --re 700 --ub 0.05 --ndtfrc 100
"""
import argparse
import os
import re
import subprocess
import sys

REF_ROOT = os.environ.get("ISLBM_REFERENCE_ROOT", "/root/reference")
CODE_DIR = os.path.join(REF_ROOT, "筆記：金的code", "0.可更改的code")
HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")

SHIM = r"""
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <cstdarg>
#include <algorithm>
#include <sys/time.h>
using std::min; using std::max;
#define __global__
#define __device__
#define __host__
#define __syncthreads() ((void)0)
struct emu_dim3 { unsigned x, y, z; };
static emu_dim3 blockIdx, threadIdx, blockDim;
typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
typedef void *cudaStream_t; typedef void *cudaEvent_t;
static inline const char *cudaGetErrorString(cudaError_t) { return "host emulation"; }
static inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) { memcpy(d, s, n); return 0; }
template <class T> static inline cudaError_t cudaMalloc(T **p, size_t n) { *p = (T *)calloc(n, 1); return *p ? 0 : 2; }
static inline cudaError_t cudaMallocHost(void **p, size_t n) { *p = calloc(n, 1); return *p ? 0 : 2; }
static inline cudaError_t cudaMemset(void *p, int v, size_t n) { memset(p, v, n); return 0; }
static inline cudaError_t cudaFree(void *p) { free(p); return 0; }
static inline cudaError_t cudaFreeHost(void *p) { free(p); return 0; }
static inline cudaError_t cudaDeviceSynchronize() { return 0; }
static inline cudaError_t cudaStreamCreate(cudaStream_t *) { return 0; }
static inline cudaError_t cudaStreamDestroy(cudaStream_t) { return 0; }
static inline cudaError_t cudaStreamSynchronize(cudaStream_t) { return 0; }
static inline cudaError_t cudaEventCreate(cudaEvent_t *) { return 0; }
static inline cudaError_t cudaEventDestroy(cudaEvent_t) { return 0; }
#define MPI_MAX_ERROR_STRING 256
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 0
#define MPI_SUM 0
static inline int MPI_Error_string(int, char *s, int *n) { s[0] = 0; *n = 0; return 0; }
static inline int MPI_Barrier(int) { return 0; }
static inline int MPI_Reduce(void *s, void *r, int c, int, int, int, int) { memcpy(r, s, (size_t)c * sizeof(double)); return 0; }
static inline int MPI_Bcast(void *, int, int, int, int) { return 0; }
static inline FILE *emu_fopen(const char *, const char *mode) { return fopen("/dev/null", mode); }
#define fopen emu_fopen
#define printf(...) ((void)0)
"""


def read(name):
    with open(os.path.join(CODE_DIR, name), encoding="utf-8") as fh:
        return fh.read()


def strip_line_comment(line):
    """Drop a // comment that is not inside a string literal."""
    out, i, in_str = [], 0, False
    while i < len(line):
        c = line[i]
        if c == '"' and (i == 0 or line[i - 1] != "\\"):
            in_str = not in_str
        if not in_str and line.startswith("//", i):
            break
        out.append(c)
        i += 1
    return "".join(out)


def sanitise_interpolation(src):
    lines = src.split("\n")
    kept = []
    for raw in lines:
        s = strip_line_comment(raw).rstrip()
        if s == "" and raw.strip() != "":
            continue  # comment-only line: drop it so it cannot end a macro body
        kept.append(s)
    # Restore continuations inside macro bodies.
    out, in_macro = [], False
    for idx, s in enumerate(kept):
        if s.lstrip().startswith("#define"):
            in_macro = True
            s = re.sub(r"\([^()]*[^\x00-\x7f][^()]*\)\)?", "", s)  # annotated parameter names
            s = re.sub(r"\(=\w+\)", "", s)
        if in_macro:
            nxt = kept[idx + 1] if idx + 1 < len(kept) else ""
            continues = nxt.strip() != "" and not nxt.lstrip().startswith("#")
            if continues and not s.endswith("\\"):
                s = s + " \\"
            if not continues:
                in_macro = False
                s = s.rstrip("\\").rstrip()
        out.append(s)
    return "\n".join(out)


def sanitise_evolution(src):
    lines = src.split("\n")
    assert lines[530].strip().startswith("//F0_in = F0_in + ModifydRho_F378"), "unexpected evolution.h layout"
    lines.insert(531, "}")  # closes if ( BFLReqF3_d[idx_xi] == 1 ){ in stream_collide (after original line 531)
    # original 842-1001 (now 843-1002) is the launcher; keep 1..841 and 1003..end (now 1004..)
    body = lines[:841] + lines[1002:]
    text = "\n".join(body)
    text = re.sub(r'#include\s+"[^"]+"', "", text)
    return text


def launch_args(evo_src, kernel, occurrence):
    """Argument list of the n-th launch of `kernel` in Launch_CollisionStreaming."""
    pat = kernel + "<<<"
    pos = -1
    for _ in range(occurrence + 1):
        pos = evo_src.index(pat, pos + 1)
    start = evo_src.index(">>>(", pos) + 4
    depth, i = 1, start
    while depth:
        c = evo_src[i]
        depth += (c == "(") - (c == ")")
        i += 1
    args = evo_src[start:i - 1]
    args = "\n".join(strip_line_comment(l) for l in args.split("\n"))
    return " ".join(args.split())


def build(nx, ny, nz, re_, ub, ndtfrc, massk=0, out=None, cxx="g++", opt="-O2"):
    evo = read("evolution.h")
    buffer_args = launch_args(evo, "stream_collide_Buffer", 0)
    interior_args = launch_args(evo, "stream_collide", 0)
    # the Buffer launch passes `start` = 3 as a literal; the body never uses it
    variables = read("variables.h")
    overrides = f"""
#undef NX
#undef NY
#undef NZ
#undef jp
#undef tau
#undef Re
#undef NDTFRC
#undef loop
#define NX {nx}
#define NY {ny}
#define NZ {nz}
#define jp 1
#define Re {re_!r}
#define tau (0.5 + 3.0*({ub!r})/((double)Re*minSize))
#define NDTFRC {ndtfrc}
#define REF_MASSK {massk}
#define REF_CALL_BUFFER stream_collide_Buffer({buffer_args})
#define REF_CALL_INTERIOR stream_collide({interior_args})
"""
    body = "\n".join([
        read("common.h"),
        read("model.h"),
        read("initialization.h").replace('#include "initializationTool.h"', read("initializationTool.h")),
        read("memory.h"),
        sanitise_interpolation(read("interpolationHillISLBM.h")),
        read("MRT_Matrix.h"),
        "#undef m_matrix",
        read("MRT_Process.h"),
        sanitise_evolution(evo),
    ])
    driver = open(os.path.join(HERE, "ref_driver.inc"), encoding="utf-8").read()
    marker = "// @@REF_BODY@@"
    head, tail = driver.split(marker, 1)
    tail = tail.split("\n", 1)[1]
    tu = "\n".join([SHIM, variables, overrides, head, body, tail])
    os.makedirs(OUT_DIR, exist_ok=True)
    if out is None:
        out = os.path.join(OUT_DIR, f"libislbm_ref_{nx}x{ny}x{nz}_re{re_:g}_nd{ndtfrc}_m{massk}.so")
    cmd = [cxx, "-x", "c++", "-", "-shared", "-fPIC", opt, "-ffp-contract=off", "-fno-fast-math",
           "-w", "-o", out]
    res = subprocess.run(cmd, input=tu.encode("utf-8"), capture_output=True)
    if res.returncode != 0:
        sys.stderr.write(res.stderr.decode("utf-8", "replace")[-6000:])
        raise RuntimeError("reference build failed")
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=32)
    ap.add_argument("--ny", type=int, default=64)
    ap.add_argument("--nz", type=int, default=48)
    ap.add_argument("--re", type=float, default=700.0)
    ap.add_argument("--ub", type=float, default=0.05)
    ap.add_argument("--ndtfrc", type=int, default=100)
    ap.add_argument("--massk", type=int, default=0)
    a = ap.parse_args()
    if not os.path.isdir(CODE_DIR):
        print("reference sources not present; nothing built")
        return 0
    print(build(a.nx, a.ny, a.nz, a.re, a.ub, a.ndtfrc, a.massk))
    return 0


if __name__ == "__main__":
    sys.exit(main())
