"""The generated sparse MRT operator (csrc/mrt_d3q19.cuh) against the dense form of the
reference (f -= Mi S (M f - M feq), C/MRT_Process.h) with the reference's own M and Mi,
which the golden-fixture check pins through the oracle."""
import os
import subprocess
import sys

import numpy as np

from conftest import PKG, ROOT

CSRC = os.path.join(PKG, "csrc")


def translate(header):
    body = header.split("T s_nu, T s_pi, T s_m) {")[1].split("\n}\n")[0]
    out = []
    for line in body.split("\n"):
        l = line.strip().replace("const T ", "").replace("T(", "(").replace("{", "").replace("}", "")
        for part in l.split(";"):
            part = part.strip()
            if not part:
                continue
            if part.count("=") == 2 and "F[" not in part:
                a, b = part.split(", ", 1)
                out += [a, b]
            else:
                out.append(part)
    return "\n".join(out)


def test_generated_header_is_current():
    res = subprocess.run([sys.executable, os.path.join(CSRC, "gen_mrt.py")], capture_output=True, text=True, check=True)
    assert res.stdout == open(os.path.join(CSRC, "mrt_d3q19.cuh")).read()


def test_sparse_operator_matches_dense(oracle_mod):
    sys.path.insert(0, CSRC)
    import gen_mrt
    M = np.array(gen_mrt.moment_rows(), dtype=float)
    O = oracle_mod.Oracle(8, 16, 16)
    Mref = np.stack([O.get("M", c) for c in range(19)])
    Miref = np.stack([O.get("Mi", q) for q in range(19)])
    assert np.array_equal(M, Mref)
    np.testing.assert_allclose(M @ Miref, np.eye(19), atol=1e-14)
    code = translate(open(os.path.join(CSRC, "mrt_d3q19.cuh")).read())
    rng = np.random.default_rng(3)
    tau = 0.5084
    s = np.array([0, 1.19, 1.4, 0, 1.2, 0, 1.2, 0, 1.2, 1 / tau, 1.4, 1 / tau, 1.4, 1 / tau, 1 / tau, 1 / tau, 1.5, 1.5, 1.5])
    for _ in range(20):
        F = rng.random(19)
        Feq = F + 1e-3 * rng.standard_normal(19)
        ref = F - Miref @ (s * (Mref @ F - Mref @ Feq))
        env = dict(F=F.copy(), d=F - Feq, s_e=1.19, s_eps=1.4, s_q=1.2, s_nu=1 / tau, s_pi=1.4, s_m=1.5)
        exec(code, {}, env)
        np.testing.assert_allclose(env["F"], ref, rtol=0, atol=1e-15)


def test_pair_form_matches_dense(oracle_mod):
    """mrt_relax_pairs (the FP32 tiled kernels' form: pair sums/differences of F - Feq given by
    the caller) against the dense reference operator."""
    O = oracle_mod.Oracle(8, 16, 16)
    Mref = np.stack([O.get("M", c) for c in range(19)])
    Miref = np.stack([O.get("Mi", q) for q in range(19)])
    header = open(os.path.join(CSRC, "mrt_d3q19.cuh")).read()
    code = translate(header.split("void mrt_relax_pairs")[1].replace(
        "T s_e, T s_eps, T s_q, T s_nu, T s_pi, T s_m) {", "T s_nu, T s_pi, T s_m) {", 1))
    pa, pb = [1, 3, 5, 7, 8, 11, 12, 15, 16], [2, 4, 6, 10, 9, 14, 13, 18, 17]
    rng = np.random.default_rng(5)
    tau = 0.6
    s = np.array([0, 1.19, 1.4, 0, 1.2, 0, 1.2, 0, 1.2, 1 / tau, 1.4, 1 / tau, 1.4, 1 / tau, 1 / tau, 1 / tau, 1.5, 1.5, 1.5])
    for _ in range(20):
        F = rng.random(19)
        d = 1e-3 * rng.standard_normal(19)
        ref = F - Miref @ (s * (Mref @ d))
        env = dict(F=F.copy(), d0=d[0], S=[d[a] + d[b] for a, b in zip(pa, pb)], A=[d[a] - d[b] for a, b in zip(pa, pb)],
                   s_e=1.19, s_eps=1.4, s_q=1.2, s_nu=1 / tau, s_pi=1.4, s_m=1.5)
        exec(code, {}, env)
        np.testing.assert_allclose(env["F"], ref, rtol=0, atol=1e-15)
