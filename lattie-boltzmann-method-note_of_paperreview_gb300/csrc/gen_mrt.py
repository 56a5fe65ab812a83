"""Generate mrt_d3q19.cuh: sparse straight-line D3Q19 MRT relaxation.

The reference applies the collision as three dense 19x19 products (m = M f, meq = M feq,
f -= Mi S (m - meq); C/MRT_Process.h:4-179 with M, Mi, S of C/MRT_Matrix.h:4-68). Here the
same operator is emitted as straight-line code:
  * m - meq = M (f - feq) is one transform of d = f - feq;
  * opposite directions are paired (q, q'), e_q' = -e_q, so even-parity moments read the
    pair sums d_q + d_q' and odd-parity moments the pair differences d_q - d_q';
  * the conserved moments (rho, j; relaxation rate 0) are skipped;
  * the inverse is M^T diag(1/|row|^2) (rows of M are orthogonal), so the back-transform
    reuses the integer entries of M and one scale per moment;
  * equal integer coefficients are grouped into one multiply.
The moment basis is generated from its defining polynomials in e (d'Humieres et al. 2002,
the ordering of C/MRT_Matrix.h:27-46) and checked against that table by the tests.

Run: python gen_mrt.py > mrt_d3q19.cuh
"""
import sys

E = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1),
     (1, 1, 0), (-1, 1, 0), (1, -1, 0), (-1, -1, 0), (1, 0, 1), (-1, 0, 1), (1, 0, -1),
     (-1, 0, -1), (0, 1, 1), (0, -1, 1), (0, 1, -1), (0, -1, -1)]


def moment_rows():
    M = [[0] * 19 for _ in range(19)]
    for q, (ex, ey, ez) in enumerate(E):
        e2 = ex * ex + ey * ey + ez * ez
        row = [1, 19 * e2 - 30, (21 * e2 * e2 - 53 * e2 + 24) // 2, ex, (5 * e2 - 9) * ex, ey, (5 * e2 - 9) * ey,
               ez, (5 * e2 - 9) * ez, 3 * ex * ex - e2, (3 * e2 - 5) * (3 * ex * ex - e2), ey * ey - ez * ez,
               (3 * e2 - 5) * (ey * ey - ez * ez), ex * ey, ey * ez, ex * ez, (ey * ey - ez * ez) * ex,
               (ez * ez - ex * ex) * ey, (ex * ex - ey * ey) * ez]
        for c in range(19):
            M[c][q] = row[c]
    return M


PAIRS = [(1, 2), (3, 4), (5, 6), (7, 10), (8, 9), (11, 14), (12, 13), (15, 18), (16, 17)]
EVEN = [1, 2, 9, 10, 11, 12, 13, 14, 15]
ODD = [4, 6, 8, 16, 17, 18]
RATE = {1: "s_e", 2: "s_eps", 4: "s_q", 6: "s_q", 8: "s_q", 9: "s_nu", 10: "s_pi", 11: "s_nu", 12: "s_pi",
        13: "s_nu", 14: "s_nu", 15: "s_nu", 16: "s_m", 17: "s_m", 18: "s_m"}


def grouped(terms):
    """terms: list of (coef, name) -> expression with equal coefficients grouped."""
    by = {}
    for c, n in terms:
        if c:
            by.setdefault(c, []).append(n)
    parts = []
    for c in sorted(by, key=lambda v: (-abs(v), v)):
        s = " + ".join(by[c])
        s = f"({s})" if len(by[c]) > 1 else s
        if c == 1:
            parts.append(("+", s))
        elif c == -1:
            parts.append(("-", s))
        else:
            parts.append(("+", f"T({c})*{s}"))
    if not parts:
        return "T(0)"
    out = ("-" if parts[0][0] == "-" else "") + parts[0][1]
    for sign, s in parts[1:]:
        out += f" {sign} {s}"
    return out


def main():
    M = moment_rows()
    for a, b in PAIRS:
        assert all(-E[a][i] == E[b][i] for i in range(3))
    norms = {c: sum(M[c][q] ** 2 for q in range(19)) for c in range(19)}
    w = sys.stdout.write
    w("// Generated by gen_mrt.py -- do not edit. Sparse D3Q19 MRT relaxation.\n")
    w("// Operator of C/MRT_Process.h:4-179 (f -= Mi S (M f - M feq)) with M, Mi, S of C/MRT_Matrix.h.\n")
    w("#pragma once\n\n")
    w("// d[q] = F[q] - Feq[q] on entry; on exit F[q] has been relaxed. Rates: s_e (s1), s_eps (s2),\n")
    w("// s_q (s4, s6, s8), s_nu (s9, s11, s13, s14, s15), s_pi (s10, s12), s_m (s16, s17, s18).\n")
    w("template <typename T>\n__device__ __forceinline__ void mrt_relax(T (&F)[19], const T (&d)[19], T s_e, T s_eps, T s_q,\n")
    w("                                          T s_nu, T s_pi, T s_m) {\n")
    for p, (a, b) in enumerate(PAIRS):
        w(f"    const T S{p} = d[{a}] + d[{b}], A{p} = d[{a}] - d[{b}];\n")
    relax_body(w, M, norms, "d[0]")
    # the same operator from the pair sums / differences of d, given by the caller
    w("// The same relaxation from d0 = d[0] and the pair sums S[p] = d[a] + d[b] and differences\n")
    w("// A[p] = d[a] - d[b] of the opposite pairs (a, b) = " + " ".join(f"({a},{b})" for a, b in PAIRS) + ".\n")
    w("template <typename T>\n__device__ __forceinline__ void mrt_relax_pairs(T (&F)[19], T d0, const T (&S)[9], const T (&A)[9],\n")
    w("                                                T s_e, T s_eps, T s_q, T s_nu, T s_pi, T s_m) {\n")
    for p in range(9):
        w(f"    const T S{p} = S[{p}], A{p} = A[{p}];\n")
    relax_body(w, M, norms, "d0")
    tail(w)


def relax_body(w, M, norms, d0):
    for c in EVEN:
        terms = [(M[c][0], d0)] + [(M[c][a], f"S{p}") for p, (a, b) in enumerate(PAIRS)]
        w(f"    const T r{c} = {RATE[c]}*T(1.0/{norms[c]}.0)*({grouped(terms)});\n")
    for c in ODD:
        terms = [(M[c][a], f"A{p}") for p, (a, b) in enumerate(PAIRS)]
        w(f"    const T r{c} = {RATE[c]}*T(1.0/{norms[c]}.0)*({grouped(terms)});\n")
    w(f"    F[0] -= {grouped([(M[c][0], f'r{c}') for c in EVEN])};\n")
    for p, (a, b) in enumerate(PAIRS):
        ev = grouped([(M[c][a], f"r{c}") for c in EVEN])
        od = grouped([(M[c][a], f"r{c}") for c in ODD])
        w(f"    {{ const T ev = {ev}, od = {od};\n")
        w(f"      F[{a}] -= ev + od; F[{b}] -= ev - od; }}\n")
    w("}\n\n")


def tail(w):
    # second-moment tensor of d (for the Smagorinsky closure): even parity -> pair sums
    w("// Non-equilibrium momentum flux Pi_ab = sum_q e_qa e_qb d_q, returned as Q = Pi:Pi.\n")
    w("template <typename T>\n__device__ __forceinline__ T pi_neq_norm2(const T (&d)[19]) {\n")
    for p, (a, b) in enumerate(PAIRS):
        w(f"    const T S{p} = d[{a}] + d[{b}];\n")
    comps = {"xx": (0, 0), "yy": (1, 1), "zz": (2, 2), "xy": (0, 1), "yz": (1, 2), "xz": (0, 2)}
    for nm, (i, j) in comps.items():
        terms = [(E[a][i] * E[a][j], f"S{p}") for p, (a, b) in enumerate(PAIRS)]
        w(f"    const T p{nm} = {grouped(terms)};\n")
    w("    return pxx*pxx + pyy*pyy + pzz*pzz + T(2)*(pxy*pxy + pyz*pyz + pxz*pxz);\n}\n")
    w("\n// The same from the pair sums S[p] = d[a] + d[b].\n")
    w("template <typename T>\n__device__ __forceinline__ T pi_neq_norm2_pairs(const T (&S)[9]) {\n")
    for nm, (i, j) in comps.items():
        terms = [(E[a][i] * E[a][j], f"S[{p}]") for p, (a, b) in enumerate(PAIRS)]
        w(f"    const T p{nm} = {grouped(terms)};\n")
    w("    return pxx*pxx + pyy*pyy + pzz*pzz + T(2)*(pxy*pxy + pyz*pyz + pxz*pxz);\n}\n")


if __name__ == "__main__":
    main()
