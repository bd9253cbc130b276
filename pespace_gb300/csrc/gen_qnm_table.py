"""Kerr quasi-normal-mode frequencies for the IMRPhenomD/HM ringdown, by
Leaver's continued-fraction method (E. W. Leaver, Proc. R. Soc. A 402, 285
(1985)), written out as the C header ``pes_qnm_table.h``.

For each mode (l, m) of spin weight s = -2 and overtone n = 0 the complex
frequency M omega(a) of a Kerr black hole of mass M and dimensionless spin a
is tabulated on a grid uniform in u = sqrt(1 - a), a in [-A_MAX, A_MAX]
(negative a continues the mode to anti-aligned remnant spins: the
retrograde branch).  The header holds, per mode, Re(M omega) and
-Im(M omega) at the nodes and the second derivatives of their natural cubic
splines in u, so that a caller evaluates a C2 interpolant.

Method, in Leaver's units (2M = 1, a_L = a/2, omega_L = 2 M omega): the
angular and radial Teukolsky equations give three-term recurrences whose
minimal solutions exist only when their continued fractions vanish; for a
given omega the angular condition fixes the separation constant A, and the
radial condition is solved for omega by secant iteration, continued in a
from the Schwarzschild value.  The continued fractions are evaluated
bottom-up from a depth at which their value has converged.

    python gen_qnm_table.py            # writes pes_qnm_table.h beside this file
"""

import cmath
import os
import sys

import numpy as np

MODES = [(2, 2), (2, 1), (3, 3), (3, 2), (4, 4), (4, 3)]
A_MAX = 0.999
N_NODES = 401
S = -2


def angular_cf(A, aw, l, m, depth=120):
    """Leaver's angular continued fraction, inverted N = l - (k1 + k2) times so
    that the root followed from a = 0 is the l-th one (it vanishes at the
    separation constant)."""
    k1, k2 = abs(m - S) / 2.0, abs(m + S) / 2.0
    N = int(round(l - (k1 + k2)))

    def alpha(n):
        return -2.0 * (n + 1) * (n + 2 * k1 + 1)

    def beta(n):
        return (n * (n - 1) + 2 * n * (k1 + k2 + 1 - 2 * aw) - (2 * aw * (2 * k1 + S + 1) - (k1 + k2) * (k1 + k2 + 1))
                - (aw * aw + S * (S + 1) + A))

    def gamma(n):
        return 2 * aw * (n + k1 + k2 + S)

    # upward part: alpha_N gamma_{N+1} / (beta_{N+1} - alpha_{N+1} gamma_{N+2} / (...))
    t = 0.0
    for n in range(N + depth, N, -1):
        t = alpha(n - 1) * gamma(n) / (beta(n) - t)
    # downward part: alpha_{N-1} gamma_N / (beta_{N-1} - alpha_{N-2} gamma_{N-1} / (... beta_0))
    d = 0.0
    for n in range(0, N):
        d = alpha(n) * gamma(n + 1) / (beta(n) - d) if n > 0 else alpha(0) * gamma(1) / beta(0)
    return beta(N) - d - t


def radial_cf(w, A, a, m, depth):
    """Leaver's radial continued fraction in units 2M = 1 (a <= 1/2)."""
    b = cmath.sqrt(1.0 - 4.0 * a * a)
    x = w / 2.0 - a * m
    c0 = 1.0 - S - 1j * w - (2j / b) * x
    c1 = -4.0 + 2j * w * (2.0 + b) + (4j / b) * x
    c2 = S + 3.0 - 3j * w - (2j / b) * x
    c3 = w * w * (4.0 + 2.0 * b - a * a) - 2.0 * a * m * w - S - 1.0 + (2.0 + b) * 1j * w - A + ((4.0 * w + 2j) / b) * x
    c4 = S + 1.0 - 2.0 * w * w - (2 * S + 3) * 1j * w - ((4.0 * w + 2j) / b) * x
    t = 0.0
    for n in range(depth, 0, -1):
        al = (n - 1) * (n - 1) + (c0 + 1.0) * (n - 1) + c0
        be = -2.0 * n * n + (c1 + 2.0) * n + c3
        ga = n * n + (c2 - 3.0) * n + c4 - c2 + 2.0
        t = al * ga / (be - t)
    return c3 - t  # beta_0 = c3


def secant(f, x0, x1, tol=1e-14, maxit=60):
    f0, f1 = f(x0), f(x1)
    for _ in range(maxit):
        if f1 == f0:
            break
        x2 = x1 - f1 * (x1 - x0) / (f1 - f0)
        x0, f0 = x1, f1
        x1, f1 = x2, f(x2)
        if abs(x1 - x0) < tol * max(1.0, abs(x1)):
            return x1
    return x1


def separation(aw, l, m, A_guess):
    return secant(lambda A: angular_cf(A, aw, l, m), A_guess, A_guess * (1 + 1e-6) + 1e-6)


def qnm(a, l, m, w_guess, A_guess, depth):
    """M omega and A at spin a (|a| < 1) from guesses (Leaver-unit omega)."""
    aL = a / 2.0
    state = {"A": A_guess}

    def f(w):
        A = separation(aL * w, l, m, state["A"])
        state["A"] = A
        return radial_cf(w, A, aL, m, depth)

    w = secant(f, w_guess, w_guess * (1 + 1e-6))
    return w, state["A"]


def mode_table(l, m, u, depth=3000):
    """M omega at a = 1 - u^2 for the grid u (continued from a = 0)."""
    a_nodes = 1.0 - u * u
    w0 = {2: 0.747343368 - 0.177924631j, 3: 1.198886 - 0.185406j, 4: 1.618357 - 0.188328j}[l]
    A0 = float(l * (l + 1) - S * (S + 1))
    out = np.zeros(len(u), dtype=complex)
    # march outward from a = 0 in both directions through the sorted nodes
    order = np.argsort(a_nodes)
    i0 = int(np.searchsorted(a_nodes[order], 0.0))
    for direction in (+1, -1):
        w, A, a_prev = w0, A0, 0.0
        w, A = qnm(0.0, l, m, w, A, depth)
        idx = range(i0, len(u)) if direction > 0 else range(i0 - 1, -1, -1)
        for k in idx:
            a_t = a_nodes[order[k]]
            # sub-steps keep the continuation on the branch
            nsub = max(1, int(abs(a_t - a_prev) / 0.01))
            for j in range(1, nsub + 1):
                a_s = a_prev + (a_t - a_prev) * j / nsub
                w, A = qnm(a_s, l, m, w, A, depth)
            a_prev = a_t
            out[order[k]] = w / 2.0  # M omega
    return out


def natural_spline_d2(x, y):
    """Second derivatives of the natural cubic spline through (x, y)."""
    n = len(x)
    h = np.diff(x)
    A = np.zeros((n, n))
    r = np.zeros(n)
    A[0, 0] = A[-1, -1] = 1.0
    for i in range(1, n - 1):
        A[i, i - 1] = h[i - 1]
        A[i, i] = 2.0 * (h[i - 1] + h[i])
        A[i, i + 1] = h[i]
        r[i] = 6.0 * ((y[i + 1] - y[i]) / h[i] - (y[i] - y[i - 1]) / h[i - 1])
    return np.linalg.solve(A, r)


def main(out_path):
    u = np.linspace(np.sqrt(1.0 - A_MAX), np.sqrt(1.0 + A_MAX), N_NODES)
    rows = []
    for l, m in MODES:
        w = mode_table(l, m, u)
        re, im = w.real, -w.imag
        rows.append((l, m, re, natural_spline_d2(u, re), im, natural_spline_d2(u, im)))
        print(f"mode ({l},{m}): a=0 -> {w[np.argmin(np.abs(1 - u * u))]:.10f}", file=sys.stderr)

    def arr(v):
        return ",\n    ".join(", ".join(f"{x:.17g}" for x in v[i:i + 4]) for i in range(0, len(v), 4))

    lines = [
        "// Generated by gen_qnm_table.py (Leaver's continued fractions); do not edit.",
        "// Kerr quasi-normal modes (s = -2, n = 0): M omega = re - i im on a grid",
        "// uniform in u = sqrt(1 - a), with natural-spline second derivatives.",
        "#pragma once",
        "",
        f"#define PES_QNM_MODES {len(MODES)}",
        f"#define PES_QNM_NODES {N_NODES}",
        f"#define PES_QNM_U0 {u[0]:.17g}",
        f"#define PES_QNM_DU {(u[-1] - u[0]) / (N_NODES - 1):.17g}",
        f"#define PES_QNM_A_MAX {A_MAX:.17g}",
        "",
        "// mode order: " + ", ".join(f"({l},{m})" for l, m in MODES),
        "static const int kQnmModeLM[PES_QNM_MODES][2] = {" + ", ".join(f"{{{l}, {m}}}" for l, m in MODES) + "};",
        "",
        "// [mode][0: re, 1: re'', 2: im, 3: im''][node]",
        "PES_QNM_STORAGE double kQnmTable[PES_QNM_MODES][4][PES_QNM_NODES] = {",
    ]
    for l, m, re, re2, im, im2 in rows:
        lines.append(f"  {{  // ({l},{m})")
        for v in (re, re2, im, im2):
            lines.append("   {" + arr(v) + "},")
        lines.append("  },")
    lines.append("};")
    with open(out_path, "w") as f:
        f.write("\n".join(lines) + "\n")
    print("wrote", out_path, file=sys.stderr)


if __name__ == "__main__":
    main(os.path.join(os.path.dirname(os.path.abspath(__file__)), "pes_qnm_table.h"))
