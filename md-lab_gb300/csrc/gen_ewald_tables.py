"""Generates xmd_ewald_tables.h: piecewise polynomials for the real-space
Ewald kernel, so that the GPU evaluates no FP64 erfc/exp per image.

    h(x) = erfc(x) + 2 x exp(-x^2) / sqrt(pi)    force:  F = s h(alpha R) r / R^3
    e(x) = erfc(x)                               energy: E = s e(alpha R) / R

(h'(x) = -4 x^2 exp(-x^2)/sqrt(pi).)  Interval i = 0..NINT-1 is centred at
i w, [(i - 1/2) w, (i + 1/2) w], so that the kernel finds it by rounding x/w
to the nearest integer; on it a degree-DEG polynomial in t = 2 (x - i w)/w is
the Chebyshev interpolant computed with 40-digit arithmetic (mpmath), stored
in monomial form for Horner evaluation.  The script measures the absolute error of the
double-precision Horner evaluation against mpmath and records it in the
header.  Absolute accuracy is what the sums need: both functions are at most
1 and each image's contribution scales with them.

The FP32 kernels use one global approximation instead (no table lookups):
h(x) = exp(-x^2) (2x/sqrt(pi) + erfcx(x)) with erfcx(x) = exp(x^2) erfc(x)
~ t P(t), t = 1/(1 + x/2), P of degree EW32_DEG, fitted here by least
squares in relative error on Chebyshev nodes of [0, EW32_XFIT].

Run:  python gen_ewald_tables.py > xmd_ewald_tables.h   (needs mpmath, numpy)
"""
import mpmath as mp
import numpy as np

mp.mp.dps = 40
W, NINT, DEG = 0.015625, 373, 6
XMAX = (NINT - 0.5) * W


def h(x):
    return mp.erfc(x) + 2 * x * mp.e ** (-x * x) / mp.sqrt(mp.pi)


def e(x):
    return mp.erfc(x)


def interpolant(f, a, b, deg):
    n = deg + 1
    nodes = [mp.cos(mp.pi * (k + mp.mpf(1) / 2) / n) for k in range(n)]
    vals = [f((a + b) / 2 + (b - a) / 2 * t) for t in nodes]
    A = mp.matrix([[t ** j for j in range(n)] for t in nodes])
    c = mp.lu_solve(A, mp.matrix(vals))
    return [c[j] for j in range(n)]


def horner(cd, t):
    acc = cd[-1]
    for c in reversed(cd[:-1]):
        acc = acc * t + c
    return acc


def table(f):
    rows, worst = [], 0.0
    for i in range(NINT):
        a, b = (mp.mpf(i) - mp.mpf(1) / 2) * W, (mp.mpf(i) + mp.mpf(1) / 2) * W
        cd = [float(c) for c in interpolant(f, a, b, DEG)]
        for s in range(401):
            t = -1 + 2 * mp.mpf(s) / 400
            x = (a + b) / 2 + (b - a) / 2 * t
            worst = max(worst, abs(horner(cd, float(t)) - f(x)))
        rows.append(cd)
    return rows, float(worst)


EW32_C, EW32_DEG, EW32_XFIT = 0.5, 8, 4.7


def erfcx(x):
    return mp.erfc(x) * mp.e ** (x * x)


def erfcx_fit():
    """coefficients c_k of erfcx(x) ~ t sum_k c_k t^k, t = 1/(1 + C x)"""
    x = EW32_XFIT * (1 - np.cos(np.linspace(0, np.pi, 3000))) / 2
    t = 1 / (1 + EW32_C * x)
    y = np.array([float(erfcx(mp.mpf(float(v)))) for v in x])
    A = np.vstack([t ** (k + 1) for k in range(EW32_DEG + 1)]).T
    c, *_ = np.linalg.lstsq(A / y[:, None], np.ones_like(y), rcond=None)
    xe = np.linspace(0, EW32_XFIT, 2001)
    te = 1 / (1 + EW32_C * xe)
    ye = np.array([float(erfcx(mp.mpf(float(v)))) for v in xe])
    fit = np.vstack([te ** (k + 1) for k in range(EW32_DEG + 1)]).T @ c
    return [float(v) for v in c], float(np.max(np.abs(fit - ye) / ye))


def emit(name, rows):
    """An initializer macro, usable for host arrays and __constant__ arrays."""
    out = [f"#define {name}_INIT {{ \\"]
    for r in rows:
        out.append("    {" + ", ".join(repr(c) for c in r) + "}, \\")
    out.append("  }")
    return "\n".join(out)


if __name__ == "__main__":
    th, eh = table(h)
    te, ee = table(e)
    print(f"""// xmd_ewald_tables.h -- generated by gen_ewald_tables.py; do not edit.
//
// Piecewise polynomials on [0, {XMAX}] ({NINT} intervals of width {W} centred
// at i w, degree {DEG}, variable t = 2 (x - i w)/w in [-1, 1]) for
//   EW_H:    erfc(x) + 2 x exp(-x^2)/sqrt(pi)   max |error| {eh:.2e}
//   EW_ERFC: erfc(x)                            max |error| {ee:.2e}
// (errors of the double-precision Horner evaluation against 40-digit values
// at 401 points per interval).
#pragma once
#define EW_XMAX {XMAX}
#define EW_NINT {NINT}
#define EW_DEG {DEG}
#define EW_INV_W {1 / W!r}
""")
    print(emit("EW_H", th))
    print(emit("EW_ERFC", te))
    c32, e32 = erfcx_fit()
    print(f"""
// FP32 form: erfcx(x) = exp(x^2) erfc(x) ~ t (c0 + c1 t + ... + c{EW32_DEG} t^{EW32_DEG}),
// t = 1/(1 + {EW32_C} x), least squares in relative error on [0, {EW32_XFIT}]:
// max relative error {e32:.2e} (double evaluation)
#define EW32_C {EW32_C!r}
#define EW32_DEG {EW32_DEG}
#define EW32_XFIT {EW32_XFIT!r}
#define EW32_ERFCX_INIT {{ {", ".join(repr(v) for v in c32)} }}""")
