"""The error budget of the FP64 form's FP32 terms, restated on the CPU.

The FP64 force kernels evaluate two groups of small terms on the FP32 pipe:
real-space Ewald images at alpha R >= 4 (from the FP32 minimum image, with
the FP32 form's h through the fitted erfcx of xmd_ewald_tables.h) and the
reciprocal columns whose force weight is below 1e-7 of the largest.  This
file emulates both in NumPy float32 (the fit's coefficients read from the
header, exp and the divisions in float32) next to an FP64 evaluation of the
same sums, and checks the bounds the design rests on; the GPU test
test_full_size_far_images_fp32_vs_strict_fp64 measures the kernels
themselves against the strict form.
"""
import math
import os
import re

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
TABLES = os.path.join(HERE, "..", "md-lab_gb300", "csrc", "xmd_ewald_tables.h")
F32 = np.float32


def _fit():
    txt = open(TABLES).read()
    c = float(re.search(r"#define EW32_C ([0-9.eE+-]+)", txt).group(1))
    coef = [float(v) for v in re.search(r"#define EW32_ERFCX_INIT \{([^}]*)\}", txt).group(1).split(",")]
    return c, coef


def _h32(R2, alpha, c, coef):
    """h(alpha R) / R^3 in float32 as ew_h32 computes it"""
    R2 = R2.astype(F32)
    ri = (F32(1) / np.sqrt(R2)).astype(F32)
    x = (F32(alpha) * (R2 * ri)).astype(F32)
    t = (F32(1) / (F32(c) * x + F32(1))).astype(F32)
    q = F32(coef[-1])
    for k in range(len(coef) - 2, -1, -1):
        q = (q * t + F32(coef[k])).astype(F32)
    e = np.exp((-(x * x)).astype(F32)).astype(F32)
    return (e * (x * F32(1.1283791670955126) + q * t).astype(F32) * (ri * ri * ri)).astype(F32)


def _real_space(N, seed, xsplit=4.0, xcut=5.2, beads=6):
    """largest |F_split - F_fp64| per bead (unit strength) over a few beads"""
    erfc = pytest.importorskip("scipy.special").erfc
    c, coef = _fit()
    rng = np.random.default_rng(seed)
    L = (4 * math.pi * N / 3) ** (1 / 3)
    alpha = 5.6 / L
    x = rng.uniform(0, L, (N, 3))
    worst = 0.0
    for a in range(min(beads, N)):
        d = x[a] - np.delete(x, a, 0)
        sh = np.rint(d / L)
        m = d - sh * L
        mf = ((x[a].astype(F32) - np.delete(x, a, 0).astype(F32)) - sh.astype(F32) * F32(L)).astype(F32)
        f64 = np.zeros(3)
        near = np.zeros(3)
        far = np.zeros(3, dtype=F32)
        for k in np.array([(i, j, l) for i in (-1, 0, 1) for j in (-1, 0, 1) for l in (-1, 0, 1)]):
            t = m - k * L
            R = np.sqrt((t * t).sum(1))
            xr = alpha * R
            val = np.where(xr < xcut, (erfc(xr) + 2 * xr * np.exp(-xr * xr) / math.sqrt(math.pi)) / R ** 3, 0.0)
            f64 += (t * val[:, None]).sum(0)
            near += (t * np.where(xr < xsplit, val, 0.0)[:, None]).sum(0)
            tf = (mf - k.astype(F32) * F32(L)).astype(F32)
            R2f = (tf * tf).sum(1).astype(F32)
            sel = (R2f >= F32((xsplit / alpha) ** 2)) & (R2f < F32((xcut / alpha) ** 2))
            far += (tf * np.where(sel, _h32(R2f, alpha, c, coef), F32(0))[:, None]).sum(0).astype(F32)
        worst = max(worst, float(np.abs(near + far.astype(np.float64) - f64).max()))
    return worst


@pytest.mark.parametrize("N", [8, 64, 512])
def test_far_images_in_fp32_stay_below_1e_12(N):
    """the far images' FP32 evaluation changes a bead's real-space force by
    under 2e-12 of the pair strength (the sum of their sizes is 1e-7 ... 4e-7
    of it, the FP32 relative error a few 1e-6)"""
    worst = max(_real_space(N, seed) for seed in range(2))
    print(N, worst)
    assert worst < 2e-12


def test_fp32_columns_stay_below_1e_12_of_each_force():
    """the reciprocal columns of force weight below 1e-7 of the largest
    (nx^2 + ny^2 >= 49 at alpha L = 5.6), with every phase factor off by a
    relative 1e-6 (far above FP32's rounding), move each particle's
    reciprocal force by under 1e-11 of its own size; the next lower
    threshold, nx^2 + ny^2 >= 36, would not stay below 1e-10"""
    rng = np.random.default_rng(1)
    N, ns = 512, 10
    L = (4 * math.pi * N / 3) ** (1 / 3)
    alpha = 5.6 / L
    x = rng.uniform(0, L, (N, 3))
    ks = np.array([(a, b, c) for a in range(ns + 1) for b in range(-ns, ns + 1) for c in range(-ns, ns + 1)
                   if (a > 0 or b > 0 or (b == 0 and c > 0)) and a * a + b * b + c * c <= 111], dtype=float)
    G = ks / L
    G2 = (G * G).sum(1)
    coef = np.exp(-math.pi ** 2 * G2 / alpha ** 2) / G2
    w = coef * np.sqrt(G2)
    E = np.exp(2j * math.pi * (x @ ks.T) / L)

    def force(Ep):
        im = (np.conj(Ep) * Ep.sum(0)[None, :]).imag
        return (im * coef[None, :]) @ G

    F = force(E)
    noise = 1e-6 * rng.standard_normal(E.shape) + 1j * 1e-6 * rng.standard_normal(E.shape)

    def err(outer):
        Ep = E.copy()
        Ep[:, outer] = E[:, outer] * (1 + noise[:, outer])
        return (np.abs(force(Ep) - F).max(1) / np.abs(F).max(1)).max()

    col_w = {}
    for (a, b, _), v in zip(ks, w):
        col_w[(a, b)] = max(col_w.get((a, b), 0.0), v)
    outer = np.array([col_w[(a, b)] < 1e-7 * w.max() for a, b, _ in ks])
    assert outer.sum() == ((ks[:, 0] ** 2 + ks[:, 1] ** 2) >= 49).sum()
    e49 = err(outer)
    e36 = err((ks[:, 0] ** 2 + ks[:, 1] ** 2) >= 36)
    print("nx^2+ny^2 >= 49:", e49, ">= 36:", e36)
    assert e49 < 1e-11
    assert e36 > 1e-11
