"""The oracle's definitions of the learned residual, checked on the CPU:
gradients against finite differences, BF16 rounding against its definition,
descriptors against a hand-computed two-particle case."""
import math

import numpy as np
import pytest

import orc

NP = 128 * 64 + 128 + 128 * 128 + 128 + 4 * 128 + 4


def random_batch(rows, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((rows, 64))
    V = np.zeros((rows, 12))
    V[:, :9] = rng.standard_normal((rows, 9))
    V[:, 9] = 1.0
    T = rng.standard_normal((rows, 4))
    p = np.zeros(NP)
    p[:128 * 64] = rng.uniform(-0.25, 0.25, 128 * 64)
    o = 128 * 64
    p[o:o + 128] = 0.1 * rng.standard_normal(128)
    o += 128
    p[o:o + 128 * 128] = rng.uniform(-0.2, 0.2, 128 * 128)
    o += 128 * 128
    p[o:o + 128] = 0.1 * rng.standard_normal(128)
    o += 128
    p[o:o + 512] = rng.uniform(-0.2, 0.2, 512)
    o += 512
    p[o:o + 4] = 0.1 * rng.standard_normal(4)
    return X, V, T, p


def test_parameter_count():
    assert orc.lib().orc_mlp_nparam() == NP


def test_bf16_rounding_ties_to_even():
    b = orc.lib().orc_bf16
    assert b(1.0) == 1.0
    # BF16 spacing at 1 is 2^-7
    assert b(1.0 + 2.0 ** -8) == 1.0  # tie, even neighbour below
    assert b(1.0 + 3 * 2.0 ** -8) == 1.0 + 2.0 ** -6  # tie, even neighbour above
    assert b(1.0 + 2.0 ** -8 + 2.0 ** -12) == 1.0 + 2.0 ** -7
    assert b(1.0 + 2.0 ** -8 - 2.0 ** -12) == 1.0
    assert b(-3.0) == -3.0


def test_gradient_matches_finite_differences():
    X, V, T, p = random_batch(6, 1)
    V[2, 9] = 0.0  # a padding row contributes nothing
    g, loss = orc.mlp_grad(X, V, T, p, we=0.7, wf=1.3)
    rng = np.random.default_rng(2)
    # every bias, and a sample of every weight matrix
    idx = list(range(128 * 64, 128 * 64 + 128)) + list(range(NP - 4, NP))
    idx += list(rng.choice(128 * 64, 40, replace=False))
    idx += list(128 * 64 + 128 + rng.choice(128 * 128, 40, replace=False))
    idx += list(NP - 4 - 512 + rng.choice(512, 20, replace=False))
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (orc.mlp_loss(X, V, T, pp, 0.7, 1.3) - orc.mlp_loss(X, V, T, pm, 0.7, 1.3)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])
    # the loss terms are reported unscaled
    total = orc.mlp_loss(X, V, T, p, 0.7, 1.3)
    assert math.isclose(total, loss.sum() / 6, rel_tol=1e-12)


def test_rounded_gradient_close_to_exact():
    X, V, T, p = random_batch(64, 3)
    g0, _ = orc.mlp_grad(X, V, T, p, bf=0)
    g1, _ = orc.mlp_grad(X, V, T, p, bf=1)
    assert np.linalg.norm(g1 - g0) <= 0.05 * np.linalg.norm(g0)


def test_two_particle_descriptor():
    box = np.array([10.0, 10.0, 10.0])
    rc, nb = 5.0, 64
    rng = np.random.default_rng(4)
    B = rng.standard_normal((nb, 32))
    mu, sg = [1.25, 2.5, 3.75], [0.75, 0.75, 0.75]
    r = 2.3456
    x = np.array([[1.0, 1.0, 1.0], [1.0 + r, 1.0, 1.0]])
    F, Vv = orc.desc_features(x, box, rc, B, mu, sg, nb)
    h = rc / nb
    t = r / h - 0.5
    b0 = int(math.floor(t))
    w = t - b0
    fc = (1 - r * r / (rc * rc)) ** 2
    expect = fc * ((1 - w) * B[b0] + w * B[b0 + 1])
    np.testing.assert_allclose(F[0, :32], expect, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(F[1, :32], expect, rtol=1e-12, atol=1e-14)
    q = [fc * math.exp(-(r - m) ** 2 / (2 * s * s)) / r for m, s in zip(mu, sg)]
    for m in range(3):
        assert math.isclose(Vv[0, 3 * m], -q[m] * r, rel_tol=1e-12)
        assert math.isclose(Vv[1, 3 * m], q[m] * r, rel_tol=1e-12)
    # structure-factor shells: |S(k)|^2 = 2 + 2 cos(k . d) for two particles,
    # averaged over each shell's half-space vectors, divided by N = 2
    shells = [1, 2, 3, 4, 5, 6, 8, 9, 10, 11, 12, 13, 14, 16, 17, 18, 19, 20, 21, 22, 24, 25, 26, 27, 29, 30,
              32, 33, 34, 35, 36, 37]
    for i, n2 in enumerate(shells):
        vals = []
        for a in range(0, 7):
            for b in range(-6, 7):
                for c in range(-6, 7):
                    if not (a > 0 or (a == 0 and b > 0) or (a == 0 and b == 0 and c > 0)):
                        continue
                    if a * a + b * b + c * c == n2:
                        vals.append(2 + 2 * math.cos(2 * math.pi * a * r / box[0]))
        assert math.isclose(F[0, 32 + i], math.sqrt(np.mean(vals) / 2), rel_tol=1e-12)
        assert F[1, 32 + i] == F[0, 32 + i]
    # minimum image: the same pair across the boundary
    x2 = np.array([[0.5, 1.0, 1.0], [0.5 - r + 10.0, 1.0, 1.0]])
    F2, _ = orc.desc_features(x2, box, rc, B, mu, sg, nb)
    np.testing.assert_allclose(F2[0], F[0], rtol=1e-10, atol=1e-12)
    # beyond the cut-off nothing is deposited
    x3 = np.array([[1.0, 1.0, 1.0], [1.0, 1.0 + 5.2, 1.0]])
    F3, V3 = orc.desc_features(x3, 2 * box, rc, B, mu, sg, nb)
    assert not F3[:, :32].any() and not V3.any()
