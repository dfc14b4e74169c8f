"""The two rewritings the CUDA path rests on, checked on the CPU against the
reference's own numbers (the golden fixtures of tests/golden/):

* the cycle energies in closed form,
      E_l^(k) = Eint[l] + (G[l-1] - G[l-k]) + link(l, l-k+1),
  G the prefix sums of Eint[c] + link(c, c+1) (the link(l, .) terms of the
  reference's recursion telescope), against the reference's ENk;
* the exchange estimator from the cycle probabilities,
      res[N] = -sum_l sum_{j<=l} G[l][j] E2[l][l-j+1],
  G[l][j] the connection probabilities of the exchange forces, against the
  reference's recursion for the primitive estimator.
"""
import numpy as np
import pytest

import fixtures
import orc
from helpers import assert_close

TIGHT = 1e-12


def _beads(fx, h, key):
    N, P, D = h["N"], h["P"], h["D"]
    return fx[key].reshape(N, P, D)  # the reference's bead order: particle-major


def _diff(a, b, box, image):
    t = a - b
    if image:
        t = t - box * np.rint(t / box)
    return t


def _closed_form_enk(fx, h):
    N, P = h["N"], h["P"]
    x = _beads(fx, h, "s1/x")
    m = fx["m"].reshape(N, P)
    w2 = h["omegaP"] ** 2
    box, image = h["box"], h["image"]

    def link(a, b):  # bead P of particle a to bead 1 of particle b, 0-based
        t = _diff(x[a, P - 1], x[b, 0], box, image)
        return 0.5 * m[a, P - 1] * w2 * float(t @ t)

    eint = np.zeros(N)
    for l in range(N):
        for j in range(P - 1):
            t = _diff(x[l, j], x[l, j + 1], box, image)
            eint[l] += 0.5 * m[l, j] * w2 * float(t @ t)
    g = np.array([eint[c] + link(c, c + 1) for c in range(N - 1)])
    G = np.concatenate([[0.0], np.cumsum(g)])  # G[n] = g[0] + ... + g[n-1]
    enk = np.zeros(orc.ntri(N))
    for l in range(1, N + 1):
        row = l * (l - 1) // 2
        enk[row] = eint[l - 1] + link(l - 1, l - 1)
        for k in range(2, l + 1):
            enk[row + k - 1] = eint[l - 1] + (G[l - 1] - G[l - k]) + link(l - 1, l - k)
    return enk, eint


@pytest.mark.parametrize("name", fixtures.PIMD_FIXTURES)
def test_cycle_energies_in_closed_form(name):
    fx = fixtures.load(name)
    h = fixtures.header(fx)
    enk, eint = _closed_form_enk(fx, h)
    assert_close(eint, fx["Eint"], TIGHT, f"{name} Eint")
    assert_close(enk, fx["ENk"], TIGHT, f"{name} ENk, closed form")


@pytest.mark.parametrize("name", fixtures.PIMD_FIXTURES)
def test_estimator_from_cycle_probabilities(name):
    fx = fixtures.load(name)
    h = fixtures.header(fx)
    N, P, D = h["N"], h["P"], h["D"]
    s = orc.OrcSim.from_fixture(fx)
    L = orc.lib()
    assert L.orc_nhc_vv3_1(s.ref, h["dt"]) == 0
    L.orc_reset_force(s.ref)
    ENk, _ = orc.fast_fill_ENk(s, N, P, h["omegaP"], h["image"])
    VBN = orc.fill_VB(N, h["beta"], h["vi"], ENk)
    Gm, _ = orc.fast_force_VB(s, N, P, h["beta"], h["vi"], h["omegaP"], h["image"], ENk, VBN)
    res = 0.0
    for l in range(1, N + 1):
        row = l * (l - 1) // 2
        for j in range(1, l + 1):
            res -= Gm[l - 1, j - 1] * ENk[row + l - j]
    add = D * N * P / (2 * h["beta"])
    assert_close([res + add], fx["s1/e_prim_exch"], TIGHT, f"{name} primitive estimator from G")
    # the probabilities of the cycles ending at each particle l, summed over
    # l, count the cycles: at least one, at most N
    ncyc = sum(Gm[l - 1, :l].sum() for l in range(1, N + 1))
    assert 1.0 - 1e-12 <= ncyc <= N + 1e-12
