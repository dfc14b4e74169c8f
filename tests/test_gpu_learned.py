"""The learned Ewald residual on the GPU: tensor-core kernels against the
oracle's definitions (forward pass, gradients, descriptors), and the whole
pipeline (collect, train, judge, attach) on a small electron gas, showing
what the trained network gains over the truncated sum alone."""
import ctypes as C
import math

import numpy as np
import pytest

import orc
import xmd_x
from gpu_common import random_state

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    return xmd_x.load(3, 4)


def ueg(lib, N, P, nsum, seed, rs=1.0, theta=0.5, vi=0.5):
    box = (4 * math.pi * N / 3) ** (1 / 3) * rs
    TF = 0.5 * (6 * math.pi ** 2 * N / box ** 3) ** (2 / 3)
    T = theta * TF
    xmd_x.set_potentials(lib, coul_s=1.0, alpha=5.6 / box, nsum=nsum)
    st = random_state(3, 4, N, P, T, box, True, seed)
    s = xmd_x.PimdSystem(lib, N, P, vi, T, box=box)
    s.set_state(**st)
    return s, box, T, st


def random_params(n, seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(n, np.float32)
    p[:8192] = rng.uniform(-0.3, 0.3, 8192)
    p[8192:8320] = 0.1 * rng.standard_normal(128)
    p[8320:8320 + 16384] = rng.uniform(-0.2, 0.2, 16384)
    p[24704:24832] = 0.1 * rng.standard_normal(128)
    p[24832:25344] = rng.uniform(-0.3, 0.3, 512)
    p[25344:] = 0.1 * rng.standard_normal(4)
    return p


@pytest.fixture(scope="module")
def small(lib):
    s, box, T, st = ueg(lib, 64, 4, 4, seed=7)
    m = xmd_x.EwaldModel(lib, s, nsum_cheap=2, capacity=2, seed=3)
    yield lib, s, m, box, st
    m.free()
    s.free()


def test_tensor_core_layout_selftest(lib):
    err = (C.c_double * 5)()
    lib.check(lib.md_gb300_tc_selftest_x(err), "self-test")
    print("self-test errors (K-major, A MN v0, A MN v1, B MN v0, B MN v1):", list(err))
    assert err[0] < 1e-3, list(err)
    # the reading the training kernel uses: stride field = M/N direction
    assert err[1] < 1e-3 and err[3] < 1e-3, list(err)


def test_forward_matches_oracle(small):
    lib, s, m, box, st = small
    p = random_params(lib.md_gb300_ewald_model_nparam_x(), 11)
    m.params(p)
    np.testing.assert_array_equal(m.params(), p)
    X = np.random.default_rng(12).standard_normal((300, 64)).astype(np.float32)  # 3 tiles, last one partial
    Y = m.forward(X)
    Yo = orc.mlp_forward(X.astype(np.float64), p.astype(np.float64), bf=1)
    err = np.abs(Y - Yo)
    # FP32 tensor-core sums vs double; a BF16 activation may round the other
    # way when its FP32 value sits on a rounding boundary (2^-8 relative)
    assert np.median(err) < 1e-5, np.median(err)
    assert err.max() < 5e-3 * max(1.0, np.abs(Yo).max()), err.max()


def _tensor_errors(g, go):
    parts = {"W1": (0, 8192), "b1": (8192, 8320), "W2": (8320, 24704), "b2": (24704, 24832),
             "W3": (24832, 25344), "b3": (25344, 25348)}
    return {k: float(np.linalg.norm(g[a:b] - go[a:b]) / max(np.linalg.norm(go[a:b]), 1e-30))
            for k, (a, b) in parts.items()}


@pytest.mark.parametrize("rows", [256, 300])
def test_gradient_matches_oracle(small, rows):
    lib, s, m, box, st = small
    p = random_params(lib.md_gb300_ewald_model_nparam_x(), 21)
    m.params(p)
    rng = np.random.default_rng(rows)
    X = rng.standard_normal((rows, 64)).astype(np.float32)
    V = np.zeros((rows, 12), np.float32)
    V[:, :9] = rng.standard_normal((rows, 9))
    V[:, 9] = 1.0
    V[::7, 9] = 0.0  # some rows carry no weight
    T = rng.standard_normal((rows, 4)).astype(np.float32)
    g, loss = m.grad(X, V, T, we=0.8, wf=1.2)
    go, lo = orc.mlp_grad(X.astype(np.float64), V.astype(np.float64), T.astype(np.float64), p.astype(np.float64),
                          0.8, 1.2, 1.0 / rows, bf=1)
    errs = _tensor_errors(g.astype(np.float64), go)
    assert max(errs.values()) < 1e-2, errs
    np.testing.assert_allclose(loss, lo, rtol=1e-4)
    # and against the exact (unrounded) gradient: BF16 costs a few per cent at most
    ge, _ = orc.mlp_grad(X.astype(np.float64), V.astype(np.float64), T.astype(np.float64), p.astype(np.float64),
                         0.8, 1.2, 1.0 / rows, bf=0)
    assert max(_tensor_errors(g.astype(np.float64), ge).values()) < 0.05


def test_descriptors_match_oracle(small):
    lib, s, m, box, st = small
    N, P = 64, 4
    F, V = m.features(s)
    rc, B, mu, sg = m.desc_info()
    assert math.isclose(rc, box / 2, rel_tol=1e-6)
    # the radial basis as defined: Gaussians at 0.5 .. rc
    h = rc / 64
    r = (np.arange(64) + 0.5) * h
    sp = (rc - 0.5) / 31
    gauss = np.exp(-(r[:, None] - (0.5 + sp * np.arange(32))[None, :]) ** 2 / (2 * sp * sp))
    np.testing.assert_allclose(B, gauss, rtol=1e-5, atol=1e-6)
    x = st["x"].reshape(N, P, 3)
    for j in range(P):
        Fo, Vo = orc.desc_features(x[:, j, :], [box] * 3, rc, B.astype(np.float64), mu, sg)
        Fj = F[j * N:(j + 1) * N].astype(np.float64)
        Vj = V[j * N:(j + 1) * N, :9].astype(np.float64)
        assert np.abs(Fj[:, :32] - Fo[:, :32]).max() <= 2e-5 * np.abs(Fo[:, :32]).max()
        assert np.abs(Fj[:, 32:] - Fo[:, 32:]).max() <= 1e-5 * np.abs(Fo[:, 32:]).max()
        assert np.abs(Vj - Vo).max() <= 2e-5 * np.abs(Vo).max()
        assert (V[j * N:(j + 1) * N, 9] == 1.0).all()


def test_learned_residual_gain_judge_and_fallback(lib):
    N, P, NSUM, CHEAP = 64, 8, 8, 2
    s, box, T, st = ueg(lib, N, P, NSUM, seed=5)
    pair = lib.fn("md_coulomb_3d_ewald_force_x")
    m = xmd_x.EwaldModel(lib, s, nsum_cheap=CHEAP, capacity=64, seed=9)
    try:
        for i in range(96):  # plain run, converged Ewald
            xmd_x.md_step(lib, s, 0.01, image=1, pair=pair, pbc=True)
            if i % 2 == 1:
                m.collect(s)
        assert m.status()["configurations"] == 48
        loss = m.train(800, 16, 2e-3)
        assert math.isfinite(loss)
        for _ in range(10):  # a configuration the network has not seen
            xmd_x.md_step(lib, s, 0.01, image=1, pair=pair, pbc=True)
        j = m.judge(s)
        # truncation alone is wrong by a visible amount; the network removes
        # most of the energy error and part of the force error
        assert j["energy_err_truncated"] > 1e-4, j
        print("judged:", j, "final loss", loss)
        assert j["energy_err"] < 0.6 * j["energy_err_truncated"], j
        assert j["force_err"] < j["force_err_truncated"], j

        # energies through the ABI: learned vs converged vs truncated
        pe = lib.fn("md_coulomb_3d_ewald_energy_x")

        def energy():
            lib.check(lib.md_pimd_calc_pair_energy_x(s.pimd, pe, s.stats))
            return s.take_energy()

        e_conv = energy()
        m.attach(s, judge_every=0)
        e_learn = energy()
        m.detach(s)
        lib.md_set_coulomb_n_sum_x(CHEAP)
        e_trunc = energy()
        lib.md_set_coulomb_n_sum_x(NSUM)
        assert abs(e_learn - e_conv) < 0.6 * abs(e_trunc - e_conv), (e_conv, e_learn, e_trunc)

        # attached with judging every 5th force call, generous tolerances
        m.attach(s, judge_every=5, force_tol=0.5, energy_tol=1e-2)
        for _ in range(10):
            xmd_x.md_step(lib, s, 0.01, image=1, pair=pair, pbc=True)
        st1 = m.status()
        assert st1["judged"] >= 3 and not st1["reverted"], st1

        # a tolerance the network cannot meet: dropped at the next judgement,
        # after which the forces are the converged ones
        m.attach(s, judge_every=1, force_tol=1e-12, energy_tol=1e-12)
        xmd_x.md_step(lib, s, 0.01, image=1, pair=pair, pbc=True)
        assert m.status()["reverted"]

        def forces():
            lib.check(lib.md_reset_force_x(s.sim))
            lib.check(lib.md_pimd_calc_pair_force_x(s.pimd, pair))
            return s.state()["f"]

        f_rev = forces()
        m.detach(s)
        f_plain = forces()
        np.testing.assert_array_equal(f_rev, f_plain)
    finally:
        m.free()
        s.free()
