"""The workloads of the configurations at their stated shapes, against the
oracle (pinned to MD-Lab's _nocl build by tests/golden/):

  * the 3D trap, N = 64 fictitious particles, P = 64, beta = 4, Gaussian
    repulsion V = 3 exp(-r^2/0.25) (g = 0.75 pi, s = 0.5), NHC length 4,
    dt = 0.005, at xi = 1, 0.75, 0.5, 0.25, 0: every stage of the first step,
    then 1000 whole steps;
  * the electron gas, N = 128 spin-polarised, rs = 2, theta = 0.5, P = 32,
    Ewald alpha = 5.6/L with the reciprocal cube |n| <= 8, dt = 0.05, at
    xi = 0.2 ... 1: every stage of the first step, the Ewald forces on sampled
    beads (the oracle's per-pair cube of 9,825 terms makes the full sum too
    slow for a test).

Initial states come from the library's own initial-condition routines
(md_random_gaussian_x / md_pimd_init_particle_uniform_pos_x,
md_init_maxwell_vel_x, md_init_nhc_x with md_get_quick_Q_x), which reproduce
the reference's bit for bit.  Exchange quantities whose conditioning exceeds
the 1e-10 bar are held to the drift bar of test_gpu_exchange_large; whole
trajectories to max(1e-10, 30x the oracle's own drift from a one-ulp change
of the initial positions).
"""
import math

import numpy as np
import pytest

import orc
import xmd_x
from gpu_common import PARITY
from helpers import assert_close, relerr
from test_gpu_exchange_large import DRIFT_FACTOR

pytestmark = pytest.mark.gpu

D, L = 3, 4


def oracle_of(st, T, box):
    nb = len(st["m"])
    return orc.OrcSim(D, L, nb, st["m"], st["x"], st["v"], st["f"], st["cf"], st["theta"], st["vtheta"], st["Q"], T,
                      [box] * 3)


def first_step_stages(lib, s, o, N, P, beta, vi, dt, image, trap, pair_fn, prm):
    """the first step's stages up to the pair forces, GPU against the oracle
    (the oracle's pair forces are left to the caller); returns the oracle's
    ENk, V_B and the bar of the G-weighted forces"""
    ck, Lo = lib.check, orc.lib()
    omegaP = math.sqrt(P) / beta
    ck(lib.md_update_nhc_VV3_1_x(s.sim, dt))
    Lo.orc_nhc_vv3_1(o.ref, dt)
    st = s.state()
    for k in ("x", "v", "theta", "vtheta"):
        assert_close(st[k], getattr(o, k), PARITY, f"VV3_1 {k}")
    # the exchange at these positions, with the oracle's one-ulp drift as
    # the conditioning bar of G-weighted quantities
    ck(lib.md_reset_force_x(s.sim))
    ck(lib.md_pimd_fast_fill_ENk_x(s.pimd, image))
    ck(lib.md_pimd_fill_VB_x(s.pimd))
    ck(lib.md_pimd_fast_fill_force_VB_x(s.pimd, image))
    o.f[:] = 0
    ENk, _ = orc.fast_fill_ENk(o, N, P, omegaP, image)
    VBN = orc.fill_VB(N, beta, vi, ENk)
    orc.fast_force_VB(o, N, P, beta, vi, omegaP, image, ENk, VBN)
    xp = o.x * (1 + np.random.default_rng(1).choice([-1.0, 1.0], o.x.shape) * 2.0 ** -52)
    o2 = oracle_of({"m": o.m, "x": xp, "v": o.v, "f": np.zeros_like(o.f), "cf": o.cf, "theta": o.theta,
                    "vtheta": o.vtheta, "Q": o.Q}, o.s.T, o.s.box[0])
    E2, _ = orc.fast_fill_ENk(o2, N, P, omegaP, image)
    orc.fast_force_VB(o2, N, P, beta, vi, omegaP, image, E2, orc.fill_VB(N, beta, vi, E2))
    ftol = max(PARITY, DRIFT_FACTOR * relerr(o2.f, o.f))
    ex = s.exchange()
    assert_close(ex["ENk"], ENk, PARITY, "ENk")
    assert_close(ex["VBN"], VBN, PARITY, "V_B")
    assert_close(s.state()["f"], o.f, ftol, "exchange spring force")
    if trap:
        ck(lib.md_pimd_calc_trap_force_x(s.pimd, lib.fn("md_harmonic_trap_force_x")))
        Lo.orc_trap_force(o.ref, N, P, orc.TRAP_HARMONIC, orc.C.byref(prm))
        assert_close(s.state()["f"], o.f, ftol, "exchange + trap force")
    ck(lib.md_pimd_calc_pair_force_x(s.pimd, lib.fn(pair_fn)))
    return ENk, VBN, ftol


def estimators(lib, s, o, N, P, beta, vi, image, ENk, VBN):
    """primitive and virial estimators (the latter reads o.f, which must hold
    the same forces as the GPU's)"""
    ck, Lo = lib.check, orc.lib()
    omegaP = math.sqrt(P) / beta
    e = Lo.orc_vbn_energy(D, N, P, beta, vi, orc.ptr(ENk), orc.ptr(VBN))
    ck(lib.md_pimd_calc_VBN_energy_x(s.pimd, s.stats))
    assert_close([s.take_energy()], [e], PARITY, "primitive estimator")
    ENk2 = np.zeros(orc.ntri(N))
    Lo.orc_fast_fill_ENk2(o.ref, N, P, omegaP, image, orc.ptr(ENk2))
    ck(lib.md_pimd_fast_fill_ENk2_x(s.pimd, image))
    assert_close(s.exchange()["ENk2"], ENk2, PARITY, "ENk2")
    ev = Lo.orc_vi_virial_energy(o.ref, N, P, beta, vi, image, orc.ptr(ENk), orc.ptr(ENk2), orc.ptr(VBN))
    ck(lib.md_pimd_calc_vi_virial_energy_x(s.pimd, s.stats, image))
    assert_close([s.take_energy()], [ev], PARITY, "virial estimator")


# ---------------------------------------------------------------------
# 3D trap, N = 64, P = 64
# ---------------------------------------------------------------------
TRAP = dict(N=64, P=64, beta=4.0, g=0.75 * math.pi, s=0.5, dt=0.005, steps=1000)


def trap_system(lib, vi, seed):
    c = TRAP
    N, P, T = c["N"], c["P"], 1.0 / c["beta"]
    s = xmd_x.PimdSystem(lib, N, P, vi, T, box=10.0)
    lib.md_set_seed_x(seed)
    x = np.array([lib.md_random_gaussian_x() for _ in range(N * P * D)])
    s.set_state(x=x, f=np.zeros(N * P * D))
    lib.md_init_particle_mass_x(s.sim, 1.0, 0, N * P)
    lib.md_init_maxwell_vel_x(s.sim, T)
    lib.md_init_nhc_x(s.sim, lib.md_get_quick_Q_x(T, s.pimd.contents.omegaP), 0, s.sim.contents.Nf, 0.0)
    xmd_x.set_potentials(lib, trap_w=1.0, gauss_g=c["g"], gauss_s=c["s"])
    return s, T


@pytest.mark.parametrize("vi", [1.0, 0.75, 0.5, 0.25, 0.0])
def test_trap_n64_p64_stages_and_1000_steps(vi):
    c = TRAP
    N, P, beta, dt = c["N"], c["P"], c["beta"], c["dt"]
    lib = xmd_x.load(D, L)
    s, T = trap_system(lib, vi, seed=2024 + int(100 * vi))
    try:
        init = s.state()
        o = oracle_of(init, T, 10.0)
        prm = orc.params(trap_w=1.0, gauss_g=c["g"], gauss_s=c["s"])
        ENk, VBN, ftol = first_step_stages(lib, s, o, N, P, beta, vi, dt, 0, True, "md_gaussian_force_x", prm)
        orc.lib().orc_pair_force(o.ref, N, P, orc.PAIR_GAUSSIAN, orc.C.byref(prm))
        assert_close(s.state()["f"], o.f, ftol, "total force")
        estimators(lib, s, o, N, P, beta, vi, 0, ENk, VBN)
        lib.check(lib.md_update_nhc_VV3_2_x(s.sim, dt))
        orc.lib().orc_nhc_vv3_2(o.ref, dt)
        st = s.state()
        for k in ("x", "v", "theta", "vtheta"):
            assert_close(st[k], getattr(o, k), max(PARITY, ftol), f"VV3_2 {k}")
        # 999 more whole steps on both, and the oracle's own drift from a
        # one-ulp change of the initial positions
        cfg = orc.StepCfg(N, P, beta, vi, math.sqrt(P) / beta, 0, orc.TRAP_HARMONIC, orc.PAIR_GAUSSIAN, 0, prm)
        trap, pair = lib.fn("md_harmonic_trap_force_x"), lib.fn("md_gaussian_force_x")
        for _ in range(c["steps"] - 1):
            xmd_x.md_step(lib, s, dt, trap=trap, pair=pair)
        wE, wEi, wV = np.zeros(orc.ntri(N)), np.zeros(N), np.zeros(N + 1)
        for _ in range(c["steps"] - 1):
            assert orc.lib().orc_step(o.ref, orc.C.byref(cfg), dt, orc.ptr(wE), orc.ptr(wEi), orc.ptr(wV)) == 0
        p = oracle_of(dict(init, x=np.nextafter(init["x"], np.inf)), T, 10.0)
        for _ in range(c["steps"]):
            assert orc.lib().orc_step(p.ref, orc.C.byref(cfg), dt, orc.ptr(wE), orc.ptr(wEi), orc.ptr(wV)) == 0
        fin = s.state()
        got = max(relerr(fin[k], getattr(o, k)) for k in ("x", "v", "theta", "vtheta"))
        own = max(relerr(getattr(p, k), getattr(o, k)) for k in ("x", "v", "theta", "vtheta"))
        print(f"trap N=64 P=64 xi={vi}: 1000 steps, GPU vs oracle {got:.2e}, oracle vs itself (1-ulp start) "
              f"{own:.2e}")
        assert got <= max(PARITY, 30 * own)
    finally:
        s.free()


# ---------------------------------------------------------------------
# electron gas, N = 128, P = 32, |n| <= 8
# ---------------------------------------------------------------------
def ueg_system(lib, vi, seed):
    N, P, rs, theta = 128, 32, 2.0, 0.5
    box = (4 * math.pi * N / 3) ** (1 / 3) * rs
    T = theta * 0.5 * (6 * math.pi ** 2 * N / box ** 3) ** (2 / 3)
    s = xmd_x.PimdSystem(lib, N, P, vi, T, box=box)
    lib.md_set_seed_x(seed)
    lib.md_init_particle_mass_x(s.sim, 1.0, 0, N * P)
    c = (xmd_x.C.c_double * 3)(box / 2, box / 2, box / 2)
    Lv = (xmd_x.C.c_double * 3)(box, box, box)
    lib.md_pimd_init_particle_uniform_pos_x(s.pimd, c, Lv, 0.05 * rs)
    lib.md_init_maxwell_vel_x(s.sim, T)
    lib.md_init_nhc_x(s.sim, lib.md_get_quick_Q_x(T, s.pimd.contents.omegaP), 0, s.sim.contents.Nf, 0.0)
    s.set_state(f=np.zeros(N * P * D))
    xmd_x.set_potentials(lib, coul_s=1.0, alpha=5.6 / box, nsum=8)
    return s, box, T


@pytest.mark.parametrize("vi", [0.2, 0.4, 0.6, 0.8, 1.0])
def test_ueg_n128_p32_nsum8_stages(vi):
    N, P, dt = 128, 32, 0.05
    lib = xmd_x.load(D, L)
    s, box, T = ueg_system(lib, vi, seed=77 + int(10 * vi))
    beta = 1.0 / T
    try:
        init = s.state()
        o = oracle_of(init, T, box)
        prm = orc.params(coul_s=1.0, coul_alpha=5.6 / box, coul_nsum=8)
        ENk, VBN, ftol = first_step_stages(lib, s, o, N, P, beta, vi, dt, 1, False, "md_coulomb_3d_ewald_force_x",
                                           prm)
        # Ewald forces on sampled beads: the oracle's per-pair formula over
        # the slice, with the reference's 1/P and higher-index mass rule
        f = s.state()["f"].reshape(N, P, D)
        fex = o.f.reshape(N, P, D)
        x = o.x.reshape(N, P, D)
        Lb = np.full(3, box)
        for (a, j) in [(0, 0), (127, 31), (64, 15), (5, 20)]:
            ref = fex[a, j].copy()
            for b in range(N):
                if b == a:
                    continue
                fb = np.zeros(3)
                p1, p2 = (x[a, j], x[b, j]) if a > b else (x[b, j], x[a, j])
                orc.lib().orc_pair_force_one(orc.PAIR_EWALD, orc.C.byref(prm), 3, orc.ptr(np.ascontiguousarray(p1)),
                                             orc.ptr(np.ascontiguousarray(p2)), orc.ptr(fb), orc.ptr(Lb), 1.0)
                ref += fb / P if a > b else -fb / P
            assert_close(f[a, j], ref, max(PARITY, ftol), f"Ewald + exchange force on bead ({a},{j})")
        # the rest of the step (the virial estimator reads the forces) with the
        # GPU's forces on both sides
        o.f[:] = s.state()["f"]
        estimators(lib, s, o, N, P, beta, vi, 1, ENk, VBN)
        lib.check(lib.md_update_nhc_VV3_2_x(s.sim, dt))
        orc.lib().orc_nhc_vv3_2(o.ref, dt)
        lib.check(lib.md_periodic_boundary_x(s.sim))
        orc.lib().orc_periodic_boundary(o.ref)
        st = s.state()
        for k in ("x", "v", "theta", "vtheta"):
            assert_close(st[k], getattr(o, k), PARITY, f"VV3_2 + wrap {k}")
    finally:
        s.free()
