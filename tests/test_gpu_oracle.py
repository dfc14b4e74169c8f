"""CUDA library vs the oracle on seeded states larger than the golden
fixtures (ragged tiles, N beyond one block, Ewald with many images), and
size-independent properties at the benchmark's full size."""
import numpy as np
import pytest

import orc
import xmd_x
from gpu_common import PARITY, make_pair, random_state
from helpers import assert_close

pytestmark = pytest.mark.gpu


def _ueg_box(N, rs):
    return (4 * np.pi * N / 3) ** (1 / 3) * rs


CASES = [
    # D, L, N, P, vi, beta, ueg, nsum, image
    (3, 4, 100, 6, 0.7, 2.0, False, 0, 0),
    (3, 4, 33, 3, 1.0, 4.0, False, 0, 0),
    (3, 4, 65, 2, 0.0, 1.0, False, 0, 0),
    (2, 4, 70, 5, 0.3, 3.0, False, 0, 0),
    (3, 8, 40, 4, 0.9, 2.0, False, 0, 0),
    (3, 4, 40, 4, 0.6, 1.0, True, 4, 1),
    (3, 4, 27, 3, 1.0, 0.5, True, 2, 1),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"d{c[0]}l{c[1]}_N{c[2]}_P{c[3]}_vi{c[4]}_{'ueg' if c[6] else 'trap'}")
def test_forces_and_estimators_vs_oracle(case):
    D, L, N, P, vi, beta, ueg, nsum, image = case
    lib = xmd_x.load(D, L)
    T = 1.0 / beta
    box = _ueg_box(N, 1.5) if ueg else 10.0
    st = random_state(D, L, N, P, T, box, ueg, seed=N * 31 + P)
    s, o = make_pair(lib, st, N, P, vi, T, box)
    alpha = 5.6 / box
    xmd_x.set_potentials(lib, trap_w=1.0, gauss_g=0.75 * np.pi, gauss_s=0.5, coul_s=1.0,
                         alpha=alpha, nsum=max(nsum, 1))
    prm = orc.params(trap_w=1.0, gauss_g=0.75 * np.pi, gauss_s=0.5, coul_s=1.0, coul_alpha=alpha,
                     coul_nsum=max(nsum, 1))
    omegaP = np.sqrt(P) / beta
    ck = lib.check
    # exchange
    ck(lib.md_reset_force_x(s.sim))
    ck(lib.md_pimd_fast_fill_ENk_x(s.pimd, image))
    ck(lib.md_pimd_fill_VB_x(s.pimd))
    ck(lib.md_pimd_fast_fill_force_VB_x(s.pimd, image))
    o.f[:] = 0
    ENk, Eint = orc.fast_fill_ENk(o, N, P, omegaP, image)
    VBN = orc.fill_VB(N, beta, vi, ENk)
    orc.fast_force_VB(o, N, P, beta, vi, omegaP, image, ENk, VBN)
    ex = s.exchange()
    assert_close(ex["ENk"], ENk, PARITY, "ENk")
    assert_close(ex["VBN"], VBN, PARITY, "VBN")
    assert_close(s.state()["f"], o.f, PARITY, "exchange force")
    # external forces
    L_ = orc.lib()
    if ueg:
        ck(lib.md_pimd_calc_pair_force_x(s.pimd, lib.fn("md_coulomb_3d_ewald_force_x")))
        L_.orc_pair_force(o.ref, N, P, orc.PAIR_EWALD, orc.C.byref(prm))
    else:
        ck(lib.md_pimd_calc_trap_force_x(s.pimd, lib.fn("md_harmonic_trap_force_x")))
        ck(lib.md_pimd_calc_pair_force_x(s.pimd, lib.fn("md_gaussian_force_x")))
        L_.orc_trap_force(o.ref, N, P, orc.TRAP_HARMONIC, orc.C.byref(prm))
        L_.orc_pair_force(o.ref, N, P, orc.PAIR_GAUSSIAN, orc.C.byref(prm))
    assert_close(s.state()["f"], o.f, PARITY, "total force")
    # estimators
    ck(lib.md_pimd_calc_VBN_energy_x(s.pimd, s.stats))
    e = L_.orc_vbn_energy(D, N, P, beta, vi, orc.ptr(ENk), orc.ptr(VBN))
    assert_close([s.take_energy()], [e], PARITY, "primitive estimator (cycle probabilities)")
    ck(lib.md_pimd_fast_fill_ENk2_x(s.pimd, image))
    ENk2 = np.zeros(orc.ntri(N))
    L_.orc_fast_fill_ENk2(o.ref, N, P, omegaP, image, orc.ptr(ENk2))
    assert_close(s.exchange()["ENk2"], ENk2, PARITY, "ENk2")
    ck(lib.md_pimd_calc_vi_virial_energy_x(s.pimd, s.stats, image))
    ev = L_.orc_vi_virial_energy(o.ref, N, P, beta, vi, image, orc.ptr(ENk), orc.ptr(ENk2), orc.ptr(VBN))
    assert_close([s.take_energy()], [ev], PARITY, "virial estimator (cycle probabilities)")
    # a fresh V_B recursion leaves no cycle probabilities of a force call:
    # both estimators then solve the recursion themselves
    ck(lib.md_pimd_fill_VB_x(s.pimd))
    ck(lib.md_pimd_calc_VBN_energy_x(s.pimd, s.stats))
    assert_close([s.take_energy()], [e], PARITY, "primitive estimator (recursion)")
    ck(lib.md_pimd_calc_vi_virial_energy_x(s.pimd, s.stats, image))
    assert_close([s.take_energy()], [ev], PARITY, "virial estimator (recursion)")
    kind = orc.PAIR_EWALD if ueg else orc.PAIR_GAUSSIAN
    pe = lib.fn("md_coulomb_3d_ewald_energy_x" if ueg else "md_gaussian_energy_x")
    ck(lib.md_pimd_calc_pair_energy_x(s.pimd, pe, s.stats))
    ep = L_.orc_pair_energy(o.ref, N, P, kind, orc.C.byref(prm))
    assert_close([s.take_energy()], [ep], PARITY, "pair energy")
    # integrator
    ck(lib.md_update_nhc_VV3_1_x(s.sim, 0.01))
    ck(lib.md_update_nhc_VV3_2_x(s.sim, 0.01))
    L_.orc_nhc_vv3_1(o.ref, 0.01)
    L_.orc_nhc_vv3_2(o.ref, 0.01)
    stt = s.state()
    for k in ("x", "v", "theta", "vtheta"):
        assert_close(stt[k], getattr(o, k), PARITY, f"NHC {k}")
    s.free()


def test_grouped_chains_vs_oracle():
    """Chains over several DOFs with constraints (f=4, fc=5)."""
    D, L, N, P = 3, 4, 9, 5
    lib = xmd_x.load(D, L)
    st = random_state(D, L, N, P, 0.5, 10.0, False, seed=5, f=4, fc=5)
    st["f"] = np.random.default_rng(6).standard_normal(N * P * D)
    s, o = make_pair(lib, st, N, P, 1.0, 0.5, 10.0, f=4, fc=5)
    for _ in range(3):
        lib.check(lib.md_update_nhc_VV3_1_x(s.sim, 0.02))
        lib.check(lib.md_update_nhc_VV3_2_x(s.sim, 0.02))
        orc.lib().orc_nhc_vv3_1(o.ref, 0.02)
        orc.lib().orc_nhc_vv3_2(o.ref, 0.02)
    stt = s.state()
    for k in ("x", "v", "theta", "vtheta"):
        assert_close(stt[k], getattr(o, k), PARITY, f"grouped NHC {k}")
    s.free()


# ---------------------------------------------------------------------
# full benchmark size: N=512, P=64 electron gas (rs=1), Ewald |n|<=10
# ---------------------------------------------------------------------
@pytest.fixture(scope="module")
def big_ueg():
    D, L, N, P = 3, 4, 512, 64
    lib = xmd_x.load(D, L)
    box = _ueg_box(N, 1.0)
    T = 0.5 * 0.5 * (6 * np.pi ** 2 * N / box ** 3) ** (2 / 3)
    st = random_state(D, L, N, P, T, box, True, seed=2025)
    s = xmd_x.PimdSystem(lib, N, P, 0.5, T, box=box)
    s.set_state(**st)
    xmd_x.set_potentials(lib, coul_s=1.0, alpha=5.6 / box, nsum=10)
    yield lib, s, st, box, T
    s.free()


def test_full_size_ewald_sampled_vs_reference_formula(big_ueg):
    """The force on sampled beads at full size equals the reference's
    per-pair Ewald formula (orc_pair_force_one, cube |n|<=10) summed over
    the slice with the reference's 1/P and mass convention."""
    lib, s, st, box, T = big_ueg
    N, P, D = 512, 64, 3
    lib.check(lib.md_reset_force_x(s.sim))
    lib.check(lib.md_pimd_calc_pair_force_x(s.pimd, lib.fn("md_coulomb_3d_ewald_force_x")))
    f = s.state()["f"].reshape(N, P, D)
    x = st["x"].reshape(N, P, D)
    prm = orc.params(coul_s=1.0, coul_alpha=5.6 / box, coul_nsum=10)
    Lb = np.full(3, box)
    for (a, j) in [(0, 0), (511, 63), (200, 17)]:
        ref = np.zeros(3)
        for b in range(N):
            if b == a:
                continue
            fb = np.zeros(3)
            p1, p2 = (x[a, j], x[b, j]) if a > b else (x[b, j], x[a, j])
            orc.lib().orc_pair_force_one(orc.PAIR_EWALD, orc.C.byref(prm), 3,
                                         orc.ptr(np.ascontiguousarray(p1)), orc.ptr(np.ascontiguousarray(p2)),
                                         orc.ptr(fb), orc.ptr(Lb), 1.0)
            ref += fb / P if a > b else -fb / P
        assert_close(f[a, j], ref, 1e-10, f"Ewald force on bead ({a},{j})")


def test_full_size_properties(big_ueg):
    lib, s, st, box, T = big_ueg
    N, P, D = 512, 64, 3
    ck = lib.check
    # Newton's third law per slice (equal masses): the pair forces sum to zero
    ck(lib.md_reset_force_x(s.sim))
    ck(lib.md_pimd_calc_pair_force_x(s.pimd, lib.fn("md_coulomb_3d_ewald_force_x")))
    f = s.state()["f"].reshape(N, P, D)
    scale = np.abs(f).max()
    assert np.abs(f.sum(axis=0)).max() <= 1e-11 * scale * N
    # translation invariance: the exchange spring forces sum to zero (no image)
    ck(lib.md_reset_force_x(s.sim))
    ck(lib.md_pimd_fast_fill_ENk_x(s.pimd, 0))
    ck(lib.md_pimd_fill_VB_x(s.pimd))
    ck(lib.md_pimd_fast_fill_force_VB_x(s.pimd, 0))
    f = s.state()["f"].reshape(N * P, D)
    assert np.abs(f.sum(axis=0)).max() <= 1e-11 * np.abs(f).max() * N * P
    # energy / force consistency of the pair term: dE/dx = -m f
    pe = lib.fn("md_coulomb_3d_ewald_energy_x")
    ck(lib.md_reset_force_x(s.sim))
    ck(lib.md_pimd_calc_pair_force_x(s.pimd, lib.fn("md_coulomb_3d_ewald_force_x")))
    f = s.state()["f"].reshape(N, P, D)
    h = 1e-5
    for (a, j, d) in [(3, 5, 0), (400, 60, 2)]:
        es = []
        for sgn in (1, -1):
            x = st["x"].copy().reshape(N, P, D)
            x[a, j, d] += sgn * h
            s.set_state(x=x.ravel())
            ck(lib.md_pimd_calc_pair_energy_x(s.pimd, pe, s.stats))
            es.append(s.take_energy())
        s.set_state(x=st["x"])
        deriv = (es[0] - es[1]) / (2 * h)
        assert abs(deriv + f[a, j, d]) <= 1e-5 * max(1.0, abs(f[a, j, d])), (deriv, f[a, j, d])


def test_full_size_far_images_fp32_vs_strict_fp64(big_ueg):
    """The default FP64 form evaluates the real-space Ewald images at
    alpha R >= 4 and the wave-vector columns whose force weight is below
    1e-7 of the largest on the FP32 pipe; against
    MD_GB_PRECISION_FP64_STRICT (every term in FP64) every bead's pair force
    agrees within 1e-10 of its own size, and the whole array within 1e-12
    of its largest component."""
    lib, s, st, box, T = big_ueg
    N, P, D = 512, 64, 3
    out = {}
    try:
        for mode in (2, 0):
            lib.check(lib.md_gb300_set_precision_x(mode))
            lib.check(lib.md_reset_force_x(s.sim))
            lib.check(lib.md_pimd_calc_pair_force_x(s.pimd, lib.fn("md_coulomb_3d_ewald_force_x")))
            out[mode] = s.state()["f"].reshape(N, P, D).copy()
    finally:
        lib.check(lib.md_gb300_set_precision_x(0))
    d = np.abs(out[0] - out[2])
    scale = np.abs(out[2]).max()
    per_bead = d.max(axis=2) / np.maximum(np.abs(out[2]).max(axis=2), 1e-300)
    print("largest difference / largest force", d.max() / scale, "largest per-bead relative", per_bead.max())
    assert d.max() <= 1e-12 * scale
    assert per_bead.max() <= 1e-10
    assert d.max() > 0  # the FP32 path ran
