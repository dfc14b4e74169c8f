"""Pins the oracle (oracle/xmd_oracle.c) to MD-Lab's own _nocl build.

Every fixture under tests/golden/ was produced by the reference library
(tests/golden/make_golden.sh).  The oracle restates the same loops with the
same expressions, so per-call results agree to a few ulp; the trajectory
comparisons allow for the amplification of those ulps over many steps.
"""
import numpy as np
import pytest

import fixtures
import orc
from helpers import assert_close

TIGHT = 1e-13


def _cfg(h):
    prm = orc.params(trap_w=1.0, gauss_g=h["g"], gauss_s=h["s"], coul_s=1.0,
                     coul_alpha=h["alpha"], coul_nsum=h["nsum"])
    trap = 0 if h["ueg"] else orc.TRAP_HARMONIC
    pair = orc.PAIR_EWALD if h["ueg"] else orc.PAIR_GAUSSIAN
    return prm, trap, pair


@pytest.mark.parametrize("name", fixtures.PIMD_FIXTURES)
def test_oracle_one_step_stages(name):
    fx = fixtures.load(name)
    h = fixtures.header(fx)
    N, P, D = h["N"], h["P"], h["D"]
    L = orc.lib()
    prm, trap, pair = _cfg(h)
    s = orc.OrcSim.from_fixture(fx)
    assert L.orc_nhc_vv3_1(s.ref, h["dt"]) == 0
    for k in ("x", "v", "theta", "vtheta"):
        assert_close(getattr(s, k), fx["s1/" + k], TIGHT, f"{name} VV3_1 {k}")
    L.orc_reset_force(s.ref)
    ENk, Eint = orc.fast_fill_ENk(s, N, P, h["omegaP"], h["image"])
    assert_close(ENk, fx["ENk"], TIGHT, "ENk")
    assert_close(Eint, fx["Eint"], TIGHT, "Eint")
    VBN = orc.fill_VB(N, h["beta"], h["vi"], ENk)
    assert_close(VBN, fx["VBN"], TIGHT, "VBN")
    orc.fast_force_VB(s, N, P, h["beta"], h["vi"], h["omegaP"], h["image"], ENk, VBN)
    assert_close(s.f, fx["f_exch/f"], TIGHT, "exchange force")
    if trap:
        L.orc_trap_force(s.ref, N, P, trap, orc.C.byref(prm))
        assert_close(s.f, fx["f_trap/f"], TIGHT, "trap force")
    L.orc_pair_force(s.ref, N, P, pair, orc.C.byref(prm))
    assert_close(s.f, fx["f_pair/f"], 1e-12, "pair force")
    # estimators at the step-1 positions
    e = L.orc_vbn_energy(D, N, P, h["beta"], h["vi"], orc.ptr(ENk), orc.ptr(VBN))
    assert_close([e], fx["s1/e_prim_exch"], TIGHT, "primitive estimator")
    ENk2 = np.zeros(orc.ntri(N))
    L.orc_fast_fill_ENk2(s.ref, N, P, h["omegaP"], h["image"], orc.ptr(ENk2))
    assert_close(ENk2, fx["s1/ENk2"], TIGHT, "ENk2")
    ev = L.orc_vi_virial_energy(s.ref, N, P, h["beta"], h["vi"], h["image"], orc.ptr(ENk),
                                orc.ptr(ENk2), orc.ptr(VBN))
    assert_close([ev], fx["s1/e_vir_exch"], 1e-12, "virial estimator")
    if trap:
        et = L.orc_trap_energy(s.ref, N, P, trap, orc.C.byref(prm))
        assert_close([et], fx["s1/e_trap"], TIGHT, "trap energy")
    ep = L.orc_pair_energy(s.ref, N, P, pair, orc.C.byref(prm))
    assert_close([ep], fx["s1/e_pair"], 1e-12, "pair energy")
    sg = L.orc_vi_sign(N, h["beta"], h["vi"], -1.0, orc.ptr(ENk), orc.ptr(VBN))
    assert_close([sg], fx["s1/sign_m1"], 1e-11, "xi=-1 reweighting")
    if D == 3:
        qs, qis = orc.sk_sphere(0.0, 0.5, 2.0)
        np.testing.assert_array_equal(qs, fx["sk/qs"])
        np.testing.assert_array_equal(qis.ravel(), fx["sk/qis"])
        res = orc.sk_structure(N, P, s.x, P // 2 + 1, qis)
        assert_close(res, fx["sk/res"], 1e-12, "spherical S(k)")
    assert L.orc_nhc_vv3_2(s.ref, h["dt"]) == 0
    for k in ("x", "v", "theta", "vtheta"):
        assert_close(getattr(s, k), fx["s2/" + k], TIGHT, f"VV3_2 {k}")
    if h["pbc"]:
        L.orc_periodic_boundary(s.ref)
        assert_close(s.x, fx["s3/x"], TIGHT, "wrapped positions")
    if h["ueg"]:
        box = np.array([h["box"]] * 3)
        mad = L.orc_madelung(orc.ptr(box), orc.C.byref(prm))
        assert_close([mad], fx["madelung"], TIGHT, "Madelung constant")


@pytest.mark.parametrize("name", fixtures.PIMD_FIXTURES)
def test_oracle_trajectory(name):
    """Whole steps through orc_step track the reference to the end of the run."""
    fx = fixtures.load(name)
    h = fixtures.header(fx)
    if h["steps"] < 2:
        pytest.skip("single-step fixture")
    N, P = h["N"], h["P"]
    prm, trap, pair = _cfg(h)
    cfg = orc.StepCfg(N, P, h["beta"], h["vi"], h["omegaP"], h["image"], trap, pair, h["pbc"], prm)
    s = orc.OrcSim.from_fixture(fx)
    ENk = np.zeros(orc.ntri(N))
    Eint = np.zeros(N)
    VBN = np.zeros(N + 1)
    L = orc.lib()
    for st in range(1, h["steps"] + 1):
        assert L.orc_step(s.ref, orc.C.byref(cfg), h["dt"], orc.ptr(ENk), orc.ptr(Eint),
                          orc.ptr(VBN)) == 0
        key = f"t{st}/e_prim_exch"
        if key in fx:
            e = L.orc_vbn_energy(h["D"], N, P, h["beta"], h["vi"], orc.ptr(ENk), orc.ptr(VBN))
            assert_close([e], fx[key], 1e-9, f"{name} step {st} primitive estimator")
    for k in ("x", "v", "theta", "vtheta"):
        assert_close(getattr(s, k), fx["final/" + k], 1e-9, f"{name} final {k}")


@pytest.mark.parametrize("name", fixtures.CUBIC_FIXTURES)
def test_oracle_cubic_paths(name):
    fx = fixtures.load(name)
    h = fixtures.header(fx, "cubic")
    N, P, D = h["N"], h["P"], h["D"]
    nb = N * P
    zeros = np.zeros(nb * D)
    s = orc.OrcSim(D, h["L"], nb, np.ones(nb), fx["init/x"], zeros, zeros, np.ones(nb * D),
                   np.zeros(nb * D * h["L"]), np.ones(nb * D * h["L"]), np.ones(nb * D * h["L"]),
                   1.0 / h["beta"], [h["box"]] * 3)
    L = orc.lib()
    ENk = np.zeros(orc.ntri(N))
    L.orc_fill_ENk_cubic(s.ref, N, P, h["omegaP"], h["image"], orc.ptr(ENk))
    assert_close(ENk, fx["ENk_cubic"], TIGHT, "cubic ENk")
    VBN = orc.fill_VB(N, h["beta"], h["vi"], ENk)
    assert_close(VBN, fx["VBN_cubic"], TIGHT, "VBN")
    L.orc_force_VB_cubic(s.ref, N, P, h["beta"], h["vi"], h["omegaP"], h["image"], orc.ptr(ENk),
                         orc.ptr(VBN))
    assert_close(s.f, fx["f_cubic/f"], TIGHT, "cubic exchange force")
    s.f[:] = 0
    ENk_f, _ = orc.fast_fill_ENk(s, N, P, h["omegaP"], h["image"])
    assert_close(ENk_f, fx["ENk_fast"], TIGHT, "fast ENk")
    VBN = orc.fill_VB(N, h["beta"], h["vi"], ENk_f)
    orc.fast_force_VB(s, N, P, h["beta"], h["vi"], h["omegaP"], h["image"], ENk_f, VBN)
    assert_close(s.f, fx["f_fast/f"], TIGHT, "fast exchange force")
    # the two reference algorithms agree with each other (internal check)
    assert_close(fx["f_fast/f"], fx["f_cubic/f"], 1e-11, "cubic vs quadratic")
    ENk2 = np.zeros(orc.ntri(N))
    L.orc_fill_ENk2_cubic(s.ref, N, P, h["omegaP"], h["image"], orc.ptr(ENk2))
    assert_close(ENk2, fx["ENk2_cubic"], TIGHT, "cubic ENk2")


def test_oracle_rng():
    fx = fixtures.load("rng")
    L = orc.lib()
    L.orc_set_seed(1234)
    u = [L.orc_random_uniform(-1.0, 2.0) for _ in range(32)]
    g = [L.orc_random_gaussian() for _ in range(32)]
    np.testing.assert_array_equal(u, fx["uniform"])
    np.testing.assert_array_equal(g, fx["gaussian"])


@pytest.mark.parametrize("fname,D", [("d3_pairs", 3), ("d2_pairs", 2)])
def test_oracle_pair_callbacks(fname, D):
    fx = fixtures.load(fname)
    L = orc.lib()
    box = fx["L"]
    pos = fx["pos"].reshape(-1, 2, D)
    prm = orc.params(gauss_g=0.75 * np.pi, gauss_s=0.5, coul_s=1.3)
    kinds = {"gauss": orc.PAIR_GAUSSIAN, "pgauss": orc.PAIR_PERIODIC_GAUSSIAN,
             "coul": orc.PAIR_COULOMB, "pcoul": orc.PAIR_PERIODIC_COULOMB}
    for a, al in enumerate((5.6, 3.0)):
        for n in (1, 2, 3):
            if D == 3:
                kinds[f"ewald_a{a}_n{n}"] = (orc.PAIR_EWALD, al / box[0], n)
    for nm, k in kinds.items():
        p = prm
        if isinstance(k, tuple):
            k, alpha, n = k
            p = orc.params(coul_s=1.3, coul_alpha=alpha, coul_nsum=n)
        f = np.zeros((len(pos), D))
        e = np.zeros(len(pos))
        for i, (p1, p2) in enumerate(pos):
            fi = np.zeros(D)
            L.orc_pair_force_one(k, orc.C.byref(p), D, orc.ptr(np.ascontiguousarray(p1)),
                                 orc.ptr(np.ascontiguousarray(p2)), orc.ptr(fi), orc.ptr(box), 1.7)
            f[i] = fi
            e[i] = L.orc_pair_energy_one(k, orc.C.byref(p), D, orc.ptr(np.ascontiguousarray(p1)),
                                         orc.ptr(np.ascontiguousarray(p2)), orc.ptr(box))
        assert_close(f.ravel(), fx[nm + "/f"], TIGHT, nm + " force")
        assert_close(e, fx[nm + "/e"], TIGHT, nm + " energy")
        if nm.startswith("ewald"):
            mad = L.orc_madelung(orc.ptr(box), orc.C.byref(p))
            assert_close([mad], fx[nm + "/mad"], TIGHT, nm + " Madelung")


@pytest.mark.parametrize("name", fixtures.TWO_FIXTURES)
def test_oracle_two_species(name):
    """Cross-species forces and energy (md_pimd_calc_pair_force_2_x,
    md_pimd_calc_pair_energy_2_x) and a two-species trajectory."""
    fx = fixtures.load(name)
    h = fixtures.header(fx, "two")
    Na, Nb, P = h["N"], h["Nb"], h["P"]
    prm, trap, pair = _cfg(h)
    a, b = orc.two_from_fixture(fx)
    a.f[:] = 0
    b.f[:] = 0
    orc.pair_force_2(a, Na, b, Nb, P, pair, prm)
    assert_close(a.f, fx["a/cross/f"], TIGHT, "cross force on a")
    assert_close(b.f, fx["b/cross/f"], TIGHT, "cross force on b")
    assert_close([orc.pair_energy_2(a, Na, b, Nb, P, pair, prm)], fx["cross/e"], TIGHT, "cross energy")
    orc.two_species_forces(a, b, Na, Nb, P, h["beta"], h["vi"], h["omegaP"], h["image"], trap, pair, prm)
    assert_close(a.f, fx["a/all/f"], TIGHT, "all forces on a")
    assert_close(b.f, fx["b/all/f"], TIGHT, "all forces on b")
    # the trajectory starts from these forces, as the reference's run did
    for _ in range(h["steps"]):
        orc.two_species_step(a, b, Na, Nb, P, h["beta"], h["vi"], h["omegaP"], h["image"], trap, pair, prm,
                             h["dt"], h["pbc"])
    for sp, s in (("a/", a), ("b/", b)):
        for k in ("x", "v", "theta", "vtheta"):
            assert_close(getattr(s, k), fx[sp + "final/" + k], 1e-9, f"{name} {sp} final {k}")
    assert_close([orc.pair_energy_2(a, Na, b, Nb, P, pair, prm)], fx["final/cross_e"], 1e-9, "final cross energy")


OBS_FIXTURES = ["d3l4_obs_ueg", "d2l4_obs_trap"]


@pytest.mark.parametrize("name", OBS_FIXTURES)
def test_oracle_observables(name):
    """plain and centroid virial estimators, g(r) with and without the
    minimum image, and the whole-polymer periodic wrap, on the state the
    reference recorded after a trajectory without the per-step wrap"""
    fx = fixtures.load(name)
    h = fixtures.header(fx)
    N, P, D = h["N"], h["P"], h["D"]
    L = orc.lib()
    nb = N * P
    s = orc.OrcSim(D, h["L"], nb, fx["m"], fx["obs/x"], np.zeros(nb * D), fx["obs/f"], np.ones(nb * D),
                   np.zeros(nb * D * h["L"]), np.zeros(nb * D * h["L"]), np.ones(nb * D * h["L"]), h["T"],
                   [h["box"]] * 3)
    assert_close([L.orc_virial_energy(s.ref, N, P)], fx["obs/e_virial"], TIGHT, "virial")
    for fc in (0, 3):
        assert_close([L.orc_centroid_virial_energy(s.ref, N, P, h["beta"], fc)], fx[f"obs/e_centroid_fc{fc}"],
                     TIGHT, f"centroid virial fc={fc}")
    pts, rmax, norm, pi = fx["gr/params"]
    for img, key in ((0, "gr/plain"), (1, "gr/image")):
        out = np.zeros(int(pts))
        out[3] = 0.25
        L.orc_pair_correlation(s.ref, N, P, int(pts), rmax, norm, int(pi), img, orc.ptr(out))
        assert np.array_equal(out, fx[key]), key  # counts of 1/norm: bit for bit
    L.orc_polymer_periodic_boundary(s.ref, N, P)
    assert np.array_equal(s.x, fx["pbc/x"])
