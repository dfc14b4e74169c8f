"""Parity of the CUDA library with MD-Lab's _nocl build.

Every fixture in tests/golden/ was produced by the reference library itself;
this test drives libxmd_x through the same C entry points in the same order
and compares every stage at 1e-10 relative (the FP64 parity bar), then
follows the trajectory to the end of the recorded run.
"""
import numpy as np
import pytest

import fixtures
import xmd_x
from gpu_common import PARITY
from helpers import assert_close, relerr

pytestmark = pytest.mark.gpu


def _setup(name):
    fx = fixtures.load(name)
    h = fixtures.header(fx)
    lib = xmd_x.load(h["D"], h["L"])
    s = xmd_x.PimdSystem(lib, h["N"], h["P"], h["vi"], h["T"], box=h["box"], f=h["f"], fc=h["fc"])
    xmd_x.set_potentials(lib, trap_w=1.0, gauss_g=h["g"], gauss_s=h["s"], coul_s=1.0,
                         alpha=h["alpha"], nsum=h["nsum"])
    s.set_state(m=fx["m"], x=fx["init/x"], v=fx["init/v"], f=fx["init/f"], theta=fx["init/theta"],
                vtheta=fx["init/vtheta"], Q=fx["init/Q"], cf=fx["init/cf"])
    trap = None if h["ueg"] else lib.fn("md_harmonic_trap_force_x")
    pair = lib.fn("md_coulomb_3d_ewald_force_x" if h["ueg"] else "md_gaussian_force_x")
    return fx, h, lib, s, trap, pair


@pytest.mark.parametrize("name", fixtures.PIMD_FIXTURES)
def test_step_stages_match_reference(name):
    fx, h, lib, s, trap, pair = _setup(name)
    ck, img = lib.check, h["image"]
    ck(lib.md_update_nhc_VV3_1_x(s.sim, h["dt"]), "VV3_1")
    st = s.state()
    for k in ("x", "v", "theta", "vtheta"):
        assert_close(st[k], fx["s1/" + k], PARITY, f"VV3_1 {k}")
    ck(lib.md_reset_force_x(s.sim))
    ck(lib.md_pimd_fast_fill_ENk_x(s.pimd, img))
    ex = s.exchange()
    assert_close(ex["ENk"], fx["ENk"], PARITY, "ENk")
    assert_close(ex["Eint"], fx["Eint"], PARITY, "Eint")
    ck(lib.md_pimd_fill_VB_x(s.pimd))
    assert_close(s.exchange()["VBN"], fx["VBN"], PARITY, "VBN")
    ck(lib.md_pimd_fast_fill_force_VB_x(s.pimd, img))
    assert_close(s.state()["f"], fx["f_exch/f"], PARITY, "exchange spring force")
    if trap:
        ck(lib.md_pimd_calc_trap_force_x(s.pimd, trap))
        assert_close(s.state()["f"], fx["f_trap/f"], PARITY, "trap force")
    ck(lib.md_pimd_calc_pair_force_x(s.pimd, pair))
    assert_close(s.state()["f"], fx["f_pair/f"], PARITY, "pair force")
    # estimators at these positions
    ck(lib.md_pimd_calc_VBN_energy_x(s.pimd, s.stats))
    assert_close([s.take_energy()], fx["s1/e_prim_exch"], PARITY, "primitive estimator")
    ck(lib.md_pimd_fast_fill_ENk2_x(s.pimd, img))
    assert_close(s.exchange()["ENk2"], fx["s1/ENk2"], PARITY, "ENk2")
    ck(lib.md_pimd_calc_vi_virial_energy_x(s.pimd, s.stats, img))
    assert_close([s.take_energy()], fx["s1/e_vir_exch"], PARITY, "virial estimator")
    if trap:
        ck(lib.md_pimd_calc_trap_energy_x(s.pimd, lib.fn("md_harmonic_trap_energy_x"), s.stats))
        assert_close([s.take_energy()], fx["s1/e_trap"], PARITY, "trap energy")
    pe = lib.fn("md_coulomb_3d_ewald_energy_x" if h["ueg"] else "md_gaussian_energy_x")
    ck(lib.md_pimd_calc_pair_energy_x(s.pimd, pe, s.stats))
    assert_close([s.take_energy()], fx["s1/e_pair"], PARITY, "pair energy")
    es, ss = lib.md_alloc_stats_x(1), lib.md_alloc_stats_x(1)
    es.contents.es[0] = 1.0
    ss.contents.es[0] = 1.0
    ck(lib.md_pimd_calc_vi_sign_x(s.pimd, es, ss, -1.0))
    assert_close([es.contents.es[0]], fx["s1/sign_m1"], 1e-9, "xi=-1 reweighting")
    if lib.D == 3:
        sk = lib.md_alloc_sk_sphere_3d_x(0.0, 0.5, 2.0)
        n = sk.contents.N
        st = lib.md_alloc_stats_x(n)
        ck(lib.md_pimd_calc_sphere_Sk_structure_x(s.pimd, st, h["P"] // 2 + 1, sk))
        got = np.array([st.contents.fxs[0][j] for j in range(n)])
        assert_close(got, fx["sk/res"], PARITY, "spherical S(k)")
    ck(lib.md_update_nhc_VV3_2_x(s.sim, h["dt"]))
    st = s.state()
    for k in ("x", "v", "theta", "vtheta"):
        assert_close(st[k], fx["s2/" + k], PARITY, f"VV3_2 {k}")
    if h["pbc"]:
        ck(lib.md_periodic_boundary_x(s.sim))
        assert_close(s.state()["x"], fx["s3/x"], PARITY, "wrapped positions")
    s.free()


def _intrinsic_divergence(fx, h):
    """How far the reference algorithm itself drifts from its own recorded
    trajectory when every initial coordinate is moved by one ulp: the
    Lyapunov-limited horizon of the run, measured with the oracle."""
    import orc
    prm = orc.params(trap_w=1.0, gauss_g=h["g"], gauss_s=h["s"], coul_s=1.0, coul_alpha=h["alpha"],
                     coul_nsum=h["nsum"])
    trap = 0 if h["ueg"] else orc.TRAP_HARMONIC
    pair = orc.PAIR_EWALD if h["ueg"] else orc.PAIR_GAUSSIAN
    N, P = h["N"], h["P"]
    cfg = orc.StepCfg(N, P, h["beta"], h["vi"], h["omegaP"], h["image"], trap, pair, h["pbc"], prm)
    o = orc.OrcSim.from_fixture(fx)
    o.x[:] = np.nextafter(o.x, np.inf)
    ENk, Eint, VBN = np.zeros(orc.ntri(N)), np.zeros(N), np.zeros(N + 1)
    est = 0.0
    for st in range(1, h["steps"] + 1):
        assert orc.lib().orc_step(o.ref, orc.C.byref(cfg), h["dt"], orc.ptr(ENk), orc.ptr(Eint),
                                  orc.ptr(VBN)) == 0
        key = f"t{st}/e_prim_exch"
        if key in fx:
            e = orc.lib().orc_vbn_energy(h["D"], N, P, h["beta"], h["vi"], orc.ptr(ENk), orc.ptr(VBN))
            est = max(est, relerr([e], fx[key]))
    fin = max(relerr(getattr(o, k), fx["final/" + k]) for k in ("x", "v", "theta", "vtheta"))
    return est, fin


@pytest.mark.parametrize("name", [n for n in fixtures.PIMD_FIXTURES])
def test_trajectory_tracks_reference(name):
    """Whole steps, device-resident between samples, against the reference's
    recorded estimators and final state.  Over short runs the bar is the
    1e-10 parity bar; over long runs chaotic dynamics amplify any rounding
    difference (the GPU's exp/log differ from glibc's by an ulp), so the bar
    is 1e-10 or 30x the drift the reference shows against itself after a
    one-ulp change of the initial positions, whichever is larger."""
    fx, h, lib, s, trap, pair = _setup(name)
    if h["steps"] < 2:
        pytest.skip("single-step fixture")
    worst = 0.0
    for st in range(1, h["steps"] + 1):
        xmd_x.md_step(lib, s, h["dt"], image=h["image"], trap=trap, pair=pair, pbc=bool(h["pbc"]))
        key = f"t{st}/e_prim_exch"
        if key in fx:
            lib.check(lib.md_pimd_calc_VBN_energy_x(s.pimd, s.stats))
            e = s.take_energy()
            worst = max(worst, relerr([e], fx[key]))
    fin = s.state()
    final = max(relerr(fin[k], fx["final/" + k]) for k in ("x", "v", "theta", "vtheta"))
    own_est, own_fin = _intrinsic_divergence(fx, h)
    print(f"{name}: {h['steps']} steps, GPU vs reference: estimator {worst:.2e}, state {final:.2e}; "
          f"reference vs itself (1-ulp start): estimator {own_est:.2e}, state {own_fin:.2e}")
    assert worst <= max(PARITY, 30 * own_est), f"{name}: estimator drift {worst:.2e} (own {own_est:.2e})"
    assert final <= max(PARITY, 30 * own_fin), f"{name}: state drift {final:.2e} (own {own_fin:.2e})"
    s.free()


@pytest.mark.parametrize("name", fixtures.CUBIC_FIXTURES)
def test_cubic_entry_points(name):
    """md_pimd_fill_ENk_x / md_pimd_fill_force_VB_x reproduce the reference's
    cubic-scaling outputs."""
    fx = fixtures.load(name)
    h = fixtures.header(fx, "cubic")
    lib = xmd_x.load(h["D"], h["L"])
    s = xmd_x.PimdSystem(lib, h["N"], h["P"], h["vi"], 1.0 / h["beta"], box=h["box"])
    nb = h["N"] * h["P"]
    s.set_state(m=np.ones(nb), x=fx["init/x"], v=np.zeros(nb * h["D"]), f=np.zeros(nb * h["D"]))
    ck = lib.check
    ck(lib.md_pimd_fill_ENk_x(s.pimd, h["image"]))
    assert_close(s.exchange()["ENk"], fx["ENk_cubic"], PARITY, "ENk")
    ck(lib.md_pimd_fill_VB_x(s.pimd))
    assert_close(s.exchange()["VBN"], fx["VBN_cubic"], PARITY, "VBN")
    ck(lib.md_pimd_fill_force_VB_x(s.pimd, h["image"]))
    assert_close(s.state()["f"], fx["f_cubic/f"], 1e-10, "cubic exchange force")
    ck(lib.md_pimd_fill_ENk2_x(s.pimd, h["image"]))
    assert_close(s.exchange()["ENk2"], fx["ENk2_cubic"], PARITY, "ENk2")
    s.free()
