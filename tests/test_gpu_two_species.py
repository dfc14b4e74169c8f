"""Two species (md_pimd_calc_pair_force_2_x, md_pimd_calc_pair_energy_2_x)
on the GPU: against vectors recorded from the reference (cross terms alone,
a full force call, a trajectory) and against the oracle on ragged sizes,
Ewald included."""
import numpy as np
import pytest

import fixtures
import orc
import xmd_x
from gpu_common import PARITY, random_state
from helpers import assert_close

pytestmark = pytest.mark.gpu


def _system(lib, fx, sp, N, P, vi, T, box, prefix="init/"):
    s = xmd_x.PimdSystem(lib, N, P, vi, T, box=box)
    m = np.full(N * P, 1.0 if sp == "a/" else fixtures.header(fx, "two")["mb"])
    q = sp + prefix
    s.set_state(m=m, x=fx[q + "x"], v=fx[q + "v"], f=fx[q + "f"], theta=fx[q + "theta"],
                vtheta=fx[q + "vtheta"], Q=fx[q + "Q"], cf=fx[q + "cf"])
    return s


def _fns(lib, ueg):
    if ueg:
        return None, lib.fn("md_coulomb_3d_ewald_force_x"), lib.fn("md_coulomb_3d_ewald_energy_x")
    return lib.fn("md_harmonic_trap_force_x"), lib.fn("md_gaussian_force_x"), lib.fn("md_gaussian_energy_x")


@pytest.mark.parametrize("name", fixtures.TWO_FIXTURES)
def test_two_species_vs_reference(name):
    fx = fixtures.load(name)
    h = fixtures.header(fx, "two")
    lib = xmd_x.load(h["D"], h["L"])
    xmd_x.set_potentials(lib, trap_w=1.0, gauss_g=h["g"], gauss_s=h["s"], coul_s=1.0, alpha=h["alpha"],
                         nsum=h["nsum"])
    Na, Nb, P = h["N"], h["Nb"], h["P"]
    a = _system(lib, fx, "a/", Na, P, h["vi"], h["T"], h["box"])
    b = _system(lib, fx, "b/", Nb, P, h["vi"], h["T"], h["box"])
    trap, pf, pe = _fns(lib, h["ueg"])
    ck = lib.check
    try:
        ck(lib.md_reset_force_x(a.sim))
        ck(lib.md_reset_force_x(b.sim))
        ck(lib.md_pimd_calc_pair_force_2_x(a.pimd, b.pimd, pf))
        assert_close(a.state()["f"], fx["a/cross/f"], PARITY, "cross force on a")
        assert_close(b.state()["f"], fx["b/cross/f"], PARITY, "cross force on b")
        ck(lib.md_pimd_calc_pair_energy_2_x(a.pimd, b.pimd, pe, a.stats))
        assert_close([a.take_energy()], fx["cross/e"], PARITY, "cross energy")
        xmd_x.two_species_forces(lib, a, b, h["image"], trap, pf)
        assert_close(a.state()["f"], fx["a/all/f"], PARITY, "all forces on a")
        assert_close(b.state()["f"], fx["b/all/f"], PARITY, "all forces on b")
        # the reference's trajectory starts from these forces
        for _ in range(h["steps"]):
            xmd_x.two_species_step(lib, a, b, h["dt"], h["image"], trap, pf, bool(h["pbc"]))
        for sp, s in (("a/", a), ("b/", b)):
            st = s.state()
            for k in ("x", "v", "theta", "vtheta"):
                assert_close(st[k], fx[sp + "final/" + k], 1e-9, f"{sp} final {k}")
        ck(lib.md_pimd_calc_pair_energy_2_x(a.pimd, b.pimd, pe, a.stats))
        assert_close([a.take_energy()], fx["final/cross_e"], 1e-9, "final cross energy")
    finally:
        a.free()
        b.free()


CASES = [
    # D, Na, Nb, P, ueg, nsum, mb
    (3, 70, 45, 3, False, 0, 2.0),
    (3, 33, 97, 2, False, 0, 0.7),
    (2, 40, 31, 4, False, 0, 1.5),
    (3, 40, 33, 3, True, 4, 1.0),
    (3, 1, 64, 2, True, 2, 1.0),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"d{c[0]}_Na{c[1]}_Nb{c[2]}_P{c[3]}_{'ueg' if c[4] else 'gauss'}")
def test_two_species_vs_oracle(case):
    D, Na, Nb, P, ueg, nsum, mb = case
    lib = xmd_x.load(D, 4)
    T = 0.5
    box = (4 * np.pi * (Na + Nb) / 3) ** (1 / 3) * 1.5 if ueg else 10.0
    alpha = 5.6 / box
    xmd_x.set_potentials(lib, gauss_g=0.75 * np.pi, gauss_s=0.5, coul_s=1.0, alpha=alpha, nsum=max(nsum, 1))
    prm = orc.params(gauss_g=0.75 * np.pi, gauss_s=0.5, coul_s=1.0, coul_alpha=alpha, coul_nsum=max(nsum, 1))
    kind = orc.PAIR_EWALD if ueg else orc.PAIR_GAUSSIAN
    _, pf, pe = _fns(lib, ueg)
    sa = random_state(D, 4, Na, P, T, box, ueg, seed=Na * 7 + Nb)
    sb = random_state(D, 4, Nb, P, T, box, ueg, seed=Nb * 11 + Na)
    sb["m"] = np.full(Nb * P, mb)
    a = xmd_x.PimdSystem(lib, Na, P, 1.0, T, box=box)
    b = xmd_x.PimdSystem(lib, Nb, P, 1.0, T, box=box)
    a.set_state(**sa)
    b.set_state(**sb)
    oa = orc.OrcSim(D, 4, Na * P, sa["m"], sa["x"], sa["v"], sa["f"], sa["cf"], sa["theta"], sa["vtheta"],
                    sa["Q"], T, [box] * 3)
    ob = orc.OrcSim(D, 4, Nb * P, sb["m"], sb["x"], sb["v"], sb["f"], sb["cf"], sb["theta"], sb["vtheta"],
                    sb["Q"], T, [box] * 3)
    try:
        lib.check(lib.md_pimd_calc_pair_force_2_x(a.pimd, b.pimd, pf))
        orc.pair_force_2(oa, Na, ob, Nb, P, kind, prm)
        fa, fb = a.state()["f"], b.state()["f"]
        assert_close(fa, oa.f, PARITY, "cross force on a")
        assert_close(fb, ob.f, PARITY, "cross force on b")
        # momentum balance: sum of m f over both species vanishes in each slice
        pa = fa.reshape(Na, P, D) * sa["m"].reshape(Na, P, 1)
        pb = fb.reshape(Nb, P, D) * sb["m"].reshape(Nb, P, 1)
        scale = max(np.abs(pa).max(), np.abs(pb).max())
        assert np.abs(pa.sum(axis=0) + pb.sum(axis=0)).max() <= 1e-12 * (Na + Nb) * scale
        lib.check(lib.md_pimd_calc_pair_energy_2_x(a.pimd, b.pimd, pe, a.stats))
        assert_close([a.take_energy()], [orc.pair_energy_2(oa, Na, ob, Nb, P, kind, prm)], PARITY, "cross energy")
    finally:
        a.free()
        b.free()


def test_two_species_error_behaviour():
    lib = xmd_x.load(3, 4)
    xmd_x.set_potentials(lib, gauss_g=0.75 * np.pi, gauss_s=0.5, coul_s=1.0, alpha=0.5, nsum=2)
    a = xmd_x.PimdSystem(lib, 5, 4, 1.0, 0.5, box=10.0)
    b = xmd_x.PimdSystem(lib, 6, 2, 1.0, 0.5, box=10.0)
    c = xmd_x.PimdSystem(lib, 6, 4, 1.0, 0.5, box=11.0)
    try:
        for s, n, p in ((a, 5, 4), (b, 6, 2), (c, 6, 4)):
            s.set_state(**random_state(3, 4, n, p, 0.5, 10.0, True, seed=n + p))
        pf = lib.fn("md_gaussian_force_x")
        # a different number of beads: -1, as the reference returns
        assert lib.md_pimd_calc_pair_force_2_x(a.pimd, b.pimd, pf) == -1
        assert lib.md_pimd_calc_pair_energy_2_x(a.pimd, b.pimd, lib.fn("md_gaussian_energy_x"), a.stats) == -1
        # a callback without a device kernel, and Ewald across two boxes
        assert lib.md_pimd_calc_pair_force_2_x(a.pimd, c.pimd, lib.fn("md_harmonic_trap_force_x")) < 0
        assert lib.md_pimd_calc_pair_force_2_x(a.pimd, c.pimd, lib.fn("md_coulomb_3d_ewald_force_x")) < 0
        # the Gaussian across boxes uses a's box, as the reference does
        assert lib.md_pimd_calc_pair_force_2_x(a.pimd, c.pimd, pf) == 0
    finally:
        a.free()
        b.free()
        c.free()
