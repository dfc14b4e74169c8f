"""Observables outside the step on the GPU, against the reference's recorded
values and the oracle: the virial about the box centre and the centroid
virial (md_pimd_x.c:3898, :3924), g(r) between bead 1 and bead pi (:2974;
bin counts bit for bit), and the whole-polymer periodic wrap (:4350)."""
import numpy as np
import pytest

import fixtures
import orc
import xmd_x
from gpu_common import PARITY
from helpers import assert_close

pytestmark = pytest.mark.gpu


def _system(fx):
    h = fixtures.header(fx)
    lib = xmd_x.load(h["D"], h["L"])
    N, P, D = h["N"], h["P"], h["D"]
    s = xmd_x.PimdSystem(lib, N, P, h["vi"], h["T"], box=h["box"])
    s.set_state(m=fx["m"], x=fx["obs/x"], f=fx["obs/f"], v=np.zeros(N * P * D))
    return lib, s, h


def _gr(lib, s, pts, rmax, norm, pi, image, seed_value=0.25):
    st = lib.md_alloc_stats_x(pts)
    st.contents.fxs[0][3] = seed_value  # the call adds to what is there
    lib.check(lib.md_pimd_calc_pair_correlation_x(s.pimd, st, rmax, norm, pi, image), "g(r)")
    out = np.array([st.contents.fxs[0][i] for i in range(pts)])
    lib.md_gb300_free_stats_x(st)
    return out


@pytest.mark.parametrize("name", ["d3l4_obs_ueg", "d2l4_obs_trap"])
def test_observables_match_reference(name):
    fx = fixtures.load(name)
    lib, s, h = _system(fx)
    try:
        lib.check(lib.md_pimd_calc_virial_energy_x(s.pimd, s.stats))
        assert_close([s.take_energy()], fx["obs/e_virial"], PARITY, "virial about the box centre")
        for fc in (0, 3):
            lib.check(lib.md_pimd_calc_centroid_virial_energy_x(s.pimd, s.stats, fc))
            assert_close([s.take_energy()], fx[f"obs/e_centroid_fc{fc}"], PARITY, f"centroid virial fc={fc}")
        pts, rmax, norm, pi = fx["gr/params"]
        for img, key in ((0, "gr/plain"), (1, "gr/image")):
            got = _gr(lib, s, int(pts), rmax, norm, int(pi), img)
            assert np.array_equal(got, fx[key]), (key, got, fx[key])
        lib.check(lib.md_pimd_polymer_periodic_boundary_x(s.pimd))
        assert np.array_equal(s.state()["x"], fx["pbc/x"])
    finally:
        s.free()


@pytest.mark.parametrize("N,P,ueg", [(256, 16, True), (300, 8, False)])
def test_observables_match_oracle(N, P, ueg):
    D, L = 3, 4
    lib = xmd_x.load(D, L)
    rng = np.random.default_rng(N + P)
    box = (4 * np.pi * N / 3) ** (1 / 3) if ueg else 4.0
    nb = N * P
    centre = rng.uniform(-0.3 * box, 1.3 * box, (N, 1, D)) if ueg else rng.standard_normal((N, 1, D))
    x = (centre + 0.2 * rng.standard_normal((N, P, D))).ravel()
    f = rng.standard_normal(nb * D)
    m = np.ones(nb)
    T, beta = 0.7, 1 / 0.7
    s = xmd_x.PimdSystem(lib, N, P, 0.5, T, box=box)
    s.set_state(m=m, x=x, f=f, v=np.zeros(nb * D))
    o = orc.OrcSim(D, L, nb, m, x, np.zeros(nb * D), f, np.ones(nb * D), np.zeros(nb * D * L), np.zeros(nb * D * L),
                   np.ones(nb * D * L), T, [box] * 3)
    Lo = orc.lib()
    try:
        lib.check(lib.md_pimd_calc_virial_energy_x(s.pimd, s.stats))
        assert_close([s.take_energy()], [Lo.orc_virial_energy(o.ref, N, P)], PARITY, "virial")
        lib.check(lib.md_pimd_calc_centroid_virial_energy_x(s.pimd, s.stats, 3))
        assert_close([s.take_energy()], [Lo.orc_centroid_virial_energy(o.ref, N, P, beta, 3)], PARITY,
                     "centroid virial")
        pts, rmax, norm = 64, box / 2, N * (N - 1) / 2.0
        for img in (0, 1):
            ref = np.zeros(pts)
            ref[3] = 0.25
            Lo.orc_pair_correlation(o.ref, N, P, pts, rmax, norm, P // 2 + 1, img, orc.ptr(ref))
            assert np.array_equal(_gr(lib, s, pts, rmax, norm, P // 2 + 1, img), ref)
        lib.check(lib.md_pimd_polymer_periodic_boundary_x(s.pimd))
        Lo.orc_polymer_periodic_boundary(o.ref, N, P)
        assert np.array_equal(s.state()["x"], o.x)
    finally:
        s.free()
