"""Ensembles: several independent systems advanced by one CUDA graph (one
launch per step, each system on its own branch, or one persistent kernel for
all of them), and the tile-shape autotuners.  The ensemble must give bit-for-bit the
states that stepping each system on its own gives; the autotuner's choice
must not change any force."""
import ctypes as C
import math

import numpy as np
import pytest

import xmd_x
from gpu_common import random_state
from helpers import relerr

pytestmark = pytest.mark.gpu

STEP_FN = C.CFUNCTYPE(C.c_int, C.c_int, C.c_void_p)


@pytest.fixture(scope="module")
def lib():
    return xmd_x.load(3, 4)


def make(lib, spec, seed):
    kind, N, P, vi, beta = spec
    T = 1.0 / beta
    if kind == "ueg":
        box = (4 * math.pi * N / 3) ** (1 / 3) * 2.0
        st = random_state(3, 4, N, P, T, box, True, seed)
    else:
        box = 10.0
        st = random_state(3, 4, N, P, T, box, False, seed)
    s = xmd_x.PimdSystem(lib, N, P, vi, T, box=box)
    s.set_state(**st)
    return s, box


def potentials(lib, kind, box):
    if kind == "ueg":
        xmd_x.set_potentials(lib, coul_s=1.0, alpha=5.6 / box, nsum=4)
    else:
        xmd_x.set_potentials(lib, trap_w=1.0, gauss_g=0.75 * math.pi, gauss_s=0.5)


def step(lib, kind, s, box):
    potentials(lib, kind, box)
    if kind == "ueg":
        xmd_x.md_step(lib, s, 0.05, image=1, pair=lib.fn("md_coulomb_3d_ewald_force_x"), pbc=True)
    else:
        xmd_x.md_step(lib, s, 0.005, trap=lib.fn("md_harmonic_trap_force_x"), pair=lib.fn("md_gaussian_force_x"))


SPECS = [("trap", 8, 16, 1.0, 2.0), ("ueg", 16, 8, 0.5, 1.0), ("trap", 12, 32, 0.25, 4.0), ("ueg", 24, 16, 0.75, 3.0)]


@pytest.mark.parametrize("mixed", [0, 1])
def test_ensemble_graph_matches_individual_steps(lib, mixed):
    lib.check(lib.md_gb300_set_precision_x(mixed))
    try:
        ens = [make(lib, sp, 100 + i) for i, sp in enumerate(SPECS)]
        ref = [make(lib, sp, 100 + i) for i, sp in enumerate(SPECS)]
        for (s, box), sp in zip(ens + ref, SPECS + SPECS):
            step(lib, sp[0], s, box)  # device state and tables exist before capture

        def cb(i, ctx):
            try:
                s, box = ens[i]
                step(lib, SPECS[i][0], s, box)
                return 0
            except Exception:
                return -1

        fn = STEP_FN(cb)
        g = C.c_void_p()
        lib.check(lib.md_gb300_capture_ensemble_x(len(SPECS), C.cast(fn, C.c_void_p), None, C.byref(g)),
                  "ensemble capture")
        assert lib.md_gb300_graph_kernel_count_x(g) > 10 * len(SPECS)
        lib.check(lib.md_gb300_graph_launch_x(g, 3))
        lib.check(lib.md_gb300_synchronize_x())
        for _ in range(3):
            for (s, box), sp in zip(ref, SPECS):
                step(lib, sp[0], s, box)
        for (a, _), (b, _) in zip(ens, ref):
            sa, sb = a.state(), b.state()
            for k in ("x", "v", "f", "vtheta", "theta"):
                np.testing.assert_array_equal(sa[k], sb[k])
        lib.md_gb300_graph_free_x(g)
        for s, _ in ens + ref:
            s.free()
    finally:
        lib.check(lib.md_gb300_set_precision_x(0))


def test_autotuned_tile_shape_leaves_forces_unchanged(lib):
    lib.check(lib.md_gb300_set_precision_x(1))
    try:
        for kind, N, P in (("ueg", 48, 16), ("trap", 32, 32)):
            s, box = make(lib, (kind, N, P, 0.5, 2.0), 7)
            potentials(lib, kind, box)
            pf = lib.fn("md_coulomb_3d_ewald_force_x" if kind == "ueg" else "md_gaussian_force_x")
            forces = []
            for wpb in (1, 2, 4, 8):
                lib.check(lib.md_gb300_set_pair_tile_x(pf, N, P, wpb))
                lib.check(lib.md_reset_force_x(s.sim))
                lib.check(lib.md_pimd_calc_pair_force_x(s.pimd, pf))
                forces.append(s.state()["f"])
            w, ms = C.c_int(), C.c_double()
            lib.check(lib.md_gb300_autotune_pair_x(s.pimd, pf, 3, C.byref(w), C.byref(ms)), "autotune")
            assert w.value in (1, 2, 4, 8) and ms.value > 0
            lib.check(lib.md_reset_force_x(s.sim))
            lib.check(lib.md_pimd_calc_pair_force_x(s.pimd, pf))
            forces.append(s.state()["f"])
            for f in forces[1:]:
                np.testing.assert_array_equal(f, forces[0])
            s.free()
    finally:
        lib.check(lib.md_gb300_set_precision_x(0))


def test_fp64_autotuner_keeps_parity(lib):
    """The FP64 launch shapes (tile blocks per SM, structure-factor layout)
    chosen by timing: the forces after tuning equal those before to rounding,
    and every layout gives the same structure-factor sums to rounding."""
    import orc
    from gpu_common import random_state
    from helpers import assert_close
    lib.check(lib.md_gb300_set_precision_x(0))
    for kind, N, P in (("ueg", 260, 2), ("trap", 96, 8)):
        box = (4 * np.pi * N / 3) ** (1 / 3) if kind == "ueg" else 10.0
        st = random_state(3, 4, N, P, 1.0, box, kind == "ueg", seed=N)
        s = xmd_x.PimdSystem(lib, N, P, 0.5, 1.0, box=box)
        s.set_state(**st)
        xmd_x.set_potentials(lib, gauss_g=0.75 * np.pi, gauss_s=0.5, coul_s=1.0, alpha=5.6 / box, nsum=4)
        pf = lib.fn("md_coulomb_3d_ewald_force_x" if kind == "ueg" else "md_gaussian_force_x")

        def forces():
            lib.check(lib.md_reset_force_x(s.sim))
            lib.check(lib.md_pimd_calc_pair_force_x(s.pimd, pf))
            return s.state()["f"]

        before = forces()
        bps, lay, ms = C.c_int(), C.c_int(), C.c_double()
        lib.check(lib.md_gb300_autotune_fp64_x(s.pimd, pf, 3, C.byref(bps), C.byref(lay), C.byref(ms)), "autotune")
        assert bps.value in (1, 2, 3) and ms.value > 0
        assert lay.value in ((1, 2, 3) if kind == "ueg" else (0,))
        assert_close(forces(), before, 1e-13, "forces after FP64 autotuning")
        if kind == "ueg":  # the untuned Ewald path is pinned by the parity tests
            s.free()
            continue
        o = orc.OrcSim(3, 4, N * P, st["m"], st["x"], st["v"], np.zeros(N * P * 3), st["cf"], st["theta"],
                       st["vtheta"], st["Q"], 1.0, [box] * 3)
        prm = orc.params(gauss_g=0.75 * np.pi, gauss_s=0.5, coul_s=1.0, coul_alpha=5.6 / box, coul_nsum=4)
        orc.lib().orc_pair_force(o.ref, N, P, orc.PAIR_EWALD if kind == "ueg" else orc.PAIR_GAUSSIAN,
                                 orc.C.byref(prm))
        assert_close(forces(), o.f, 1e-10, "tuned FP64 forces vs the oracle")
        s.free()


# uneven systems for the persistent kernel: traps with Gaussian repulsion and
# electron gases (Ewald |n| <= 4 and 8), N from 8 to 160 (more than one
# staged chunk of 128 particles, five 32-row chunks of the recursion), P from
# 2 to 32, xi from 0 to 1
PERSISTENT = [("trap", 8, 16, 1.0, 2.0, 0), ("ueg", 16, 8, 0.5, 1.0, 4), ("trap", 12, 32, 0.25, 4.0, 0),
              ("ueg", 24, 16, 0.75, 3.0, 8), ("ueg", 40, 4, 0.0, 2.0, 8), ("trap", 70, 8, 1.0, 5.0, 0),
              ("ueg", 160, 2, 1.0, 1.5, 4), ("trap", 33, 3, 0.5, 8.0, 0)]


def persistent_step(lib, spec, s, box):
    kind, nsum = spec[0], spec[5]
    if kind == "ueg":
        xmd_x.set_potentials(lib, coul_s=1.0, alpha=5.6 / box, nsum=nsum)
        xmd_x.md_step(lib, s, 0.05, image=1, pair=lib.fn("md_coulomb_3d_ewald_force_x"), pbc=True)
    else:
        xmd_x.set_potentials(lib, trap_w=1.0, gauss_g=0.75 * math.pi, gauss_s=0.5)
        xmd_x.md_step(lib, s, 0.005, trap=lib.fn("md_harmonic_trap_force_x"), pair=lib.fn("md_gaussian_force_x"))


def _persistent_pair(lib):
    ens = [make(lib, sp[:5], 300 + i) for i, sp in enumerate(PERSISTENT)]
    ref = [make(lib, sp[:5], 300 + i) for i, sp in enumerate(PERSISTENT)]
    for (s, box), sp in zip(ens + ref, PERSISTENT + PERSISTENT):
        persistent_step(lib, sp, s, box)  # device state and Ewald tables exist before planning

    def cb(i, ctx):
        try:
            s, box = ens[i]
            persistent_step(lib, PERSISTENT[i], s, box)
            return 0
        except Exception:
            return -1

    return ens, ref, STEP_FN(cb)


def test_persistent_ensemble_matches_individual_steps(lib):
    """One persistent launch per step against the same steps made by the
    per-system calls: positions, velocities, thermostats, forces, V_B and the
    primitive estimator after 3 steps."""
    lib.check(lib.md_gb300_set_precision_x(1))
    try:
        ens, ref, fn = _persistent_pair(lib)
        g = C.c_void_p()
        lib.check(lib.md_gb300_capture_ensemble_persistent_x(len(PERSISTENT), C.cast(fn, C.c_void_p), None,
                                                             C.byref(g)), "persistent capture")
        assert lib.md_gb300_graph_kernel_count_x(g) == 1
        lib.check(lib.md_gb300_graph_launch_x(g, 3))
        lib.check(lib.md_gb300_ensemble_status_x(g), "persistent step status")
        for _ in range(3):
            for (s, box), sp in zip(ref, PERSISTENT):
                persistent_step(lib, sp, s, box)
        worst = {}
        for (a, _), (b, _), sp in zip(ens, ref, PERSISTENT):
            sa, sb = a.state(), b.state()
            for k in ("x", "v", "theta", "vtheta", "f"):
                worst[k] = max(worst.get(k, 0.0), relerr(sa[k], sb[k]))
            ea, eb = a.exchange(), b.exchange()
            for k in ("ENk", "VBN"):
                worst[k] = max(worst.get(k, 0.0), relerr(ea[k], eb[k]))
            est = []
            for s in (a, b):
                lib.check(lib.md_pimd_calc_VBN_energy_x(s.pimd, s.stats))
                est.append(s.take_energy())
            worst["E_primitive"] = max(worst.get("E_primitive", 0.0), abs(est[0] - est[1]) / abs(est[1]))
        print("persistent vs per-system, largest relative differences:", worst)
        for k in ("x", "v", "theta", "vtheta", "ENk", "VBN", "E_primitive"):
            assert worst[k] <= 1e-12, (k, worst[k])
        assert worst["f"] <= 1e-9, worst["f"]
        lib.md_gb300_graph_free_x(g)
        for s, _ in ens + ref:
            s.free()
    finally:
        lib.check(lib.md_gb300_set_precision_x(0))


def test_persistent_ensemble_autotuner_and_refusals(lib):
    """The grid-shape autotuner (blocks per SM, groups) picks a shape that
    runs; the capture then uses it and still matches the per-system calls.  A step with a call that is
    not part of the reference driver's step, or in FP64 mode, is refused."""
    lib.check(lib.md_gb300_set_precision_x(1))
    try:
        ens, ref, fn = _persistent_pair(lib)
        bps, grp, ms = C.c_int(), C.c_int(), C.c_double()
        lib.check(lib.md_gb300_autotune_ensemble_x(len(PERSISTENT), C.cast(fn, C.c_void_p), None, 2, C.byref(bps),
                                                   C.byref(grp), C.byref(ms)), "ensemble autotune")
        assert bps.value in (1, 2, 3) and grp.value in (1, 2, 4, 8, 16, 32) and ms.value > 0
        # the autotuner advanced the systems: the per-system copies restart
        # from their state
        for (a, _), (b, _) in zip(ens, ref):
            st = a.state()
            b.set_state(**st)
        g = C.c_void_p()
        lib.check(lib.md_gb300_capture_ensemble_persistent_x(len(PERSISTENT), C.cast(fn, C.c_void_p), None,
                                                             C.byref(g)), "persistent capture")
        lib.check(lib.md_gb300_graph_launch_x(g, 2))
        lib.check(lib.md_gb300_ensemble_status_x(g), "persistent step status")
        for _ in range(2):
            for (s, box), sp in zip(ref, PERSISTENT):
                persistent_step(lib, sp, s, box)
        for (a, _), (b, _) in zip(ens, ref):
            sa, sb = a.state(), b.state()
            assert relerr(sa["x"], sb["x"]) <= 1e-12
            assert relerr(sa["f"], sb["f"]) <= 1e-9
        lib.md_gb300_graph_free_x(g)

        def bad(i, ctx):
            s, box = ens[i]
            r = lib.md_update_nhc_VV3_1_x(s.sim, 0.01)
            if r:
                return r
            return lib.md_pimd_calc_VBN_energy_x(s.pimd, s.stats)  # not a step call

        bad_fn = STEP_FN(bad)
        assert lib.md_gb300_capture_ensemble_persistent_x(1, C.cast(bad_fn, C.c_void_p), None, C.byref(g)) != 0
        lib.check(lib.md_gb300_set_precision_x(0))
        assert lib.md_gb300_capture_ensemble_persistent_x(len(PERSISTENT), C.cast(fn, C.c_void_p), None,
                                                          C.byref(g)) != 0
        # the refusals left no recording behind: ordinary calls work
        for (s, box), sp in zip(ens, PERSISTENT):
            persistent_step(lib, sp, s, box)
        for s, _ in ens + ref:
            s.free()
    finally:
        lib.check(lib.md_gb300_set_precision_x(0))


@pytest.mark.parametrize("variant", [(2, 4), (3, 8)], ids=["d2l4", "d3l8"])
def test_persistent_ensemble_other_variants(variant):
    """The persistent kernel's other instantiations: D = 2 (traps with the
    periodic Gaussian pair force, minimum image) and chains of length 8
    (traps and an electron gas), against the per-system calls."""
    D, L = variant
    vl = xmd_x.load(D, L)
    vl.check(vl.md_gb300_set_precision_x(1))
    try:
        specs = [("trap", 10, 8, 1.0, 2.0), ("trap", 40, 4, 0.5, 3.0), ("trap", 70, 16, 0.0, 1.0)]
        if D == 3:
            specs.append(("ueg", 24, 8, 0.75, 2.0))

        def make_v(spec, seed):
            kind, N, P, vi, beta = spec
            T = 1.0 / beta
            box = (4 * math.pi * N / 3) ** (1 / 3) * 2.0 if kind == "ueg" else 6.0
            st = random_state(D, L, N, P, T, box, kind == "ueg", seed)
            s = xmd_x.PimdSystem(vl, N, P, vi, T, box=box)
            s.set_state(**st)
            return s, box

        def stepv(spec, s, box):
            if spec[0] == "ueg":
                xmd_x.set_potentials(vl, coul_s=1.0, alpha=5.6 / box, nsum=4)
                xmd_x.md_step(vl, s, 0.05, image=1, pair=vl.fn("md_coulomb_3d_ewald_force_x"), pbc=True)
            elif D == 2:
                xmd_x.set_potentials(vl, trap_w=1.0, gauss_g=0.75 * math.pi, gauss_s=0.5)
                xmd_x.md_step(vl, s, 0.005, image=1, trap=vl.fn("md_harmonic_trap_force_x"),
                              pair=vl.fn("md_periodic_gaussian_force_x"))
            else:
                xmd_x.set_potentials(vl, trap_w=1.0, gauss_g=0.75 * math.pi, gauss_s=0.5)
                xmd_x.md_step(vl, s, 0.005, trap=vl.fn("md_harmonic_trap_force_x"), pair=vl.fn("md_gaussian_force_x"))

        ens = [make_v(sp, 500 + i) for i, sp in enumerate(specs)]
        ref = [make_v(sp, 500 + i) for i, sp in enumerate(specs)]
        for (s, box), sp in zip(ens + ref, specs + specs):
            stepv(sp, s, box)

        def cb(i, ctx):
            try:
                s, box = ens[i]
                stepv(specs[i], s, box)
                return 0
            except Exception:
                return -1

        fn = STEP_FN(cb)
        g = C.c_void_p()
        vl.check(vl.md_gb300_capture_ensemble_persistent_x(len(specs), C.cast(fn, C.c_void_p), None, C.byref(g)),
                 "persistent capture")
        vl.check(vl.md_gb300_graph_launch_x(g, 3))
        vl.check(vl.md_gb300_ensemble_status_x(g), "persistent step status")
        for _ in range(3):
            for (s, box), sp in zip(ref, specs):
                stepv(sp, s, box)
        for (a, _), (b, _) in zip(ens, ref):
            sa, sb = a.state(), b.state()
            for k in ("x", "v", "theta", "vtheta", "f"):
                assert relerr(sa[k], sb[k]) <= (1e-9 if k == "f" else 1e-12), k
        vl.md_gb300_graph_free_x(g)
        for s, _ in ens + ref:
            s.free()
    finally:
        vl.check(vl.md_gb300_set_precision_x(0))
