"""C-ABI checks that need no GPU: the library loads, exports every entry
point its headers declare, keeps the reference's struct layout, reproduces the
reference's host-side initial conditions bit for bit, and refuses device work
loudly when there is no GPU."""
import ctypes as C
import glob
import os
import re
import subprocess

import numpy as np
import pytest

import fixtures
from conftest import ROOT

import sys
sys.path.insert(0, os.path.join(ROOT, "md-lab_gb300"))
import xmd_x  # noqa: E402

INCLUDE = os.path.join(ROOT, "include")
REF = os.path.join(ROOT, "oracle", "_ref")


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(INCLUDE, "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(md_\w+)\s*\(", src, flags=re.M):
            if "typedef" in src[m.start():m.end()]:
                continue
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module", params=[(3, 4), (2, 4), (3, 8)], ids=lambda v: f"d{v[0]}l{v[1]}")
def lib(request):
    D, L = request.param
    return xmd_x.load(D, L)


def test_headers_declare_the_path():
    names = declared_functions()
    for must in ("md_pimd_fast_fill_ENk_x", "md_pimd_fill_VB_x", "md_pimd_fast_fill_force_VB_x",
                 "md_pimd_calc_pair_force_x", "md_update_nhc_VV3_1_x", "md_update_nhc_VV3_2_x",
                 "md_coulomb_3d_ewald_force_x", "md_pimd_calc_vi_virial_energy_x",
                 "md_gb300_capture_begin_x"):
        assert must in names


def test_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib.path], capture_output=True, text=True,
                         check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    for g in ("md_trap_frequency_x", "md_gaussian_strength_x", "md_coulomb_n_sum_x", "md_pimd_mode_x"):
        assert g in exported


def test_struct_layout(lib):
    D, L = lib.D, lib.L
    assert C.sizeof(lib.Particle) == 8 * (1 + 3 * D)
    assert C.sizeof(lib.Nhc) == 8 + 24 * L
    dim, ln = C.c_int(), C.c_int()
    lib.md_gb300_variant_x(C.byref(dim), C.byref(ln))
    assert (dim.value, ln.value) == (D, L)


@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "libxmd_x_d3l4.so")),
                    reason="MD-Lab's own build is not present")
def test_struct_layout_matches_reference_build():
    """Compile a probe against the reference headers and compare offsets."""
    probe = os.path.join(REF, "layout_probe.c")
    with open(probe, "w") as fh:
        fh.write('#include <stdio.h>\n#include <stddef.h>\n#include "md_pimd_x.h"\n'
                 'int main(void){printf("%zu %zu %zu %zu %zu %zu %zu\\n", sizeof(md_particle_t_x),'
                 ' sizeof(md_nhc_t_x), sizeof(md_simulation_t_x), sizeof(md_pimd_t_x),'
                 ' offsetof(md_pimd_t_x, VBN), offsetof(md_pimd_t_x, worm_pos), sizeof(md_stats_t_x));}\n')
    exe = os.path.join(REF, "layout_probe")
    subprocess.run(["gcc", "-I", os.path.join(REF, "src_d3l4"), "-o", exe, probe], check=True)
    ref = list(map(int, subprocess.run([exe], capture_output=True, text=True).stdout.split()))
    lib = xmd_x.load(3, 4)
    mine = [C.sizeof(lib.Particle), C.sizeof(lib.Nhc), C.sizeof(lib.Sim), C.sizeof(lib.Pimd),
            lib.Pimd.VBN.offset, lib.Pimd.worm_pos.offset, C.sizeof(lib.Stats)]
    assert mine == ref


def test_rng_matches_reference(lib):
    fx = fixtures.load("rng")
    lib.md_set_seed_x(1234)
    u = [lib.md_random_uniform_x(-1.0, 2.0) for _ in range(32)]
    g = [lib.md_random_gaussian_x() for _ in range(32)]
    np.testing.assert_array_equal(u, fx["uniform"])
    np.testing.assert_array_equal(g, fx["gaussian"])


def _init_like_golden(lib, name):
    """Initial conditions through the library's own host ABI, exactly as
    tests/golden/make_golden.c builds them with the reference."""
    fx = fixtures.load(name)
    h = fixtures.header(fx)
    if h["D"] != lib.D or h["L"] != lib.L:
        pytest.skip("other variant")
    lib.md_set_seed_x(int({"d2l4_cfg1": 2024, "d3l4_trap_vi1": 11, "d3l4_trap_chain3": 17,
                           "d3l4_ueg": 18, "d3l8_trap": 19}[name]))
    s = xmd_x.PimdSystem(lib, h["N"], h["P"], h["vi"], h["T"], box=h["box"], f=h["f"], fc=h["fc"])
    lib.md_init_particle_mass_x(s.sim, 1.0, 0, s.nb)
    p = s._particles()
    D = lib.D
    if h["ueg"]:
        c = np.full(D, h["box"] / 2)
        Lv = np.full(D, h["box"])
        lib.md_pimd_init_particle_uniform_pos_x(s.pimd, c.ctypes.data_as(xmd_x._dp),
                                                Lv.ctypes.data_as(xmd_x._dp), 0.05 * 2.0)
    else:
        for b in range(s.nb):
            for d in range(D):
                p[b, 1 + d] = lib.md_random_gaussian_x()
    lib.md_init_maxwell_vel_x(s.sim, h["T"])
    Q = lib.md_get_quick_Q_x(h["T"], h["omegaP"])
    lib.md_init_nhc_x(s.sim, Q, 0, s.sim.contents.Nf, 0.0)
    return fx, s


@pytest.mark.parametrize("name", ["d2l4_cfg1", "d3l4_trap_vi1", "d3l4_trap_chain3", "d3l4_ueg",
                                  "d3l8_trap"])
def test_initial_conditions_match_reference(lib, name):
    fx, s = _init_like_golden(lib, name)
    p = s._particles()
    D = lib.D
    np.testing.assert_array_equal(p[:, 1:1 + D].ravel(), fx["init/x"])
    np.testing.assert_array_equal(p[:, 1 + D:1 + 2 * D].ravel(), fx["init/v"])
    c = s._chains()
    np.testing.assert_array_equal(c["Q"].ravel(), fx["init/Q"])
    np.testing.assert_array_equal(c["vtheta"].ravel(), fx["init/vtheta"])
    np.testing.assert_array_equal(c["f"].astype(float), fx["init/cf"])
    pc = s.pimd.contents
    h = fixtures.header(fx)
    assert pc.omegaP == h["omegaP"] and pc.beta == h["beta"]


def test_madelung_host(lib):
    if lib.D != 3:
        pytest.skip("3D only")
    fx = fixtures.load("d3_pairs")
    box = fx["L"].copy()
    for a, al in enumerate((5.6, 3.0)):
        for n in (1, 2, 3):
            xmd_x.set_potentials(lib, coul_s=1.3, alpha=al / box[0], nsum=n)
            v = lib.md_calc_3d_ueg_madelung_x(box.ctypes.data_as(xmd_x._dp))
            assert abs(v - fx[f"ewald_a{a}_n{n}/mad"][0]) <= 1e-13 * abs(v)


def test_no_gpu_fails_loudly():
    """Without a GPU every device entry point returns MD_GB_ERR_NO_DEVICE."""
    lib = xmd_x.load(3, 4)
    if lib.md_gb300_device_count_x() > 0:
        pytest.skip("a GPU is present")
    s = xmd_x.PimdSystem(lib, 4, 4, 1.0, 1.0)
    assert lib.md_reset_force_x(s.sim) == -1001
    assert lib.md_pimd_fast_fill_ENk_x(s.pimd, 0) == -1001
    assert lib.md_update_nhc_VV3_1_x(s.sim, 0.01) == -1001
    assert "no CUDA device" in lib.err()


def test_sk_sphere_builder_matches_reference():
    """md_alloc_sk_sphere_3d_x (host) against the reference's own shells"""
    import fixtures
    lib = xmd_x.load(3, 4)
    fx = fixtures.load("d3l4_trap_vi1")
    sk = lib.md_alloc_sk_sphere_3d_x(0.0, 0.5, 2.0)
    n = sk.contents.N
    assert n == len(fx["sk/qs"])
    np.testing.assert_array_equal(np.ctypeslib.as_array(sk.contents.qs, (n,)), fx["sk/qs"])
    np.testing.assert_array_equal(np.ctypeslib.as_array(sk.contents.qis, (3 * n,)), fx["sk/qis"])
