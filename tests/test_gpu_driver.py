"""The key/value-input driver runs the reference's step sequence on the GPU
library: its estimator samples equal those of the same sequence driven
through the C ABI from Python (same seed, same initial conditions), and its
first sampled step agrees with the oracle."""
import math
import os
import subprocess

import numpy as np
import pytest

import xmd_x

pytestmark = pytest.mark.gpu

BIN = os.path.join(xmd_x.HERE, "bin")


def run_driver(D, L, text, tmp_path):
    p = tmp_path / "input.txt"
    p.write_text(text)
    out = subprocess.run([os.path.join(BIN, f"xmd_run_d{D}l{L}"), str(p)], capture_output=True, text=True,
                         check=True).stdout
    samples = [tuple(float(v) for v in ln.split()[1:]) for ln in out.splitlines() if ln.startswith("sample")]
    result = [ln for ln in out.splitlines() if ln.startswith("result")]
    return np.array(samples), result[0].split()


def python_run(D, L, N, P, T, omega, vi, g, s, dt, equil, steps, every, seed):
    """the driver's sequence through the Python binding"""
    lib = xmd_x.load(D, L)
    sysm = xmd_x.PimdSystem(lib, N, P, vi, T, box=10.0)
    lib.md_set_seed_x(seed)
    x = np.array([lib.md_random_gaussian_x() / math.sqrt(omega) for _ in range(N * P * D)])
    sysm.set_state(x=x)
    lib.md_init_particle_mass_x(sysm.sim, 1.0, 0, N * P)
    lib.md_init_maxwell_vel_x(sysm.sim, T)
    lib.md_init_nhc_x(sysm.sim, lib.md_get_quick_Q_x(T, sysm.pimd.contents.omegaP), 0, sysm.sim.contents.Nf, 0.0)
    xmd_x.set_potentials(lib, trap_w=omega, gauss_g=g, gauss_s=s)
    lib.check(lib.md_gb300_set_precision_x(0))
    trap = lib.fn("md_harmonic_trap_force_x")
    pair = lib.fn("md_gaussian_force_x") if g != 0 else None
    out = []
    for it in range(1, equil + steps + 1):
        xmd_x.md_step(lib, sysm, dt, trap=trap, pair=pair)
        if it > equil and (it - equil) % every == 0:
            ck = lib.check
            ck(lib.md_pimd_calc_trap_energy_x(sysm.pimd, lib.fn("md_harmonic_trap_energy_x"), sysm.stats))
            pot = sysm.take_energy()
            if pair:
                ck(lib.md_pimd_calc_pair_energy_x(sysm.pimd, lib.fn("md_gaussian_energy_x"), sysm.stats))
                pot += sysm.take_energy()
            ck(lib.md_pimd_calc_VBN_energy_x(sysm.pimd, sysm.stats))
            ep = sysm.take_energy() + pot
            ck(lib.md_pimd_fast_fill_ENk2_x(sysm.pimd, 0))
            ck(lib.md_pimd_calc_vi_virial_energy_x(sysm.pimd, sysm.stats, 0))
            out.append((it, ep, sysm.take_energy() + pot))
    sysm.free()
    return np.array(out)


@pytest.mark.parametrize("D,L,g", [(2, 4, 0.0), (3, 4, 2.0), (3, 8, 1.0)])
def test_driver_matches_the_same_calls_from_python(tmp_path, D, L, g):
    N, P, T, omega, vi, s, dt, equil, steps, every, seed = 40, 12, 0.4, 1.0, 0.8, 0.5, 0.01, 10, 30, 5, 3
    text = (f"N {N}\nP {P}\nT {T}\nomega {omega}\nvi {vi}\ng {g}\ns {s}\ndt {dt}\nequil {equil}\n"
            f"steps {steps}\nevery {every}\nseed {seed}\nblocks 3\n")
    got, result = run_driver(D, L, text, tmp_path)
    ref = python_run(D, L, N, P, T, omega, vi, g, s, dt, equil, steps, every, seed)
    assert got.shape == ref.shape == (steps // every, 3)
    assert np.array_equal(got[:, 0], ref[:, 0])
    scale = np.abs(ref[:, 1:]).max()
    assert np.abs(got[:, 1:] - ref[:, 1:]).max() <= 1e-12 * scale
    assert result[0] == "result" and int(result[result.index("samples") + 1]) == steps // every
    assert abs(float(result[2]) - ref[:, 1].mean()) <= 1e-12 * scale
