"""The mixed-precision form (md_gb300_set_precision_x(MD_GB_PRECISION_MIXED)):
pair and real-space Ewald forces in FP32 (per-tile FP32 sums of at most 32
terms, tile partials in FP64), reciprocal space from double-float structure
factors.  Its error against the FP64 form is measured and bounded here,
force by force, up to the benchmark's full size."""
import numpy as np
import pytest

import xmd_x
from gpu_common import random_state
from helpers import relerr

pytestmark = pytest.mark.gpu

# max |f32 - f64| / max |f64|.  The FP32 rounding of the pair separations
# (about 1e-6 absolute in a box of 13) sets the error: 2.1e-5 at the
# benchmark's size (512 electrons, 64 beads, |n| <= 10).
MIXED_FORCE_TOL = 5e-5


def _forces(lib, s, pf, mode):
    lib.check(lib.md_gb300_set_precision_x(mode))
    try:
        lib.check(lib.md_reset_force_x(s.sim))
        lib.check(lib.md_pimd_calc_pair_force_x(s.pimd, pf))
        return s.state()["f"]
    finally:
        lib.md_gb300_set_precision_x(0)


@pytest.mark.parametrize("case", [
    ("md_coulomb_3d_ewald_force_x", 3, 64, 8, 6, True),
    ("md_coulomb_3d_ewald_force_x", 3, 512, 4, 10, True),
    ("md_coulomb_3d_ewald_force_x", 3, 512, 64, 10, True),
    ("md_gaussian_force_x", 3, 100, 8, 0, False),
    ("md_periodic_gaussian_force_x", 2, 70, 6, 0, True),
    ("md_coulomb_periodic_force_x", 3, 45, 4, 0, True),
], ids=lambda c: f"{c[0][3:-8]}_d{c[1]}_N{c[2]}_P{c[3]}")
def test_mixed_forces_close_to_fp64(case):
    fn, D, N, P, nsum, periodic = case
    lib = xmd_x.load(D, 4)
    box = (4 * np.pi * N / 3) ** (1 / 3) if periodic else 10.0
    st = random_state(D, 4, N, P, 1.0, box, periodic, seed=N + P)
    s = xmd_x.PimdSystem(lib, N, P, 0.5, 1.0, box=box)
    s.set_state(**st)
    xmd_x.set_potentials(lib, gauss_g=0.75 * np.pi, gauss_s=0.5, coul_s=1.0, alpha=5.6 / box, nsum=max(nsum, 1))
    pf = lib.fn(fn)
    f64 = _forces(lib, s, pf, 0)
    f32 = _forces(lib, s, pf, 1)
    err = relerr(f32, f64)
    print(f"{fn} N={N} P={P}: mixed vs FP64 force error {err:.2e} of max |f| {np.abs(f64).max():.3e}")
    assert err <= MIXED_FORCE_TOL
    s.free()
