"""The work models bench.py's roofline lines use, checked on the CPU: the
FP64 form's split of the reciprocal columns and of the real-space images
partitions the work of the strict form, with the fractions the design
states."""
import math
import sys

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_column_split_partitions_the_kept_vectors():
    full = bench.kept_nz_pairs(10)
    fp64, fp32 = bench.kept_nz_pairs(10, "fp64"), bench.kept_nz_pairs(10, "fp32")
    assert fp64 + fp32 == full
    # the FP32 columns (nx^2 + ny^2 >= 49) hold a third to a half of the +-nz pairs
    assert 0.3 < fp32 / full < 0.5


def test_real_space_split_moves_more_than_half_of_the_images():
    n_all, n_fp64 = bench.n_images(5.2), bench.n_images(4.0)
    assert math.isclose(n_all, 4 / 3 * math.pi * (5.2 / 5.6) ** 3, rel_tol=1e-12)
    # images at alpha R >= 4 of those inside 5.2: 1 - (4 / 5.2)^3 = 54.5%
    assert math.isclose(1 - n_fp64 / n_all, 1 - (4 / 5.2) ** 3, rel_tol=1e-12)
    strict, split = bench.kernel_flops("pair_tiles_ewald_real"), bench.kernel_flops("pair_tiles_ewald_real", split=True)
    # 47 flop x 1.53 images + 39 a pair against 47 x 3.35 + 39: 56%
    assert 0.5 * strict < split < 0.6 * strict
    # the FP32 kernels' models do not depend on the split
    assert bench.kernel_flops("recip_force32", split=True) == bench.kernel_flops("recip_force32")
    assert bench.kernel_flops("recip_force", split=True) < bench.kernel_flops("recip_force")
