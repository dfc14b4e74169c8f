"""Speed of the oracle port against MD-Lab's own _nocl build on the same host.

Test infrastructure: the CPU baseline of bench.py times the oracle port
(xmd_oracle.c), because MD-Lab's sources are not on the GPU machine and its
x86 build does not run there.  This script measures, where the reference
build exists (oracle/_ref/libxmd_x_d3l4.so, made by `make -C oracle ref` from
the MD-Lab tree), how the port's speed compares with the reference's on the
same sample of the bench workload's dominant operation: the Ewald pair force
md_coulomb_3d_ewald_force_x (md_simulation_x.c:259-293) of the N=512
electron gas (rs = 1, alpha = 5.6 / L, |n| <= 10), on random pairs in the box.
Both are timed on one core, single-threaded, with the same pairs; the forces
are compared too.  Prints one JSON line.

    python oracle/time_reference.py [pairs]
"""
import ctypes as C
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import orc  # noqa: E402

N_BENCH, RS, ALPHA_L, NSUM = 512, 1.0, 5.6, 10


def main():
    pairs = int(sys.argv[1]) if len(sys.argv) > 1 else 2000
    path = os.path.join(HERE, "_ref", "libxmd_x_d3l4.so")
    if not os.path.exists(path):
        print(json.dumps({"unavailable": "no reference build at oracle/_ref (make -C oracle ref where the MD-Lab "
                                         "sources are mounted)"}))
        return 0
    ref = C.CDLL(path)
    box = (4 * math.pi * N_BENCH / 3) ** (1 / 3) * RS
    alpha = ALPHA_L / box
    ref.md_set_coulomb_force_strength_x(C.c_double(1.0))
    ref.md_set_coulomb_truc_x(C.c_double(alpha))
    ref.md_set_coulomb_n_sum_x(C.c_int(NSUM))
    fn = ref.md_coulomb_3d_ewald_force_x
    dp = C.POINTER(C.c_double)
    fn.argtypes = [dp, dp, dp, dp, C.c_double]
    fn.restype = None
    rng = np.random.default_rng(7)
    pts = rng.uniform(0, box, size=(pairs, 2, 3))
    Lb = np.full(3, box)
    f_ref = np.zeros((pairs, 3))
    f_orc = np.zeros((pairs, 3))
    t0 = time.perf_counter()
    for i in range(pairs):
        f = np.zeros(3)
        fn(pts[i, 0].ctypes.data_as(dp), pts[i, 1].ctypes.data_as(dp), f.ctypes.data_as(dp), Lb.ctypes.data_as(dp),
           C.c_double(1.0))
        f_ref[i] = f
    t_ref = time.perf_counter() - t0
    prm = orc.params(coul_s=1.0, coul_alpha=alpha, coul_nsum=NSUM)
    L_ = orc.lib()
    t0 = time.perf_counter()
    for i in range(pairs):
        f = np.zeros(3)
        L_.orc_pair_force_one(orc.PAIR_EWALD, C.byref(prm), 3, orc.ptr(pts[i, 0]), orc.ptr(pts[i, 1]), orc.ptr(f),
                              orc.ptr(Lb), 1.0)
        f_orc[i] = f
    t_orc = time.perf_counter() - t0
    diff = float(np.max(np.abs(f_orc - f_ref)) / max(np.max(np.abs(f_ref)), 1e-300))
    print(json.dumps({"pairs": pairs, "reference_us_per_pair": 1e6 * t_ref / pairs,
                      "port_us_per_pair": 1e6 * t_orc / pairs, "port_over_reference_time": t_orc / t_ref,
                      "max_relative_force_difference": diff, "workload": "Ewald pair force, N=512 electron gas box, "
                      "alpha L = 5.6, |n| <= 10, random pairs, one core"}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
