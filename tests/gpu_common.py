"""Helpers shared by the GPU parity tests: build the same ring-polymer state
in the CUDA library (through its C ABI) and in the oracle."""
import os
import sys

import numpy as np

from conftest import ROOT

sys.path.insert(0, os.path.join(ROOT, "md-lab_gb300"))
import orc  # noqa: E402
import xmd_x  # noqa: E402

PARITY = 1e-10  # relative tolerance of the FP64 path against the reference


def random_state(D, L, N, P, T, box, ueg, seed, f=1, fc=0):
    """Seeded state in the reference's bead-major order."""
    rng = np.random.default_rng(seed)
    nb = N * P
    if ueg:
        centre = rng.uniform(0, box, size=(N, 1, D))
        x = (centre + 0.1 * rng.standard_normal((N, P, D))).reshape(nb * D)
    else:
        centre = rng.standard_normal((N, 1, D))
        x = (centre + 0.3 * rng.standard_normal((N, P, D))).reshape(nb * D)
    v = rng.standard_normal(nb * D) * np.sqrt(T)
    ndof = D * nb - fc
    nf = ndof // f + (ndof % f != 0)
    cf = np.array([f if (i + 1) * f <= ndof else ndof - i * f for i in range(nf)], dtype=np.float64)
    theta = 0.01 * rng.standard_normal(nf * L)
    vtheta = 1 + 0.1 * rng.standard_normal(nf * L)
    Q = np.full(nf * L, 0.3)
    Q[::L] *= cf
    return {"m": np.ones(nb), "x": x, "v": v, "f": np.zeros(nb * D), "theta": theta,
            "vtheta": vtheta, "Q": Q, "cf": cf}


def make_pair(lib, st, N, P, vi, T, box, f=1, fc=0):
    s = xmd_x.PimdSystem(lib, N, P, vi, T, box=box, f=f, fc=fc)
    s.set_state(**st)
    o = orc.OrcSim(lib.D, lib.L, N * P, st["m"], st["x"], st["v"], st["f"], st["cf"], st["theta"],
                   st["vtheta"], st["Q"], T, [box] * 3)
    return s, o
