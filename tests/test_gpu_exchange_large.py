"""The exchange path at the sizes the benchmark runs, against the oracle.

Above four 32-row chunks (N > 128) the recursions are solved by the
thread-block-cluster kernel; below, by the single-block kernel.  Here both
are compared with the oracle's restatement of MD-Lab's _nocl recursions
(md_pimd_x.c:814-953, :2369-2721) on ring-polymer states with real exchange
(Brownian-bridge rings whose neighbours overlap), for every quantity of the
path: the cycle energies ENk, V_B, the backward recursion tmpV, the
connection probabilities G, the exchange spring forces, and both exchange
estimators on both of their paths (from the force call's cycle probabilities
and from the recursion).  A second test forces each solve kernel at the same
N and compares the two directly.

Tolerance.  ENk, V_B and tmpV are held to 1e-10 (V_B and tmpV element by
element).  G = exp(-beta(V_B^(j-1) + E + tmpV - V_B^(N))) takes the
difference of numbers of size beta V_B^(N) (up to ~2e5 here), so G, the
forces it weights and the estimator built from it inherit that condition
number: in the reference itself they move by up to 5e-9 relative when the
positions change by one unit in the last place.  Those quantities are held
to max(1e-10, DRIFT_FACTOR x that one-ulp drift of the oracle), the drift
measured on the same state in the same test.
"""
import numpy as np
import pytest

import orc
import xmd_x
from gpu_common import PARITY
from helpers import assert_close, relerr

pytestmark = pytest.mark.gpu

D, L = 3, 4
SOLVE_AUTO, SOLVE_BLOCK, SOLVE_CLUSTER = 0, 1, 2


def ueg_box(N, rs=1.0):
    return (4 * np.pi * N / 3) ** (1 / 3) * rs


def ring_state(N, P, beta, ueg, box, seed):
    """Closed Brownian-bridge rings (link spread sqrt(beta/P) per axis, the
    free ring polymer's) whose centres follow a random walk in particle
    order, so that particles l and l+1 overlap: the exchange cycles of the
    recursion join particles j..l in index order, and these states give
    them real weight.  The walk is wrapped into the box for the electron
    gas."""
    rng = np.random.default_rng(seed)
    sig = np.sqrt(beta / P)
    hop = 0.6 * np.sqrt(beta / 2)  # a centre-to-centre step of about a thermal wavelength / 3
    centre = np.cumsum(rng.standard_normal((N, 1, D)) * hop, axis=0)
    if ueg:
        centre = np.mod(centre + rng.uniform(0, box, size=(1, 1, D)), box)
    steps = rng.standard_normal((N, P, D)) * sig
    walk = np.cumsum(steps, axis=1)
    bridge = walk - (np.arange(1, P + 1)[None, :, None] / P) * walk[:, -1:, :]
    x = (centre + bridge).reshape(N * P * D)
    nb = N * P
    return {"m": np.ones(nb), "x": x, "v": np.zeros(nb * D), "f": np.zeros(nb * D),
            "theta": np.zeros(nb * D * L), "vtheta": np.zeros(nb * D * L),
            "Q": np.ones(nb * D * L), "cf": np.ones(nb * D)}


def tables(lib, s, N):
    tmpV = np.zeros(N + 1)
    G = np.zeros(N * N)
    lib.check(lib.md_gb300_exchange_tables_x(s.pimd, tmpV.ctypes.data_as(xmd_x._dp), G.ctypes.data_as(xmd_x._dp)),
              "exchange tables")
    return tmpV, G.reshape(N, N)


def assert_elementwise(a, b, tol, what):
    a, b = np.asarray(a), np.asarray(b)
    floor = 1e-12 * max(np.abs(b).max(), 1e-300)
    e = float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))
    assert e <= tol, f"{what}: elementwise relative error {e:.3e} > {tol:.1e}"


def exchange_on_gpu(lib, s, image):
    ck = lib.check
    ck(lib.md_reset_force_x(s.sim))
    ck(lib.md_pimd_fast_fill_ENk_x(s.pimd, image))
    ck(lib.md_pimd_fill_VB_x(s.pimd))
    ck(lib.md_pimd_fast_fill_force_VB_x(s.pimd, image))
    ex = s.exchange()
    tmpV, G = tables(lib, s, s.N)
    return {"ENk": ex["ENk"], "VBN": ex["VBN"], "tmpV": tmpV, "G": G, "f": s.state()["f"]}


def exchange_on_oracle(o, N, P, beta, vi, image):
    omegaP = np.sqrt(P) / beta
    o.f[:] = 0
    ENk, _ = orc.fast_fill_ENk(o, N, P, omegaP, image)
    VBN = orc.fill_VB(N, beta, vi, ENk)
    G, tmpV = orc.fast_force_VB(o, N, P, beta, vi, omegaP, image, ENk, VBN)
    return {"ENk": ENk, "VBN": VBN, "tmpV": tmpV, "G": G, "f": o.f.copy()}


DRIFT_FACTOR = 30.0  # the factor the trajectory tests allow over the reference's one-ulp drift


def oracle_all(st, N, P, T, box, beta, vi, image, x=None):
    """every quantity of the exchange path and both estimators, by the oracle"""
    o = orc.OrcSim(D, L, N * P, st["m"], st["x"] if x is None else x, st["v"], st["f"], st["cf"], st["theta"],
                   st["vtheta"], st["Q"], T, [box] * 3)
    out = exchange_on_oracle(o, N, P, beta, vi, image)
    Lo = orc.lib()
    ENk, VBN = out["ENk"], out["VBN"]
    out["e"] = np.array([Lo.orc_vbn_energy(D, N, P, beta, vi, orc.ptr(ENk), orc.ptr(VBN))])
    ENk2 = np.zeros(orc.ntri(N))
    Lo.orc_fast_fill_ENk2(o.ref, N, P, np.sqrt(P) / beta, image, orc.ptr(ENk2))
    out["ENk2"] = ENk2
    out["ev"] = np.array([Lo.orc_vi_virial_energy(o.ref, N, P, beta, vi, image, orc.ptr(ENk), orc.ptr(ENk2),
                                                  orc.ptr(VBN))])
    return out


def tolerances(st, N, P, T, box, beta, vi, image, ref):
    """max(1e-10, DRIFT_FACTOR x the oracle's own change under a one-ulp
    perturbation of every position) for each quantity"""
    rng = np.random.default_rng(12345)
    x2 = st["x"] * (1 + rng.choice([-1.0, 1.0], size=st["x"].shape) * 2.0 ** -52)
    pert = oracle_all(st, N, P, T, box, beta, vi, image, x=x2)
    tol = {k: max(PARITY, DRIFT_FACTOR * relerr(pert[k], ref[k])) for k in ("G", "f", "e", "ev")}
    tol.update({k: PARITY for k in ("ENk", "VBN", "tmpV", "ENk2")})
    return tol


def setup(N, P, vi, ueg, seed):
    lib = xmd_x.load(D, L)
    if ueg:  # the spin-polarised electron gas at rs = 1, theta = 0.5
        box = ueg_box(N)
        T = 0.5 * 0.5 * (6 * np.pi ** 2 * N / box ** 3) ** (2 / 3)
    else:
        box, T = 10.0, 0.5
    beta = 1.0 / T
    st = ring_state(N, P, beta, ueg, box, seed)
    s = xmd_x.PimdSystem(lib, N, P, vi, T, box=box)
    s.set_state(**st)
    o = orc.OrcSim(D, L, N * P, st["m"], st["x"], st["v"], st["f"], st["cf"], st["theta"], st["vtheta"],
                   st["Q"], T, [box] * 3)
    return lib, s, o, beta, 1 if ueg else 0, st, T, box


def compare(got, ref, tol, what):
    assert_close(got["ENk"], ref["ENk"], tol["ENk"], f"{what} ENk")
    assert_elementwise(got["VBN"], ref["VBN"], tol["VBN"], f"{what} V_B")
    assert_elementwise(got["tmpV"], ref["tmpV"], tol["tmpV"], f"{what} tmpV")
    assert_close(got["G"], ref["G"], tol["G"], f"{what} G")
    assert_close(got["f"], ref["f"], tol["f"], f"{what} exchange spring force")


CASES = [(N, P, kind, vi) for N in (129, 160, 512, 1024, 2048) for P in (8, 64) for kind in ("trap", "ueg")
         for vi in (0.0, 0.5, 1.0)]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"N{c[0]}_P{c[1]}_{c[2]}_xi{c[3]}")
def test_exchange_and_estimators_vs_oracle(case):
    N, P, kind, vi = case
    lib, s, o, beta, image, st, T, box = setup(N, P, vi, kind == "ueg", seed=N * 7 + P + int(10 * vi))
    try:
        assert lib.md_gb300_get_solve_path_x(N) == (SOLVE_CLUSTER if N > 128 else SOLVE_BLOCK)
        got = exchange_on_gpu(lib, s, image)
        ref = oracle_all(st, N, P, T, box, beta, vi, image)
        tol = tolerances(st, N, P, T, box, beta, vi, image, ref)
        compare(got, ref, tol, f"N={N} P={P} {kind} xi={vi}")
        ck = lib.check
        # estimators: first from the force call's cycle probabilities ...
        ck(lib.md_pimd_calc_VBN_energy_x(s.pimd, s.stats))
        assert_close([s.take_energy()], ref["e"], tol["e"], "primitive estimator (cycle probabilities)")
        ck(lib.md_pimd_fast_fill_ENk2_x(s.pimd, image))
        assert_close(s.exchange()["ENk2"], ref["ENk2"], tol["ENk2"], "ENk2")
        ck(lib.md_pimd_calc_vi_virial_energy_x(s.pimd, s.stats, image))
        assert_close([s.take_energy()], ref["ev"], tol["ev"], "virial estimator (cycle probabilities)")
        # ... then, after a fresh V_B fill, from the recursion solve
        ck(lib.md_pimd_fill_VB_x(s.pimd))
        ck(lib.md_pimd_calc_VBN_energy_x(s.pimd, s.stats))
        assert_close([s.take_energy()], ref["e"], tol["e"], "primitive estimator (recursion)")
        ck(lib.md_pimd_calc_vi_virial_energy_x(s.pimd, s.stats, image))
        assert_close([s.take_energy()], ref["ev"], tol["ev"], "virial estimator (recursion)")
        print(f"N={N} P={P} {kind} xi={vi}: G {relerr(got['G'], ref['G']):.2e} (tol {tol['G']:.1e}), "
              f"f {relerr(got['f'], ref['f']):.2e} (tol {tol['f']:.1e}), "
              f"V_B {relerr(got['VBN'], ref['VBN']):.2e}, tmpV {relerr(got['tmpV'], ref['tmpV']):.2e}")
        # the state has real exchange: cycles of two or more particles
        # (G[l][j], j < l) carry weight
        if vi > 0:
            assert np.tril(ref["G"], -1).max() > 1e-3
    finally:
        s.free()


@pytest.mark.parametrize("N,kind", [(12, "trap"), (100, "ueg"), (160, "trap"), (512, "ueg"), (1024, "trap")])
def test_block_and_cluster_solves_agree(N, kind):
    """The same recursions through each solve kernel, forced, at the same N:
    both match the oracle and each other."""
    P, vi = 16, 0.5
    lib, s, o, beta, image, st, T, box = setup(N, P, vi, kind == "ueg", seed=N + 99)
    ref = oracle_all(st, N, P, T, box, beta, vi, image)
    tol = tolerances(st, N, P, T, box, beta, vi, image, ref)
    out = {}
    try:
        for path in (SOLVE_BLOCK, SOLVE_CLUSTER):
            lib.check(lib.md_gb300_set_solve_path_x(path))
            assert lib.md_gb300_get_solve_path_x(N) == path
            out[path] = exchange_on_gpu(lib, s, image)
            compare(out[path], ref, tol, f"solve path {path}")
    finally:
        lib.md_gb300_set_solve_path_x(SOLVE_AUTO)
        s.free()
    a, b = out[SOLVE_BLOCK], out[SOLVE_CLUSTER]
    for k in ("VBN", "tmpV"):
        assert_elementwise(a[k], b[k], 1e-13, f"block vs cluster {k}")
    assert_close(a["G"], b["G"], max(1e-13, tol["G"] / DRIFT_FACTOR), "block vs cluster G")


def extended_precision_G(ENk, N, beta, vi):
    """V_B, tmpV and G by the reference's recursions (md_pimd_x.c:814-953,
    :2588-2673) in numpy's long double (64 or 113 mantissa bits), from the
    same ENk: a reference for G accurate to well below the FP64 rounding of
    the exponent."""
    LD = np.longdouble
    b = LD(beta)
    lv = np.log(LD(vi)) if vi > 0 else LD(0)
    tri = lambda l: l * (l - 1) // 2  # noqa: E731
    E = ENk.astype(LD)

    def lse(a):
        m = a.max()
        return m + np.log(np.exp(a - m).sum())

    V = np.zeros(N + 1, dtype=LD)
    for n in range(1, N + 1):
        k = np.arange(1, n + 1)
        a = -b * (E[tri(n) + k - 1] + V[n - k]) + (k - 1) * lv - np.log(LD(n))
        if vi == 0:
            a = np.where(k == 1, a, -np.inf)
        V[n] = -lse(a) / b
    tv = np.zeros(N + 1, dtype=LD)
    for u in range(N, 0, -1):
        l = np.arange(u, N + 1)
        k = l - u + 1
        a = -b * (E[l * (l - 1) // 2 + k - 1] + tv[l]) + (k - 1) * lv - np.log(l.astype(LD))
        if vi == 0:
            a = np.where(k == 1, a, -np.inf)
        tv[u - 1] = -lse(a) / b
    G = np.zeros((N, N), dtype=LD)
    for l in range(1, N + 1):
        j = np.arange(1, l + 1)
        a = -b * (V[j - 1] + E[tri(l) + l - j] + tv[l] - V[N]) + (l - j) * lv
        if vi == 0:
            a = np.where(j == l, a, -np.inf)
        G[l - 1, :l] = np.exp(a) / l
        if l < N:
            G[l - 1, l] = 1 - np.exp(-b * (V[l] + tv[l] - V[N]))
    return G.astype(np.float64)


@pytest.mark.parametrize("N,P,kind,vi", [(512, 64, "ueg", 0.5), (1024, 64, "trap", 1.0), (2048, 64, "ueg", 0.5)])
def test_connection_probabilities_against_extended_precision(N, P, kind, vi):
    """G from the extended-range solve is closer to an extended-precision
    evaluation of the reference's own formula than the reference's FP64
    evaluation is: the differences above 1e-10 between this library and the
    reference at these sizes are the reference's rounding."""
    if np.finfo(np.longdouble).eps > 1e-18:
        pytest.skip("long double is not wider than double here")
    lib, s, o, beta, image, st, T, box = setup(N, P, vi, kind == "ueg", seed=N * 7 + P + int(10 * vi))
    try:
        got = exchange_on_gpu(lib, s, image)
    finally:
        s.free()
    ref = oracle_all(st, N, P, T, box, beta, vi, image)
    exact = extended_precision_G(ref["ENk"], N, beta, vi)
    e_gpu, e_ref = relerr(got["G"], exact), relerr(ref["G"], exact)
    print(f"N={N} P={P} {kind} xi={vi}: G against extended precision: this library {e_gpu:.2e}, "
          f"the reference's formula in FP64 {e_ref:.2e}")
    assert e_gpu <= 5e-11
    assert e_gpu <= 0.2 * e_ref


def test_solve_autotuner_records_its_choice():
    N, P, vi = 384, 8, 1.0
    lib, s, o, beta, image, st, T, box = setup(N, P, vi, False, seed=5)
    try:
        lib.check(lib.md_pimd_fast_fill_ENk_x(s.pimd, image))
        path = xmd_x.C.c_int()
        ms = xmd_x.C.c_double()
        lib.check(lib.md_gb300_autotune_solve_x(s.pimd, 5, xmd_x.C.byref(path), xmd_x.C.byref(ms)))
        assert path.value in (SOLVE_BLOCK, SOLVE_CLUSTER) and ms.value > 0
        assert lib.md_gb300_get_solve_path_x(N) == path.value
        ref = oracle_all(st, N, P, T, box, beta, vi, image)
        compare(exchange_on_gpu(lib, s, image), ref, tolerances(st, N, P, T, box, beta, vi, image, ref),
                "after autotuning")
    finally:
        s.free()
