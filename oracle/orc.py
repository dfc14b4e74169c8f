"""ctypes front end of the oracle (oracle/xmd_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product.  ``OrcSim`` wraps numpy
arrays in the reference's own bead-major order; see xmd_oracle.h.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

TRAP_HARMONIC, TRAP_HARMONIC_2, TRAP_NEG_HARMONIC = 1, 2, 3
PAIR_GAUSSIAN, PAIR_PERIODIC_GAUSSIAN, PAIR_COULOMB, PAIR_PERIODIC_COULOMB, PAIR_EWALD = 1, 2, 3, 4, 5

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class _Sim(C.Structure):
    _fields_ = [("D", C.c_int), ("L", C.c_int), ("nb", C.c_int), ("m", _dp), ("x", _dp),
                ("v", _dp), ("f", _dp), ("nf", C.c_int), ("cf", _ip), ("theta", _dp),
                ("vtheta", _dp), ("Q", _dp), ("T", C.c_double), ("box", C.c_double * 3)]


class Params(C.Structure):
    _fields_ = [("trap_w", C.c_double), ("trap_w2", C.c_double * 3), ("trap_c", C.c_double * 3),
                ("gauss_g", C.c_double), ("gauss_s", C.c_double), ("coul_s", C.c_double),
                ("coul_alpha", C.c_double), ("coul_nsum", C.c_int)]


class StepCfg(C.Structure):
    _fields_ = [("N", C.c_int), ("P", C.c_int), ("beta", C.c_double), ("vi", C.c_double),
                ("omegaP", C.c_double), ("image", C.c_int), ("trap_kind", C.c_int),
                ("pair_kind", C.c_int), ("pbc", C.c_int), ("prm", Params)]


def build():
    """Compile liborc.so with oracle/Makefile (gcc only)."""
    subprocess.run(["make", "-s", "-C", HERE, "liborc.so"], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liborc.so")
        srcs = [os.path.join(HERE, f) for f in ("xmd_oracle.c", "xmd_oracle.h", "orc_learned.c")]
        if not os.path.exists(path) or any(os.path.getmtime(path) < os.path.getmtime(f) for f in srcs):
            build()
        L = C.CDLL(path)
        d, i, vp = C.c_double, C.c_int, C.c_void_p
        sig = {
            "orc_minimum_image": (d, [d, d]),
            "orc_reset_force": (None, [vp]),
            "orc_nhc_vv3_1": (i, [vp, d]),
            "orc_nhc_vv3_2": (i, [vp, d]),
            "orc_periodic_boundary": (None, [vp]),
            "orc_fast_fill_ENk": (i, [vp, i, i, d, i, _dp, _dp]),
            "orc_fill_ENk_cubic": (i, [vp, i, i, d, i, _dp]),
            "orc_fill_VB": (i, [i, d, d, _dp, _dp]),
            "orc_fast_force_VB": (i, [vp, i, i, d, d, d, i, _dp, _dp, _dp, _dp]),
            "orc_force_VB_cubic": (i, [vp, i, i, d, d, d, i, _dp, _dp]),
            "orc_trap_force": (i, [vp, i, i, i, vp]),
            "orc_pair_force": (i, [vp, i, i, i, vp]),
            "orc_pair_force_one": (None, [i, vp, i, _dp, _dp, _dp, _dp, d]),
            "orc_pair_force_2": (i, [vp, i, vp, i, i, i, vp]),
            "orc_pair_energy_2": (d, [vp, i, vp, i, i, i, vp]),
            "orc_vbn_energy": (d, [i, i, i, d, d, _dp, _dp]),
            "orc_fast_fill_ENk2": (i, [vp, i, i, d, i, _dp]),
            "orc_fill_ENk2_cubic": (i, [vp, i, i, d, i, _dp]),
            "orc_vi_virial_energy": (d, [vp, i, i, d, d, i, _dp, _dp, _dp]),
            "orc_trap_energy": (d, [vp, i, i, i, vp]),
            "orc_pair_energy": (d, [vp, i, i, i, vp]),
            "orc_pair_energy_one": (d, [i, vp, i, _dp, _dp, _dp]),
            "orc_madelung": (d, [_dp, vp]),
            "orc_virial_energy": (d, [vp, i, i]),
            "orc_centroid_virial_energy": (d, [vp, i, i, d, i]),
            "orc_polymer_periodic_boundary": (None, [vp, i, i]),
            "orc_pair_correlation": (None, [vp, i, i, i, d, d, i, i, _dp]),
            "orc_vi_sign": (d, [i, d, d, d, _dp, _dp]),
            "orc_step": (i, [vp, vp, d, _dp, _dp, _dp]),
            "orc_set_seed": (None, [C.c_uint]),
            "orc_random_uniform": (d, [d, d]),
            "orc_random_gaussian": (d, []),
            "orc_mlp_nparam": (i, []),
            "orc_bf16": (d, [d]),
            "orc_desc_features": (None, [i, _dp, _dp, d, i, _dp, _dp, _dp, _dp, _dp]),
            "orc_mlp_forward": (None, [i, _dp, _dp, i, _dp, _dp, _dp]),
            "orc_mlp_loss": (d, [i, _dp, _dp, _dp, _dp, d, d, d, i]),
            "orc_mlp_grad": (None, [i, _dp, _dp, _dp, _dp, d, d, d, i, _dp, _dp]),
            "orc_sk_sphere": (i, [d, d, d, i, _dp, _dp]),
            "orc_sk_structure": (None, [i, i, _dp, i, i, _dp, _dp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def ptr(a, ct=C.c_double):
    return a.ctypes.data_as(C.POINTER(ct))


def ntri(n):
    return n * (n + 1) // 2


class OrcSim:
    """Simulation state held in numpy arrays, shared with the C oracle."""

    def __init__(self, D, L, nb, m, x, v, f, cf, theta, vtheta, Q, T, box):
        self.D, self.L, self.nb = D, L, nb
        self.m = np.ascontiguousarray(m, dtype=np.float64).copy()
        self.x = np.ascontiguousarray(x, dtype=np.float64).copy()
        self.v = np.ascontiguousarray(v, dtype=np.float64).copy()
        self.f = np.ascontiguousarray(f, dtype=np.float64).copy()
        self.cf = np.ascontiguousarray(cf, dtype=np.int32).copy()
        self.theta = np.ascontiguousarray(theta, dtype=np.float64).copy()
        self.vtheta = np.ascontiguousarray(vtheta, dtype=np.float64).copy()
        self.Q = np.ascontiguousarray(Q, dtype=np.float64).copy()
        self.s = _Sim(D, L, nb, ptr(self.m), ptr(self.x), ptr(self.v), ptr(self.f),
                      len(self.cf), ptr(self.cf, C.c_int), ptr(self.theta), ptr(self.vtheta),
                      ptr(self.Q), float(T), (C.c_double * 3)(*(list(box) + [0.0] * 3)[:3]))

    @property
    def ref(self):
        return C.byref(self.s)

    @classmethod
    def from_fixture(cls, fx, prefix="init/"):
        from_h = fx["hdr"]
        D, L, N, P = int(from_h[0]), int(from_h[1]), int(from_h[2]), int(from_h[3])
        T, box = from_h[9], from_h[10]
        return cls(D, L, N * P, fx["m"], fx[prefix + "x"], fx[prefix + "v"], fx[prefix + "f"],
                   fx[prefix + "cf"], fx[prefix + "theta"], fx[prefix + "vtheta"], fx[prefix + "Q"],
                   T, [box] * 3)


def two_from_fixture(fx, prefix="init/"):
    """The two species' states ("a/" and "b/" records) of a two-species fixture."""
    h = fx["hdr"]
    D, L, Na, Nb, P = (int(v) for v in h[:5])
    T, box, mb = h[8], h[9], h[19]
    out = []
    for sp, N, m in (("a/", Na, 1.0), ("b/", Nb, mb)):
        q = sp + prefix
        out.append(OrcSim(D, L, N * P, np.full(N * P, m), fx[q + "x"], fx[q + "v"], fx[q + "f"], fx[q + "cf"],
                          fx[q + "theta"], fx[q + "vtheta"], fx[q + "Q"], T, [box] * 3))
    return out


def pair_force_2(a, Na, b, Nb, P, kind, prm):
    """Cross-species pair forces added into a.f and b.f (md_pimd_calc_pair_force_2_x)."""
    assert lib().orc_pair_force_2(a.ref, Na, b.ref, Nb, P, kind, C.byref(prm)) == 0


def pair_energy_2(a, Na, b, Nb, P, kind, prm):
    return lib().orc_pair_energy_2(a.ref, Na, b.ref, Nb, P, kind, C.byref(prm))


def two_species_forces(a, b, Na, Nb, P, beta, vi, omegaP, image, trap, pair, prm):
    """Forces of a two-species step in the order a driver calls the reference:
    each species' exchange, trap and pair forces, then the cross term."""
    L = lib()
    for s, N in ((a, Na), (b, Nb)):
        L.orc_reset_force(s.ref)
        ENk, _ = fast_fill_ENk(s, N, P, omegaP, image)
        VBN = fill_VB(N, beta, vi, ENk)
        fast_force_VB(s, N, P, beta, vi, omegaP, image, ENk, VBN)
        if trap:
            L.orc_trap_force(s.ref, N, P, trap, C.byref(prm))
        L.orc_pair_force(s.ref, N, P, pair, C.byref(prm))
    pair_force_2(a, Na, b, Nb, P, pair, prm)


def two_species_step(a, b, Na, Nb, P, beta, vi, omegaP, image, trap, pair, prm, dt, pbc):
    L = lib()
    assert L.orc_nhc_vv3_1(a.ref, dt) == 0 and L.orc_nhc_vv3_1(b.ref, dt) == 0
    two_species_forces(a, b, Na, Nb, P, beta, vi, omegaP, image, trap, pair, prm)
    assert L.orc_nhc_vv3_2(a.ref, dt) == 0 and L.orc_nhc_vv3_2(b.ref, dt) == 0
    if pbc:
        L.orc_periodic_boundary(a.ref)
        L.orc_periodic_boundary(b.ref)


def params(trap_w=1.0, trap_c=(0, 0, 0), trap_w2=(1, 1, 1), gauss_g=0.0, gauss_s=1.0,
           coul_s=1.0, coul_alpha=1.0, coul_nsum=1):
    return Params(trap_w, (C.c_double * 3)(*trap_w2), (C.c_double * 3)(*trap_c), gauss_g,
                  gauss_s, coul_s, coul_alpha, coul_nsum)


def fast_fill_ENk(sim, N, P, omegaP, image):
    ENk = np.zeros(ntri(N))
    Eint = np.zeros(N)
    lib().orc_fast_fill_ENk(sim.ref, N, P, omegaP, image, ptr(ENk), ptr(Eint))
    return ENk, Eint


def fill_VB(N, beta, vi, ENk):
    VBN = np.zeros(N + 1)
    lib().orc_fill_VB(N, beta, vi, ptr(np.ascontiguousarray(ENk)), ptr(VBN))
    return VBN


def fast_force_VB(sim, N, P, beta, vi, omegaP, image, ENk, VBN):
    G = np.zeros(N * N)
    tmpV = np.zeros(N + 1)
    rc = lib().orc_fast_force_VB(sim.ref, N, P, beta, vi, omegaP, image,
                                 ptr(np.ascontiguousarray(ENk)), ptr(np.ascontiguousarray(VBN)),
                                 ptr(G), ptr(tmpV))
    assert rc == 0
    return G.reshape(N, N), tmpV


# ---- learned residual (orc_learned.c) ----
def mlp_forward(X, p, bf=1):
    X = np.ascontiguousarray(X, np.float64)
    p = np.ascontiguousarray(p, np.float64)
    Y = np.zeros((X.shape[0], 4))
    lib().orc_mlp_forward(X.shape[0], ptr(X), ptr(p), bf, ptr(Y), None, None)
    return Y


def mlp_loss(X, V, T, p, we=1.0, wf=1.0, inv_rows=None, bf=0):
    X, V, T, p = (np.ascontiguousarray(a, np.float64) for a in (X, V, T, p))
    inv = 1.0 / X.shape[0] if inv_rows is None else inv_rows
    return lib().orc_mlp_loss(X.shape[0], ptr(X), ptr(V), ptr(T), ptr(p), we, wf, inv, bf)


def mlp_grad(X, V, T, p, we=1.0, wf=1.0, inv_rows=None, bf=0):
    X, V, T, p = (np.ascontiguousarray(a, np.float64) for a in (X, V, T, p))
    inv = 1.0 / X.shape[0] if inv_rows is None else inv_rows
    g = np.zeros(lib().orc_mlp_nparam())
    loss = np.zeros(2)
    lib().orc_mlp_grad(X.shape[0], ptr(X), ptr(V), ptr(T), ptr(p), we, wf, inv, bf, ptr(g), ptr(loss))
    return g, loss


def desc_features(x, box, rc, basis, vmu, vsig, nb=64):
    """x: positions [N][3] of one bead slice"""
    x = np.ascontiguousarray(x, np.float64)
    N = x.shape[0]
    L = np.ascontiguousarray(box, np.float64)
    B = np.ascontiguousarray(basis, np.float64)
    mu = np.ascontiguousarray(vmu, np.float64)
    sg = np.ascontiguousarray(vsig, np.float64)
    F = np.zeros((N, 64))
    V = np.zeros((N, 9))
    lib().orc_desc_features(N, ptr(x), ptr(L), rc, nb, ptr(B), ptr(mu), ptr(sg), ptr(F), ptr(V))
    return F, V


def sk_sphere(q0, qincre, qmax, max_n=4096):
    qs = np.zeros(max_n)
    qis = np.zeros(3 * max_n)
    n = lib().orc_sk_sphere(q0, qincre, qmax, max_n, ptr(qs), ptr(qis))
    return qs[:n].copy(), qis[:3 * n].reshape(n, 3).copy()


def sk_structure(N, P, x, pi, qis):
    x = np.ascontiguousarray(x, np.float64)
    q = np.ascontiguousarray(qis, np.float64).reshape(-1)
    res = np.zeros(len(q) // 3)
    lib().orc_sk_structure(N, P, ptr(x), pi, len(res), ptr(q), ptr(res))
    return res
