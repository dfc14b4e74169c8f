"""Text checkpoints: the reference's "%f" format by default, and the exact
"%.17g" form (md_gb300_set_text_exact_x) with which a resumed run continues
bit for bit.  Host-only: runs without a GPU."""
import ctypes as C
import os

import numpy as np

import xmd_x


def _libc():
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    return libc


def _roundtrip(lib, s, path, exact):
    libc = _libc()
    lib.md_gb300_set_text_exact_x(exact)
    try:
        f = libc.fopen(path.encode(), b"w")
        assert lib.h.md_fprint_particle_pos_x(C.c_void_p(f), s.sim) == 0
        assert lib.h.md_fprint_particle_vel_x(C.c_void_p(f), s.sim) == 0
        assert lib.h.md_fprint_nhcs_x(C.c_void_p(f), s.sim) == 0
        libc.fclose(f)
        before = s.state()
        s.set_state(x=np.zeros_like(before["x"]), v=np.zeros_like(before["v"]),
                    theta=np.zeros_like(before["theta"]), vtheta=np.zeros_like(before["vtheta"]))
        f = libc.fopen(path.encode(), b"r")
        assert lib.h.md_fread_particle_pos_x(C.c_void_p(f), s.sim) == 0
        assert lib.h.md_fread_particle_vel_x(C.c_void_p(f), s.sim) == 0
        assert lib.h.md_fread_nhcs_x(C.c_void_p(f), s.sim) == 0
        libc.fclose(f)
        return before, s.state()
    finally:
        lib.md_gb300_set_text_exact_x(0)


def test_exact_checkpoint_roundtrip(tmp_path):
    lib = xmd_x.load(3, 4)
    for name, argt in (("md_fprint_particle_pos_x", [C.c_void_p, C.c_void_p]),
                       ("md_fprint_particle_vel_x", [C.c_void_p, C.c_void_p]),
                       ("md_fprint_nhcs_x", [C.c_void_p, C.c_void_p]),
                       ("md_fread_particle_pos_x", [C.c_void_p, C.c_void_p]),
                       ("md_fread_particle_vel_x", [C.c_void_p, C.c_void_p]),
                       ("md_fread_nhcs_x", [C.c_void_p, C.c_void_p]),
                       ("md_gb300_set_text_exact_x", [C.c_int])):
        getattr(lib.h, name).argtypes = argt
        getattr(lib.h, name).restype = C.c_int
    rng = np.random.default_rng(3)
    s = xmd_x.PimdSystem(lib, 5, 4, 0.5, 0.7, box=4.0)
    nb = 20
    s.set_state(m=np.ones(nb), x=rng.standard_normal(nb * 3) * np.pi, v=rng.standard_normal(nb * 3) / 3,
                theta=rng.standard_normal(nb * 3 * 4) * 1e-3, vtheta=rng.standard_normal(nb * 3 * 4),
                Q=np.full(nb * 3 * 4, 0.3), cf=np.ones(nb * 3))
    b, a = _roundtrip(lib, s, str(tmp_path / "exact.txt"), 1)
    for k in ("x", "v", "theta", "vtheta"):
        np.testing.assert_array_equal(a[k], b[k])
    b, a = _roundtrip(lib, s, str(tmp_path / "lossy.txt"), 0)
    assert np.abs(a["x"] - b["x"]).max() <= 5e-7 and np.abs(a["x"] - b["x"]).max() > 0
    text = open(tmp_path / "lossy.txt").read().split("\n")[1].split()
    assert all(len(t.split(".")[1]) == 6 for t in text)  # the reference's %f
    s.free()
