"""The key/value-input driver (md-lab_gb300/drivers/xmd_run.c) and the
reader under it, md_read_attr_pair_x (MD-Lab md_util_x.c:95-119), without a
GPU: the driver resolves an input written in the format of MD-Lab's sample
inputs, and refuses to compute when no device is present."""
import ctypes as C
import os
import subprocess

import pytest

import xmd_x

BIN = os.path.join(xmd_x.HERE, "bin")


def driver(D, L):
    p = os.path.join(BIN, f"xmd_run_d{D}l{L}")
    if not os.path.exists(p):
        pytest.fail(f"{p} is missing: build the library first")
    return p


def write_input(tmp_path, text):
    p = tmp_path / "input.txt"
    p.write_text(text)
    return str(p)


def test_reader_parses_key_value_pairs(tmp_path):
    lib = xmd_x.load(3, 4)
    path = write_input(tmp_path, "N 500\nP 72\nT 0.166666667\nomega 1.0\nvi 1.0\ng 0.0\ns 0.5")
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    fh = libc.fopen(path.encode(), b"r")

    class Attr(C.Structure):
        _fields_ = [("N", C.c_int), ("names", C.c_void_p), ("values", C.POINTER(C.c_double))]

    lib.h.md_read_attr_pair_x.restype = C.POINTER(Attr)
    lib.h.md_read_attr_pair_x.argtypes = [C.c_void_p, C.c_void_p]
    lib.h.md_get_attr_value_x.restype = C.c_double
    lib.h.md_get_attr_value_x.argtypes = [C.POINTER(Attr), C.c_char_p, C.POINTER(C.c_int)]
    a = lib.h.md_read_attr_pair_x(fh, None)
    libc.fclose(fh)
    assert a and a.contents.N == 7
    found = C.c_int()
    assert lib.h.md_get_attr_value_x(a, b"P", C.byref(found)) == 72 and found.value == 1
    assert lib.h.md_get_attr_value_x(a, b"T", C.byref(found)) == 0.166666667
    assert lib.h.md_get_attr_value_x(a, b"missing", C.byref(found)) == 0 and found.value == 0


@pytest.mark.parametrize("D,L", [(2, 4), (3, 4), (3, 8)])
def test_driver_resolves_parameters(tmp_path, D, L):
    path = write_input(tmp_path, "N 24\nP 12\nT 0.25\nomega 2.0\nvi 0.5\ng 1.5\ns 0.7\ndt 0.02\nsteps 30\nevery 3\n")
    out = subprocess.run([driver(D, L), path, "--parse-only"], capture_output=True, text=True, check=True).stdout
    got = {ln.split()[1]: float(ln.split()[2]) for ln in out.splitlines() if ln.startswith("param")}
    want = {"N": 24, "P": 12, "D": D, "T": 0.25, "omega": 2.0, "vi": 0.5, "g": 1.5, "s": 0.7, "dt": 0.02,
            "steps": 30, "every": 3, "equil": 1000, "seed": 1, "ueg": 0}
    for k, v in want.items():
        assert got[k] == v, k


def test_driver_electron_gas_parameters(tmp_path):
    path = write_input(tmp_path, "N 128\nP 32\nueg 1\nrs 2\ntheta 0.5\nnsum 8\nvi 0.6\n")
    out = subprocess.run([driver(3, 4), path, "--parse-only"], capture_output=True, text=True, check=True).stdout
    got = {ln.split()[1]: float(ln.split()[2]) for ln in out.splitlines() if ln.startswith("param")}
    import math
    box = (4 * math.pi * 128 / 3) ** (1 / 3) * 2
    assert abs(got["L"] - box) < 1e-12 * box
    assert abs(got["T"] - 0.5 * 0.5 * (6 * math.pi ** 2 * 128 / box ** 3) ** (2 / 3)) < 1e-12


def test_driver_rejects_bad_input(tmp_path):
    path = write_input(tmp_path, "N 24\nP\n")
    r = subprocess.run([driver(3, 4), path, "--parse-only"], capture_output=True, text=True)
    assert r.returncode == 1 and "key value" in r.stderr
    r = subprocess.run([driver(3, 4), write_input(tmp_path, "N 4\nP 1\n"), "--parse-only"], capture_output=True,
                       text=True)
    assert r.returncode == 1


def test_driver_fails_loudly_without_a_gpu(tmp_path):
    lib = xmd_x.load(3, 4)
    if lib.md_gb300_device_count_x() > 0:
        pytest.skip("a GPU is present")
    r = subprocess.run([driver(3, 4), write_input(tmp_path, "N 8\nP 4\nsteps 2\nequil 0\n")], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "no CUDA device" in r.stderr
