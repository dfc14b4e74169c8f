"""Reader for the golden fixtures written by tests/golden/make_golden.c.

A fixture is a sequence of records ``char name[32]; int64 count;
double data[count]`` produced by running MD-Lab's own _nocl build.
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

HDR_PIMD = ["D", "L", "N", "P", "f", "fc", "vi", "beta", "omegaP", "T", "box", "dt",
            "image", "pbc", "ueg", "g", "s", "alpha", "nsum", "steps", "every"]
HDR_CUBIC = ["D", "L", "N", "P", "vi", "beta", "omegaP", "image", "box"]
HDR_TWO = ["D", "L", "N", "Nb", "P", "vi", "beta", "omegaP", "T", "box", "dt", "image", "pbc",
           "ueg", "g", "s", "alpha", "nsum", "steps", "mb"]


def load(name):
    """Return {record name: float64 array} for tests/golden/<name>.bin."""
    path = os.path.join(HERE, name if name.endswith(".bin") else name + ".bin")
    out = {}
    with open(path, "rb") as fh:
        raw = fh.read()
    pos = 0
    while pos < len(raw):
        nm = raw[pos:pos + 32].split(b"\0", 1)[0].decode()
        cnt = int(np.frombuffer(raw, dtype="<i8", count=1, offset=pos + 32)[0])
        pos += 40
        out[nm] = np.frombuffer(raw, dtype="<f8", count=cnt, offset=pos).copy()
        pos += 8 * cnt
    return out


def header(fx, kind="pimd"):
    keys = {"pimd": HDR_PIMD, "cubic": HDR_CUBIC, "two": HDR_TWO}[kind]
    h = fx["hdr"]
    out = {}
    for k, v in zip(keys, h):
        out[k] = int(v) if k in ("D", "L", "N", "Nb", "P", "f", "fc", "image", "pbc", "ueg",
                                 "nsum", "steps", "every") else float(v)
    return out


PIMD_FIXTURES = ["d2l4_cfg1", "d3l4_trap_vi1", "d3l4_trap_vi05", "d3l4_trap_vi0",
                 "d3l4_trap_n37p6", "d3l4_trap_p2", "d3l4_trap_n1", "d3l4_trap_chain3",
                 "d3l4_ueg", "d3l8_trap"]
CUBIC_FIXTURES = ["d3l4_cubic", "d3l4_cubic_img"]
TWO_FIXTURES = ["d3l4_two_ueg", "d3l4_two_trap", "d2l4_two_trap"]
