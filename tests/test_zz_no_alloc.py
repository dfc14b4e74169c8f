"""The allocation-free pair-force entry point, md_gb300_pair_force_noalloc_x.

It exists for callers that cannot let the library allocate device memory
(an application whose own allocator owns the GPU's memory, or a plugin that
must keep the process's footprint fixed): it works on the caller's device
buffers and uses a fixed array inside the library for its scratch.  Its
results must equal those of the ordinary entry point md_pimd_calc_pair_force_x
on the same configuration, call after call, since consecutive calls share
and reuse that array.

This file is collected last so that a stop-at-first-failure run has already
run every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import xmd_x
from gpu_common import PARITY, random_state
from helpers import assert_close

pytestmark = pytest.mark.gpu


def _soa(a, N, P, D, ld):
    """bead-major host array [(l*P + j)*D + d] -> slice-major [j][d][l] with leading dim ld"""
    out = np.zeros((P, D, ld))
    out[:, :, :N] = np.asarray(a).reshape(N, P, D).transpose(1, 2, 0)
    return out


@pytest.mark.parametrize("kind", ["md_gaussian_force_x", "md_coulomb_periodic_force_x"])
def test_noalloc_pair_force_matches_ordinary_entry_point(kind):
    torch = pytest.importorskip("torch")
    D, L, N, P, ld = 3, 4, 100, 8, 104
    lib = xmd_x.load(D, L)
    box = 6.0
    st = random_state(D, L, N, P, 0.5, box, True, seed=77)
    s = xmd_x.PimdSystem(lib, N, P, 1.0, 0.5, box=box)
    s.set_state(**st)
    xmd_x.set_potentials(lib, gauss_g=0.75 * np.pi, gauss_s=0.5, coul_s=1.0)
    pf = lib.fn(kind)
    # the ordinary entry point, on the library's own device copy
    lib.check(lib.md_reset_force_x(s.sim))
    lib.check(lib.md_pimd_calc_pair_force_x(s.pimd, pf))
    ref = _soa(s.state()["f"], N, P, D, ld)
    s.free()
    # the allocation-free entry point, on buffers the caller owns
    dev = torch.device("cuda", 0)
    x = torch.tensor(_soa(st["x"], N, P, D, ld), dtype=torch.float64, device=dev)
    m = torch.ones((P, ld), dtype=torch.float64, device=dev)
    f = torch.zeros((P, D, ld), dtype=torch.float64, device=dev)
    Lh = np.full(D, box)
    stream = torch.cuda.current_stream(dev)
    for call in range(2):
        f.zero_()
        rc = lib.md_gb300_pair_force_noalloc_x(pf, x.data_ptr(), m.data_ptr(), f.data_ptr(), N, P, ld,
                                               Lh.ctypes.data_as(xmd_x._dp), stream.cuda_stream)
        assert rc == 0, lib.err()
        stream.synchronize()
        got = f.cpu().numpy()
        assert_close(got[:, :, :N], ref[:, :, :N], PARITY, f"{kind}, call {call + 1}")


def test_noalloc_refuses_configurations_beyond_its_fixed_scratch():
    lib = xmd_x.load(3, 4)
    pf = lib.fn("md_gaussian_force_x")
    dummy = C.c_void_p(1 << 20)  # never dereferenced: the size check comes first
    rc = lib.md_gb300_pair_force_noalloc_x(pf, dummy, dummy, dummy, 1024, 64, 1024, None, None)
    assert rc == -1005
    assert "fixed" in lib.err()
