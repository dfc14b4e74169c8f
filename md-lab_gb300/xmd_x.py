"""ctypes binding of the MD-Lab C ABI (md_pimd_x.h / md_simulation_x.h).

The same binding drives any library that exports that ABI: the GB300
library built here (``lib/libxmd_x_d<D>l<L>.so``) or MD-Lab's own build.
Struct layouts follow include/md_particle_x.h for a given dimension D and
chain length L.

    lib = load(3, 4)                    # libxmd_x_d3l4.so from lib/
    s = PimdSystem(lib, N=8, P=8, vi=1.0, T=0.25)
    s.set_state(x=..., v=...)           # host state, uploaded on first use
    md_step(lib, s, dt, trap=lib.fn("md_harmonic_trap_force_x"),
            pair=lib.fn("md_gaussian_force_x"))
    s.state()["f"]                      # host copy of the forces

Loading fails loudly if the library has not been built (run
``python -c "import __graft_entry__ as g; g.build()"``): there is no
fallback implementation.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(HERE, "lib")

_d, _i, _vp = C.c_double, C.c_int, C.c_void_p
_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)


def lib_path(D, L):
    return os.path.join(LIBDIR, f"libxmd_x_d{D}l{L}.so")


def structs(D, L):
    """ctypes mirrors of the public structs for one (D, L) variant."""

    class Particle(C.Structure):
        _fields_ = [("m", _d), ("x", _d * D), ("v", _d * D), ("f", _d * D)]

    class Nhc(C.Structure):
        _fields_ = [("f", _i), ("theta", _d * L), ("vtheta", _d * L), ("Q", _d * L)]

    class Box(C.Structure):
        _fields_ = [("type", _i), ("box", _vp)]

    class Rect(C.Structure):
        _fields_ = [("L", _d * D)]

    class Sim(C.Structure):
        _fields_ = [("N", _i), ("particles", C.POINTER(Particle)), ("fc", _i), ("Nf", _i),
                    ("fs", C.POINTER(_i)), ("f0s", C.POINTER(_i)), ("nhcs", C.POINTER(Nhc)),
                    ("box", C.POINTER(Box)), ("T", _d), ("pcount_in", _i), ("pcount_ex", _i),
                    ("pair_in", _vp), ("pair_ex", _vp)]

    class Pimd(C.Structure):
        _fields_ = [("sim", C.POINTER(Sim)), ("N", _i), ("P", _i), ("ENk_count", _i),
                    ("ENk", C.POINTER(_dp)), ("ENk2", C.POINTER(_dp)), ("ENk3", C.POINTER(_dp)),
                    ("VBN", _dp), ("vi", _d), ("omegaP", _d), ("beta", _d), ("pcount_in", _i),
                    ("pcount_ex", _i), ("pair_in", _vp), ("pair_ex", _vp), ("Eindices", _vp),
                    ("minE", _dp), ("cut_Pj", _i), ("Eint", _dp), ("Evir", _dp), ("mc_par", _i),
                    ("pbc", _i), ("pbW", _vp), ("worm_index", _i), ("worm_pos", _d * D),
                    ("old_worm_index", _i), ("old_worm_pos", _d * D)]

    class Stats(C.Structure):
        _fields_ = [("N", _i), ("count", _i), ("e", _d), ("es", _dp), ("T", _d), ("Ts", _dp),
                    ("points", _i), ("fx", _dp), ("fxs", C.POINTER(_dp))]

    return Particle, Nhc, Box, Rect, Sim, Pimd, Stats


class SkSphere(C.Structure):
    _fields_ = [("N", _i), ("qs", _dp), ("qis", _dp)]


class XLib:
    """One loaded library exporting the MD-Lab ABI for dimension D, chain length L."""

    def __init__(self, path, D, L, gb300=True):
        if not os.path.exists(path):
            raise FileNotFoundError(
                f"{path} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        self.path, self.D, self.L, self.gb300 = path, D, L, gb300
        self.h = C.CDLL(path)
        (self.Particle, self.Nhc, self.Box, self.Rect, self.Sim, self.Pimd,
         self.Stats) = structs(D, L)
        ps, pp, pst = C.POINTER(self.Sim), C.POINTER(self.Pimd), C.POINTER(self.Stats)
        sig = {
            "md_set_pimd_mode_x": (None, [_i]),
            "md_set_seed_x": (None, [C.c_uint]),
            "md_random_uniform_x": (_d, [_d, _d]),
            "md_random_gaussian_x": (_d, []),
            "md_get_quick_Q_x": (_d, [_d, _d]),
            "md_alloc_simulation_x": (ps, [_i, _i, _i, _i]),
            "md_init_nd_rect_box_x": (_i, [C.POINTER(self.Box), _dp]),
            "md_alloc_pimd_x": (pp, [ps, _i, _i, _d, _d]),
            "md_init_particle_mass_x": (_i, [ps, _d, _i, _i]),
            "md_init_maxwell_vel_x": (_i, [ps, _d]),
            "md_init_nhc_x": (_i, [ps, _d, _i, _i, _d]),
            "md_pimd_init_particle_uniform_pos_x": (_i, [pp, _dp, _dp, _d]),
            "md_simulation_sync_host_x": (ps, [ps, _i]),
            "md_pimd_sync_host_x": (pp, [pp, _i]),
            "md_stats_sync_host_x": (pst, [pst]),
            "md_alloc_stats_x": (pst, [_i]),
            "md_reset_force_x": (_i, [ps]),
            "md_update_nhc_VV3_1_x": (_i, [ps, _d]),
            "md_update_nhc_VV3_2_x": (_i, [ps, _d]),
            "md_periodic_boundary_x": (_i, [ps]),
            "md_pimd_fast_fill_ENk_x": (_i, [pp, _i]),
            "md_pimd_fill_ENk_x": (_i, [pp, _i]),
            "md_pimd_fill_VB_x": (_i, [pp]),
            "md_pimd_fast_fill_force_VB_x": (_i, [pp, _i]),
            "md_pimd_fill_force_VB_x": (_i, [pp, _i]),
            "md_pimd_calc_trap_force_x": (_i, [pp, _vp]),
            "md_pimd_calc_pair_force_x": (_i, [pp, _vp]),
            "md_pimd_calc_VBN_energy_x": (_i, [pp, pst]),
            "md_pimd_fast_fill_ENk2_x": (_i, [pp, _i]),
            "md_pimd_fill_ENk2_x": (_i, [pp, _i]),
            "md_pimd_calc_vi_virial_energy_x": (_i, [pp, pst, _i]),
            "md_pimd_calc_trap_energy_x": (_i, [pp, _vp, pst]),
            "md_pimd_calc_pair_energy_x": (_i, [pp, _vp, pst]),
            "md_pimd_calc_pair_force_2_x": (_i, [pp, pp, _vp]),
            "md_pimd_calc_pair_energy_2_x": (_i, [pp, pp, _vp, pst]),
            "md_pimd_calc_vi_sign_x": (_i, [pp, pst, pst, _d]),
            "md_pimd_calc_virial_energy_x": (_i, [pp, pst]),
            "md_pimd_calc_centroid_virial_energy_x": (_i, [pp, pst, _i]),
            "md_pimd_polymer_periodic_boundary_x": (_i, [pp]),
            "md_pimd_calc_pair_correlation_x": (_i, [pp, pst, _d, _d, _i, _i]),
            "md_reset_stats_f_x": (_i, [pst, _d]),
            "md_stats_add_to_f_x": (_i, [pst, pst]),
            "md_stats_copy_to_f_x": (_i, [pst, pst]),
            "md_stats_mult_to_f_x": (_i, [pst, pst]),
            "md_calc_3d_ueg_madelung_x": (_d, [_dp]),
            "md_set_harmonic_trap_frequency_x": (None, [_d]),
            "md_set_harmonic_trap_center_x": (None, [_dp]),
            "md_set_gaussian_force_strength_x": (None, [_d]),
            "md_set_guassian_force_range_x": (None, [_d]),
            "md_set_coulomb_force_strength_x": (None, [_d]),
            "md_set_coulomb_truc_x": (None, [_d]),
            "md_set_coulomb_n_sum_x": (None, [_i]),
            "md_reset_stats_x": (_i, [pst, _d]),
            "md_alloc_sk_sphere_3d_x": (C.POINTER(SkSphere), [_d, _d, _d]),
            "md_pimd_calc_sphere_Sk_structure_x": (_i, [pp, pst, _i, C.POINTER(SkSphere)]),
        }
        if gb300:
            sig.update({
                "md_gb300_last_error_x": (C.c_char_p, []),
                "md_gb300_device_count_x": (_i, []),
                "md_gb300_launch_count_x": (C.c_ulonglong, []),
                "md_gb300_synchronize_x": (_i, []),
                "md_gb300_capture_begin_x": (_i, []),
                "md_gb300_capture_end_x": (_i, [C.POINTER(_vp)]),
                "md_gb300_graph_launch_x": (_i, [_vp, _i]),
                "md_gb300_graph_kernel_count_x": (_i, [_vp]),
                "md_gb300_graph_free_x": (None, [_vp]),
                "md_gb300_free_simulation_x": (None, [ps]),
                "md_gb300_free_pimd_x": (None, [pp]),
                "md_gb300_free_stats_x": (None, [pst]),
                "md_gb300_variant_x": (None, [C.POINTER(_i), C.POINTER(_i)]),
                "md_gb300_get_stream_x": (_vp, []),
                "md_gb300_profile_x": (_i, [_i]),
                "md_gb300_profile_report_x": (_i, [C.c_char_p, _i]),
                "md_gb300_fp64_peak_x": (_d, []),
                "md_gb300_fp32_peak_x": (_d, []),
                "md_gb300_set_device_x": (_i, [_i]),
                "md_gb300_set_precision_x": (_i, [_i]),
                "md_gb300_get_precision_x": (_i, []),
                "md_gb300_pair_force_noalloc_x": (_i, [_vp, _vp, _vp, _vp, _i, _i, _i, _dp, _vp]),
                "md_gb300_tc_selftest_x": (_i, [_dp]),
                "md_gb300_set_wait_limit_x": (_i, [C.c_longlong]),
                "md_gb300_get_wait_limit_x": (C.c_longlong, []),
                "md_gb300_wait_selftest_x": (_i, [C.c_longlong, C.POINTER(_i), C.POINTER(C.c_longlong)]),
                "md_gb300_autotune_pair_x": (_i, [pp, _vp, _i, C.POINTER(_i), _dp]),
                "md_gb300_set_pair_tile_x": (_i, [_vp, _i, _i, _i]),
                "md_gb300_set_solve_path_x": (_i, [_i]),
                "md_gb300_autotune_fp64_x": (_i, [pp, _vp, _i, C.POINTER(_i), C.POINTER(_i), _dp]),
                "md_gb300_get_solve_path_x": (_i, [_i]),
                "md_gb300_autotune_solve_x": (_i, [pp, _i, C.POINTER(_i), _dp]),
                "md_gb300_exchange_tables_x": (_i, [pp, _dp, _dp]),
                "md_gb300_capture_ensemble_x": (_i, [_i, _vp, _vp, C.POINTER(_vp)]),
                "md_gb300_capture_ensemble_persistent_x": (_i, [_i, _vp, _vp, C.POINTER(_vp)]),
                "md_gb300_autotune_ensemble_x": (_i, [_i, _vp, _vp, _i, C.POINTER(_i), C.POINTER(_i), _dp]),
                "md_gb300_ensemble_status_x": (_i, [_vp]),
                "md_gb300_ensemble_phase_times_x": (_i, [_vp, _dp, _i]),
                "md_gb300_ewald_model_nparam_x": (_i, []),
                "md_gb300_ewald_model_create_x": (_i, [C.POINTER(_vp), pp, _i, C.c_long, C.c_uint]),
                "md_gb300_ewald_model_free_x": (None, [_vp]),
                "md_gb300_ewald_model_collect_x": (_i, [_vp, pp]),
                "md_gb300_ewald_model_train_x": (_i, [_vp, _i, _i, _d, _dp]),
                "md_gb300_ewald_model_attach_x": (_i, [pp, _vp, _i, _d, _d]),
                "md_gb300_ewald_model_judge_x": (_i, [_vp, pp, _dp]),
                "md_gb300_ewald_model_status_x": (_i, [_vp, C.POINTER(C.c_long), C.POINTER(_i), C.POINTER(_i), _dp]),
                "md_gb300_ewald_model_params_x": (_i, [_vp, _fp, _i]),
                "md_gb300_mlp_forward_x": (_i, [_vp, _fp, _i, _fp]),
                "md_gb300_mlp_grad_x": (_i, [_vp, _fp, _fp, _fp, _i, _d, _d, _fp, _fp]),
                "md_gb300_ewald_model_features_x": (_i, [_vp, pp, _fp, _fp]),
                "md_gb300_ewald_model_desc_info_x": (_i, [_vp, _dp, _fp, _dp, _dp]),
            })
        for name, (res, args) in sig.items():
            fn = getattr(self.h, name)
            fn.restype = res
            fn.argtypes = args

    def __getattr__(self, name):
        return getattr(self.h, name)

    def fn(self, name):
        """Address of an exported function (potentials are passed by pointer)."""
        return C.cast(getattr(self.h, name), _vp).value

    def err(self):
        return self.h.md_gb300_last_error_x().decode() if self.gb300 else ""

    def check(self, rc, what=""):
        if rc != 0:
            raise RuntimeError(f"{what} failed with {rc}: {self.err()}")
        return rc

    def profile_report(self):
        """{kernel: (total_ms, launches)} recorded since the last report."""
        buf = C.create_string_buffer(1 << 16)
        self.h.md_gb300_profile_report_x(buf, len(buf))
        out = {}
        for item in buf.value.decode().split(";"):
            if item.strip():
                name, ms, n = item.split()
                out[name] = (float(ms), int(n))
        return out

    def global_double(self, name):
        return C.c_double.in_dll(self.h, name).value


def load(D=3, L=4):
    return XLib(lib_path(D, L), D, L, gb300=True)


class PimdSystem:
    """A ring-polymer system allocated through the library's own ABI."""

    def __init__(self, lib, N, P, vi, T, box=10.0, f=1, fc=0, pimd_mode=1):
        self.lib, self.N, self.P = lib, N, P
        lib.md_set_pimd_mode_x(pimd_mode)
        self.sim = lib.md_alloc_simulation_x(N * P, f, fc, 0)
        if not self.sim:
            raise MemoryError("md_alloc_simulation_x failed")
        self.box = np.full(lib.D, float(box))
        lib.md_init_nd_rect_box_x(self.sim.contents.box, self.box.ctypes.data_as(_dp))
        self.pimd = lib.md_alloc_pimd_x(self.sim, N, P, vi, T)
        if not self.pimd:
            raise MemoryError("md_alloc_pimd_x failed")
        self.stats = lib.md_alloc_stats_x(1)

    # ---- host views (valid after a host sync) ----
    @property
    def nb(self):
        return self.N * self.P

    def _particles(self):
        D = self.lib.D
        n = self.nb * (1 + 3 * D)
        buf = C.cast(self.sim.contents.particles, C.POINTER(C.c_double * n)).contents
        return np.frombuffer(buf, dtype=np.float64).reshape(self.nb, 1 + 3 * D)

    def _chains(self):
        L = self.lib.L
        dt = np.dtype([("f", "<i4"), ("pad", "<i4"), ("theta", "<f8", L), ("vtheta", "<f8", L),
                       ("Q", "<f8", L)])
        assert dt.itemsize == C.sizeof(self.lib.Nhc)
        nf = self.sim.contents.Nf
        buf = C.cast(self.sim.contents.nhcs, C.POINTER(C.c_char * (dt.itemsize * nf))).contents
        return np.frombuffer(buf, dtype=dt)

    def state(self):
        """Copy of x, v, f, m and the chains (syncs the host, device keeps authority)."""
        lib = self.lib
        if not lib.md_simulation_sync_host_x(self.sim, 1):
            raise RuntimeError("sync failed: " + lib.err())
        D = lib.D
        p = self._particles().copy()
        c = self._chains().copy()
        return {"m": p[:, 0].copy(), "x": p[:, 1:1 + D].ravel().copy(),
                "v": p[:, 1 + D:1 + 2 * D].ravel().copy(), "f": p[:, 1 + 2 * D:].ravel().copy(),
                "theta": c["theta"].ravel().copy(), "vtheta": c["vtheta"].ravel().copy(),
                "Q": c["Q"].ravel().copy(), "cf": c["f"].astype(np.float64)}

    def set_state(self, m=None, x=None, v=None, f=None, theta=None, vtheta=None, Q=None, cf=None):
        """Write host state; the next device call uploads it."""
        lib = self.lib
        if not lib.md_simulation_sync_host_x(self.sim, 0):
            raise RuntimeError("sync failed: " + lib.err())
        D = lib.D
        p = self._particles()
        if m is not None:
            p[:, 0] = m
        if x is not None:
            p[:, 1:1 + D] = np.asarray(x).reshape(self.nb, D)
        if v is not None:
            p[:, 1 + D:1 + 2 * D] = np.asarray(v).reshape(self.nb, D)
        if f is not None:
            p[:, 1 + 2 * D:] = np.asarray(f).reshape(self.nb, D)
        c = self._chains()
        nf = len(c)
        if theta is not None:
            c["theta"][:] = np.asarray(theta).reshape(nf, -1)
        if vtheta is not None:
            c["vtheta"][:] = np.asarray(vtheta).reshape(nf, -1)
        if Q is not None:
            c["Q"][:] = np.asarray(Q).reshape(nf, -1)
        if cf is not None:
            c["f"][:] = np.asarray(cf).astype(np.int32)

    def exchange(self):
        """ENk (triangle), Eint, VBN, ENk2 after a host sync."""
        lib = self.lib
        if not lib.md_pimd_sync_host_x(self.pimd, 1):
            raise RuntimeError("sync failed: " + lib.err())
        pc = self.pimd.contents
        nt = pc.ENk_count
        return {"ENk": np.ctypeslib.as_array(pc.ENk[0], (nt,)).copy(),
                "ENk2": np.ctypeslib.as_array(pc.ENk2[0], (nt,)).copy(),
                "Eint": np.ctypeslib.as_array(pc.Eint, (self.N,)).copy(),
                "VBN": np.ctypeslib.as_array(pc.VBN, (self.N + 1,)).copy()}

    def take_energy(self):
        """Value accumulated in the statistics object since the last take."""
        lib = self.lib
        st = lib.md_stats_sync_host_x(self.stats)
        if not st:
            raise RuntimeError("stats sync failed: " + lib.err())
        e = self.stats.contents.es[0]
        self.stats.contents.es[0] = 0.0
        return e

    def free(self):
        if self.lib.gb300:
            self.lib.md_gb300_free_stats_x(self.stats)
            self.lib.md_gb300_free_pimd_x(self.pimd)
            self.lib.md_gb300_free_simulation_x(self.sim)
            self.sim = self.pimd = self.stats = None


def set_potentials(lib, trap_w=1.0, center=None, gauss_g=0.0, gauss_s=1.0, coul_s=1.0,
                   alpha=1.0, nsum=1):
    c = np.zeros(lib.D) if center is None else np.asarray(center, dtype=np.float64)
    lib.md_set_harmonic_trap_frequency_x(trap_w)
    lib.md_set_harmonic_trap_center_x(c.ctypes.data_as(_dp))
    lib.md_set_gaussian_force_strength_x(gauss_g)
    lib.md_set_guassian_force_range_x(gauss_s)
    lib.md_set_coulomb_force_strength_x(coul_s)
    lib.md_set_coulomb_truc_x(alpha)
    lib.md_set_coulomb_n_sum_x(nsum)


def md_step(lib, s, dt, image=0, trap=None, pair=None, pbc=False):
    """One MD step in the reference driver's call order; returns 0 or raises."""
    ck = lib.check
    ck(lib.md_update_nhc_VV3_1_x(s.sim, dt), "VV3_1")
    ck(lib.md_reset_force_x(s.sim), "reset_force")
    ck(lib.md_pimd_fast_fill_ENk_x(s.pimd, image), "fast_fill_ENk")
    ck(lib.md_pimd_fill_VB_x(s.pimd), "fill_VB")
    ck(lib.md_pimd_fast_fill_force_VB_x(s.pimd, image), "fast_fill_force_VB")
    if trap:
        ck(lib.md_pimd_calc_trap_force_x(s.pimd, trap), "trap force")
    if pair:
        ck(lib.md_pimd_calc_pair_force_x(s.pimd, pair), "pair force")
    ck(lib.md_update_nhc_VV3_2_x(s.sim, dt), "VV3_2")
    if pbc:
        ck(lib.md_periodic_boundary_x(s.sim), "periodic boundary")
    return 0


def two_species_forces(lib, a, b, image=0, trap=None, pair=None):
    """Forces of two species (same P) in the reference driver's call order:
    each species' exchange, trap and pair forces, then the cross pairs
    (md_pimd_calc_pair_force_2_x)."""
    ck = lib.check
    for s in (a, b):
        ck(lib.md_reset_force_x(s.sim), "reset_force")
        ck(lib.md_pimd_fast_fill_ENk_x(s.pimd, image), "fast_fill_ENk")
        ck(lib.md_pimd_fill_VB_x(s.pimd), "fill_VB")
        ck(lib.md_pimd_fast_fill_force_VB_x(s.pimd, image), "fast_fill_force_VB")
        if trap:
            ck(lib.md_pimd_calc_trap_force_x(s.pimd, trap), "trap force")
        if pair:
            ck(lib.md_pimd_calc_pair_force_x(s.pimd, pair), "pair force")
    if pair:
        ck(lib.md_pimd_calc_pair_force_2_x(a.pimd, b.pimd, pair), "cross-species pair force")


def two_species_step(lib, a, b, dt, image=0, trap=None, pair=None, pbc=False):
    """One MD step of two species; returns 0 or raises."""
    ck = lib.check
    for s in (a, b):
        ck(lib.md_update_nhc_VV3_1_x(s.sim, dt), "VV3_1")
    two_species_forces(lib, a, b, image, trap, pair)
    for s in (a, b):
        ck(lib.md_update_nhc_VV3_2_x(s.sim, dt), "VV3_2")
        if pbc:
            ck(lib.md_periodic_boundary_x(s.sim), "periodic boundary")
    return 0


class EwaldModel:
    """The learned Ewald residual of one system (md_gb300_ewald_model_*_x)."""

    def __init__(self, lib, system, nsum_cheap=3, capacity=16, seed=1):
        self.lib, self.h = lib, C.c_void_p()
        lib.check(lib.md_gb300_ewald_model_create_x(C.byref(self.h), system.pimd, nsum_cheap, capacity, seed),
                  "model create")
        self.N, self.P = system.N, system.P

    def collect(self, system):
        self.lib.check(self.lib.md_gb300_ewald_model_collect_x(self.h, system.pimd), "collect")

    def train(self, steps, batch_tiles, lr):
        loss = C.c_double()
        self.lib.check(self.lib.md_gb300_ewald_model_train_x(self.h, steps, batch_tiles, lr, C.byref(loss)), "train")
        return loss.value

    def attach(self, system, judge_every=50, force_tol=1e-2, energy_tol=1e-4):
        self.lib.check(self.lib.md_gb300_ewald_model_attach_x(system.pimd, self.h, judge_every, force_tol,
                                                              energy_tol), "attach")

    def detach(self, system):
        self.lib.check(self.lib.md_gb300_ewald_model_attach_x(system.pimd, None, 0, 0.0, 0.0), "detach")

    def judge(self, system):
        out = (C.c_double * 4)()
        self.lib.check(self.lib.md_gb300_ewald_model_judge_x(self.h, system.pimd, out), "judge")
        return {"force_err": out[0], "energy_err": out[1], "force_err_truncated": out[2],
                "energy_err_truncated": out[3]}

    def status(self):
        n, j, r = C.c_long(), C.c_int(), C.c_int()
        last = (C.c_double * 4)()
        self.lib.check(self.lib.md_gb300_ewald_model_status_x(self.h, C.byref(n), C.byref(j), C.byref(r), last))
        return {"configurations": n.value, "judged": j.value, "reverted": bool(r.value), "last": list(last)}

    def params(self, p=None):
        import numpy as np
        n = self.lib.md_gb300_ewald_model_nparam_x()
        if p is None:
            out = np.zeros(n, np.float32)
            self.lib.check(self.lib.md_gb300_ewald_model_params_x(self.h, out.ctypes.data_as(_fp), 0))
            return out
        q = np.ascontiguousarray(p, np.float32)
        assert q.size == n
        self.lib.check(self.lib.md_gb300_ewald_model_params_x(self.h, q.ctypes.data_as(_fp), 1))

    def forward(self, X):
        import numpy as np
        X = np.ascontiguousarray(X, np.float32)
        Y = np.zeros((X.shape[0], 4), np.float32)
        self.lib.check(self.lib.md_gb300_mlp_forward_x(self.h, X.ctypes.data_as(_fp), X.shape[0],
                                                       Y.ctypes.data_as(_fp)), "forward")
        return Y

    def grad(self, X, V, T, we=1.0, wf=1.0):
        import numpy as np
        X, V, T = (np.ascontiguousarray(a, np.float32) for a in (X, V, T))
        g = np.zeros(self.lib.md_gb300_ewald_model_nparam_x(), np.float32)
        loss = np.zeros(2, np.float32)
        self.lib.check(self.lib.md_gb300_mlp_grad_x(self.h, X.ctypes.data_as(_fp), V.ctypes.data_as(_fp),
                                                    T.ctypes.data_as(_fp), X.shape[0], we, wf,
                                                    g.ctypes.data_as(_fp), loss.ctypes.data_as(_fp)), "grad")
        return g, loss

    def features(self, system):
        import numpy as np
        F = np.zeros((self.N * self.P, 64), np.float32)
        V = np.zeros((self.N * self.P, 12), np.float32)
        self.lib.check(self.lib.md_gb300_ewald_model_features_x(self.h, system.pimd, F.ctypes.data_as(_fp),
                                                                V.ctypes.data_as(_fp)), "features")
        return F, V

    def desc_info(self):
        import numpy as np
        rc = C.c_double()
        B = np.zeros((64, 32), np.float32)
        mu, sg = (C.c_double * 3)(), (C.c_double * 3)()
        self.lib.check(self.lib.md_gb300_ewald_model_desc_info_x(self.h, C.byref(rc), B.ctypes.data_as(_fp), mu, sg))
        return rc.value, B, list(mu), list(sg)

    def free(self):
        if self.h:
            self.lib.md_gb300_ewald_model_free_x(self.h)
            self.h = C.c_void_p()
