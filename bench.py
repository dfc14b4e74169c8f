"""Benchmark: bead-steps/s of the path-integral MD step for the periodic
electron gas, N=512 particles x P=64 beads, rs=1, theta=0.5, xi=0.5, Ewald
with alpha=5.6/L over the converged reciprocal cube |n|<=10 (plain FP64).

One step is the reference driver's call sequence through the C ABI:
VV3_1, reset, fast ENk, V_B, exchange spring forces, Ewald pair forces,
VV3_2, periodic wrap.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl gb300|reference]

gb300 arm: `value` replays the step as a CUDA graph with the state resident
in HBM, L2 flushed (256 MB write) between steps outside the per-step CUDA
events; `e2e` runs the same calls with the host structs authoritative every
step (state uploaded from page-locked host memory before and read back
after every step, plus the estimator read).  reference arm: the oracle
port (MD-Lab's _nocl algorithm restated in C) on a bounded sample of the
same workload on all host cores.  Under torchrun every rank runs an
independent replica (the path does not shard); rank 0 prints one JSON line.
"""
import argparse
import ctypes as C
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "md-lab_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

N, P, RS, THETA, XI, NSUM, DT = 512, 64, 1.0, 0.5, 0.5, 10, 0.01
ALPHA_L = 5.6
METRIC = "bead-steps/s UEG N=512 P=64: learned+FP32 vs plain FP64 on 1 GB300, at stated ΔE/N"


def workload():
    box = (4 * math.pi * N / 3) ** (1 / 3) * RS
    n = N / box ** 3
    TF = 0.5 * (6 * math.pi ** 2 * n) ** (2 / 3)
    return box, THETA * TF


def config(form):
    box, T = workload()
    return {"workload": "PIMD step, periodic electron gas (spin-polarised), Ewald",
            "N": N, "P": P, "rs": RS, "theta": THETA, "xi": XI, "dt": DT, "box": box, "T": T,
            "ewald_alpha": ALPHA_L / box, "ewald_nsum": NSUM, "nhc_length": 4, "form": form,
            "l2": "flushed between timed steps (256 MB write outside the per-step events)",
            "parallelism": "replicas"}


# ---------------------------------------------------------------------
# distributed plumbing (one independent replica per rank)
# ---------------------------------------------------------------------
def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1
    import torch.distributed as dist
    backend = "nccl"
    dist.init_process_group(backend=backend)
    return dist, dist.get_rank(), ws


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, idx):
        self.idx, self.rows, self.proc = idx, [], None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.rows.append([c.strip() for c in ln.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        sm, reasons, mx = [], set(), None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
                for nm, v in zip(names, r[3:7]):
                    if v.lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------
# CPU baseline: the oracle port on a bounded sample
# ---------------------------------------------------------------------
def _pair_sample_worker(args):
    npairs, seed = args
    import numpy as np
    import orc
    box, T = workload()
    rng = np.random.default_rng(seed)
    prm = orc.params(coul_s=1.0, coul_alpha=ALPHA_L / box, coul_nsum=NSUM)
    Lb = np.full(3, box)
    pts = rng.uniform(0, box, size=(npairs, 2, 3))
    f = np.zeros(3)
    L_ = orc.lib()
    t0 = time.perf_counter()
    for i in range(npairs):
        L_.orc_pair_force_one(orc.PAIR_EWALD, C.byref(prm), 3, orc.ptr(pts[i, 0]), orc.ptr(pts[i, 1]),
                              orc.ptr(f), orc.ptr(Lb), 1.0)
    return time.perf_counter() - t0


def cpu_step_estimate(cores, budget_s):
    """Seconds per full step of the oracle port, from a bounded sample: the
    per-pair Ewald cost (timed on `cores` processes) times P*N(N-1)/2 pairs,
    plus the exchange and thermostat stages timed once on the full system."""
    import numpy as np
    import orc
    orc.build()
    box, T = workload()
    beta = 1 / T
    # exchange + integrator on the full system, single thread
    nb = N * P
    rng = np.random.default_rng(1)
    x = (rng.uniform(0, box, (N, 1, 3)) + 0.05 * rng.standard_normal((N, P, 3))).ravel()
    o = orc.OrcSim(3, 4, nb, np.ones(nb), x, rng.standard_normal(nb * 3), np.zeros(nb * 3),
                   np.ones(nb * 3), np.zeros(nb * 12), np.ones(nb * 12), np.full(nb * 12, 0.1), T, [box] * 3)
    t0 = time.perf_counter()
    orc.lib().orc_nhc_vv3_1(o.ref, DT)
    ENk, _ = orc.fast_fill_ENk(o, N, P, math.sqrt(P) / beta, 1)
    VBN = orc.fill_VB(N, beta, XI, ENk)
    orc.fast_force_VB(o, N, P, beta, XI, math.sqrt(P) / beta, 1, ENk, VBN)
    orc.lib().orc_nhc_vv3_2(o.ref, DT)
    orc.lib().orc_periodic_boundary(o.ref)
    t_rest = time.perf_counter() - t0
    # per-pair Ewald cost
    probe = _pair_sample_worker((8, 0))
    per_pair = probe / 8
    npairs = max(8, int(budget_s / per_pair))
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        t0 = time.perf_counter()
        times = pool.map(_pair_sample_worker, [(npairs, s + 1) for s in range(cores)])
        wall = time.perf_counter() - t0
    per_pair_all = max(times) / npairs / cores  # seconds per pair with `cores` workers
    pairs = P * N * (N - 1) // 2
    step = per_pair_all * pairs + t_rest
    sample = (f"{npairs * cores} Ewald pair evaluations (|n|<={NSUM}) on {cores} process(es) in "
              f"{wall:.1f} s, extrapolated to {pairs} pair-slices per step; exchange recursion, "
              f"NHC and wrap timed once on the full N={N}, P={P} system ({t_rest:.2f} s)")
    return step, sample


# ---------------------------------------------------------------------
# GB300 arm
# ---------------------------------------------------------------------
# algorithmic FP64 work per launch of each kernel, FMA = 2 flops (the design doc
# section 4 derives each count from the kernel's arithmetic)
def kernel_flops(name, launches_per_step):
    ncol = NSUM * (2 * NSUM + 1) + NSUM + 1  # wave-vector columns (nx, ny)
    if name == "recip_force":
        return 177.0 * ncol * N * P
    if name == "sk":
        return 88.0 * ncol * N * P
    if name == "pair_tiles_ewald_real":
        box, _ = workload()
        rc = 5.8 / (ALPHA_L / box)
        # expected images inside the cut-off per pair: (4/3) pi rc^3 / V
        n_img = 4 / 3 * math.pi * rc ** 3 / box ** 3
        pairs = P * N * (N - 1) / 2
        return pairs * (47.0 * n_img + 39.0)
    return None


def make_system(lib):
    import xmd_x
    box, T = workload()
    s = xmd_x.PimdSystem(lib, N, P, XI, T, box=box)
    lib.md_set_seed_x(2024)
    lib.md_init_particle_mass_x(s.sim, 1.0, 0, N * P)
    c = (C.c_double * 3)(box / 2, box / 2, box / 2)
    Lv = (C.c_double * 3)(box, box, box)
    lib.md_pimd_init_particle_uniform_pos_x(s.pimd, c, Lv, 0.05 * RS)
    lib.md_init_maxwell_vel_x(s.sim, T)
    Q = lib.md_get_quick_Q_x(T, s.pimd.contents.omegaP)
    lib.md_init_nhc_x(s.sim, Q, 0, s.sim.contents.Nf, 0.0)
    xmd_x.set_potentials(lib, coul_s=1.0, alpha=ALPHA_L / box, nsum=NSUM)
    return s


def run_gb300(args, dist, rank, ws):
    import torch
    import xmd_x
    lib = xmd_x.load(3, 4)
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    lib.check(lib.md_gb300_set_device_x(dev), "set device")
    s = make_system(lib)
    pair = lib.fn("md_coulomb_3d_ewald_force_x")
    step = lambda: xmd_x.md_step(lib, s, DT, image=1, pair=pair, pbc=True)  # noqa: E731
    for _ in range(args.warmup):
        step()
    lib.check(lib.md_gb300_synchronize_x(), "sync")
    stream = torch.cuda.ExternalStream(lib.md_gb300_get_stream_x())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed_graph(nsteps):
        """capture one step, replay it; per-step CUDA events, L2 flushed in between"""
        g = C.c_void_p()
        lib.check(lib.md_gb300_capture_begin_x(), "capture begin")
        step()
        lib.check(lib.md_gb300_capture_end_x(C.byref(g)), "capture end")
        kps = lib.md_gb300_graph_kernel_count_x(g)
        for _ in range(max(3, args.warmup)):
            lib.check(lib.md_gb300_graph_launch_x(g, 1))
        lib.check(lib.md_gb300_synchronize_x())
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(nsteps)]
        barrier(dist)
        torch.cuda.synchronize()
        with Clocks(dev) as clk:
            t0 = time.perf_counter()
            with torch.cuda.stream(stream):
                for e0, e1 in evs:
                    flush.zero_()
                    e0.record(stream)
                    lib.check(lib.md_gb300_graph_launch_x(g, 1))
                    e1.record(stream)
            lib.check(lib.md_gb300_synchronize_x())
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
        barrier(dist)
        lib.md_gb300_graph_free_x(g)
        ms = sum(a.elapsed_time(b) for a, b in evs) / nsteps
        return max_over_ranks(dist, ms), kps, wall, clk.summary()

    step_ms, kernels_per_step, wall, clocks = timed_graph(args.steps)
    value = ws * N * P / (step_ms * 1e-3)
    # the mixed-precision form on the same state: time and force error
    forms = {"plain_fp64": {"value": value, "ms_per_step": step_ms}}
    if not args.no_mixed:
        def forces(mode):
            lib.check(lib.md_gb300_set_precision_x(mode))
            lib.check(lib.md_reset_force_x(s.sim))
            lib.check(lib.md_pimd_calc_pair_force_x(s.pimd, pair))
            return s.state()["f"]
        import numpy as np
        f64, f32 = forces(0), forces(1)
        ferr = float(np.max(np.abs(f32 - f64)) / np.max(np.abs(f64)))
        mixed_ms, _, _, mixed_clocks = timed_graph(args.steps)
        lib.check(lib.md_gb300_set_precision_x(0))
        forms["mixed_fp32_forces"] = {"value": ws * N * P / (mixed_ms * 1e-3), "ms_per_step": mixed_ms,
                                      "force_error_vs_fp64": ferr, "clocks": mixed_clocks}
    # live per-kernel timing of two plain steps (outside the timed region)
    lib.check(lib.md_gb300_profile_x(1))
    for _ in range(2):
        step()
    lib.check(lib.md_gb300_synchronize_x())
    prof = lib.profile_report()
    lib.check(lib.md_gb300_profile_x(0))
    total = sum(v[0] for v in prof.values())
    top = max(prof.items(), key=lambda kv: kv[1][0])
    fp64_peak = lib.md_gb300_fp64_peak_x()
    per_launch_ms = top[1][0] / top[1][1]
    flops = kernel_flops(top[0], top[1][1] / 2)
    roof = {"kernel": top[0], "bound": "fp64", "unit": "TFLOP/s",
            "share": top[1][0] / total if total else None,
            "launch_ms": per_launch_ms,
            "peak": fp64_peak, "peak_source": "live DFMA probe on this GPU (md_gb300_fp64_peak_x)",
            "traffic": None}
    if flops:
        roof["achieved"] = flops / (per_launch_ms * 1e-3) / 1e12
        roof["frac"] = roof["achieved"] / fp64_peak if fp64_peak > 0 else None
    # e2e: host structs authoritative every step
    ke = min(args.steps, args.e2e_steps)
    pe = lib.fn("md_coulomb_3d_ewald_energy_x")
    h2d = C.sizeof(lib.Particle) * N * P + C.sizeof(lib.Nhc) * s.sim.contents.Nf
    lib.check(lib.md_gb300_synchronize_x())
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(ke):
        if not lib.md_simulation_sync_host_x(s.sim, 0):  # device -> host, host authoritative
            raise RuntimeError(lib.err())
        step()  # first call uploads the host state
        lib.check(lib.md_pimd_calc_VBN_energy_x(s.pimd, s.stats))
        s.take_energy()  # estimator read
    if not lib.md_simulation_sync_host_x(s.sim, 1):
        raise RuntimeError(lib.err())
    e2e_s = (time.perf_counter() - t0) / ke
    e2e_s = max_over_ranks(dist, e2e_s)
    launches = kernels_per_step * args.steps
    result = {"metric": METRIC, "value": value, "unit": "bead-steps/s", "n_gpus": ws,
              "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
              "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
              "data": "synthetic (seeded uniform electron-gas configuration from the library's own "
                      "initial-condition routines)",
              "config": config("plain FP64"), "gpu_launches": launches, "forms": forms,
              "kernels_per_step": kernels_per_step, "wall_s_timed": wall,
              "e2e": {"value": ws * N * P / e2e_s, "unit": "bead-steps/s", "h2d_bytes_per_step": h2d,
                      "d2h_bytes_per_step": h2d + 8, "steps": ke},
              "roofline": roof, "kernel_ms_per_step": {k: v[0] / 2 for k, v in prof.items()},
              "clocks": clocks}
    if rank == 0 and ws == 1 and not args.no_cpu:
        st, sample = cpu_step_estimate(1, args.cpu_budget)
        result["cpu_baseline"] = {"value": N * P / st, "unit": "bead-steps/s", "cores": 1,
                                  "kind": "port", "sample": sample}
    s.free()
    return result


def run_reference(args, rank):
    cores = os.cpu_count() or 1
    vals = []
    sample = ""
    for i in range(args.warmup + args.steps):
        st, sample = cpu_step_estimate(cores, args.cpu_budget / 4)
        if i >= args.warmup:
            vals.append(st)
    step_s = statistics.median(vals)
    v = N * P / step_s
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "bead-steps/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config("plain FP64 (CPU oracle port)"),
            "cpu_baseline": {"value": v, "unit": "bead-steps/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "bead-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-budget", type=float, default=8.0, help="seconds of CPU sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision form")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        if rank != 0:
            return
        print(json.dumps(run_reference(args, rank)))
        return
    dist, rank, ws = dist_init()
    res = run_gb300(args, dist, rank, ws)
    if rank == 0:
        print(json.dumps(res))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
