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
NSUM_CHEAP, JUDGE_EVERY = 3, 50
METRIC = "bead-steps/s UEG N=512 P=64: learned+FP32 vs plain FP64 on 1 GB300, at stated ΔE/N"


def workload():
    box = (4 * math.pi * N / 3) ** (1 / 3) * RS
    n = N / box ** 3
    TF = 0.5 * (6 * math.pi ** 2 * n) ** (2 / 3)
    return box, THETA * TF


def config():
    """the workload both arms run (the arithmetic form is reported beside it)"""
    box, T = workload()
    return {"workload": "PIMD step, periodic electron gas (spin-polarised), Ewald",
            "N": N, "P": P, "rs": RS, "theta": THETA, "xi": XI, "dt": DT, "box": box, "T": T,
            "ewald_alpha": ALPHA_L / box, "ewald_nsum": NSUM, "nhc_length": 4,
            "l2": "flushed between timed steps (256 MB write outside the per-step events)",
            "parallelism": "replicas"}


# ---------------------------------------------------------------------
# distributed plumbing (one independent replica per rank)
# ---------------------------------------------------------------------
def dist_init(backend=None):
    """one process per GPU (torchrun); NCCL on GPUs, gloo otherwise"""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1
    import torch
    import torch.distributed as dist
    if backend is None:
        backend = "nccl" if torch.cuda.is_available() else "gloo"
    dist.init_process_group(backend=backend)
    return dist, dist.get_rank(), ws


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_result(dist, ws, beads_per_replica, ms_local):
    """whole-job throughput of independent replicas: every rank advances its
    own system; the job's step time is the slowest rank's"""
    ms = max_over_ranks(dist, ms_local)
    return ws * beads_per_replica / (ms * 1e-3), ms


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

    def started(self, limit=5.0):
        """wait (bounded) for nvidia-smi's first row, so that sampling covers
        the region that follows; rows before it are not counted"""
        t = time.perf_counter()
        while self.proc and not self.rows and time.perf_counter() - t < limit:
            time.sleep(0.005)
        self.n0 = len(self.rows)
        return self

    def fresh(self):
        return len(self.rows) - getattr(self, "n0", 0)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        sm, reasons, mx = [], set(), None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows[getattr(self, "n0", 0):]:
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
def n_images(xcut=5.2):
    """expected real-space images per pair inside the cut-off alpha R < xcut
    (5.2 in the FP64 force kernels, 3.6 in the FP32 ones)"""
    box, _ = workload()
    rc = xcut / (ALPHA_L / box)
    return 4 / 3 * math.pi * rc ** 3 / box ** 3


# algorithmic work per launch of each kernel (FMA = 2 flops); the same count
# for the FP64 and FP32 versions of a kernel, each derived from the kernel's
# arithmetic per pair, image or wave vector
def kept_nz_pairs(nsum, part=None):
    """sum over the kept wave-vector columns (nx, ny) of their largest kept
    |nz|: the library leaves out vectors whose force weight |G| c(n) is
    below 1e-17 of the largest (RECIP_KEEP), so the column kernels run
    this many +-nz pairs instead of ncol * nsum (cubic box, alpha L = ALPHA_L).
    part "fp64" / "fp32": only the columns the FP64 form's split keeps in
    FP64 / sends to the FP32 kernels (largest weight in the column at or
    above / below 1e-7 of the largest, RECIP_SPLIT)"""
    w = {}
    for nx in range(nsum + 1):
        for ny in range(-nsum, nsum + 1):
            if nx == 0 and ny < 0:
                continue
            for nz in range(1 if nx == 0 and ny == 0 else -nsum, nsum + 1):
                g2 = nx * nx + ny * ny + nz * nz
                w[(nx, ny, nz)] = math.exp(-math.pi ** 2 * g2 / ALPHA_L ** 2) / math.sqrt(g2)
    wmax = max(w.values())
    nzmax, wcol = {}, {}
    for (nx, ny, nz), v in w.items():
        if v >= 1e-17 * wmax:
            nzmax[(nx, ny)] = max(nzmax.get((nx, ny), 0), abs(nz))
            wcol[(nx, ny)] = max(wcol.get((nx, ny), 0.0), v)
    if part == "fp64":
        return sum(z for c, z in nzmax.items() if wcol[c] >= 1e-7 * wmax)
    if part == "fp32":
        return sum(z for c, z in nzmax.items() if wcol[c] < 1e-7 * wmax)
    return sum(nzmax.values())


def shell_vectors(count=32):
    """half-space wave vectors of the `count` lowest shells |n|^2 (the
    descriptors' structure-factor features)"""
    shells, n2 = [], 0
    while len(shells) < count:
        n2 += 1
        if any(a * a + b * b <= n2 and int(round(math.sqrt(n2 - a * a - b * b))) ** 2 == n2 - a * a - b * b
               for a in range(int(math.sqrt(n2)) + 1) for b in range(int(math.sqrt(n2)) + 1)):
            shells.append(n2)
    m = int(math.sqrt(shells[-1]))
    return sum(1 for a in range(m + 1) for b in range(-m, m + 1) for c in range(-m, m + 1)
               if (a > 0 or (a == 0 and b > 0) or (a == 0 and b == 0 and c > 0)) and a * a + b * b + c * c in shells)


def kernel_flops(name, nsum=NSUM, split=False):
    """split: the FP64 form's kernels with their FP32 parts split off (real-
    space images at alpha R >= 4 and the small-weight wave-vector columns
    on the FP32 pipe): the FP64 work of the FP64 kernels"""
    part = "fp64" if split else None
    if name in ("recip_force", "recip_force32"):
        # 17.7 flop per +-nz pair of a kept column per particle and slice
        return 17.7 * kept_nz_pairs(nsum, part if name == "recip_force" else None) * N * P
    if name in ("sk", "sk32"):
        return 8.8 * kept_nz_pairs(nsum, part if name == "sk" else None) * N * P
    if name == "pair_tiles_ewald_real":
        pairs = P * N * (N - 1) / 2
        return pairs * (47.0 * n_images(4.0 if split else 5.2) + 39.0)
    if name == "pair_tiles32_ewald_real":
        pairs = P * N * (N - 1) / 2
        return pairs * (47.0 * n_images(3.6) + 39.0)
    if name == "desc":
        # per ordered pair: 15 flop for the minimum-image distance and the
        # cut-off test, and for the (4/3) pi (1/2)^3 = 52% inside rc = L/2
        # another 45 (r, cut-off weight, bin weights, two deposits, three
        # Gaussian-weighted vector features); per particle the 64 x 32
        # histogram-to-feature product
        return N * N * P * (15.0 + 0.5236 * 45.0) + N * P * 2.0 * 64 * 32
    if name == "desc_shells":
        # per slice, wave vector of the 32 lowest shells and particle: two
        # complex products and the complex add (14 flop)
        return P * shell_vectors() * N * 14.0
    if name == "mlp_forward":
        return 2.0 * N * P * (64 * 128 + 128 * 128 + 128 * 16)
    return None


# DRAM traffic per launch (dram__bytes_read.sum + dram__bytes_write.sum) of
# each kernel with a FLOP model, from one ncu capture on this workload
# (summaries in profiles/, named for the kernel)
TRAFFIC = {"desc": 822272, "pair_tiles32_ewald_real": 424192, "pair_tiles_ewald_real": 1125632,
           "sk": 17358592, "recip_force": 23965184, "mlp_forward": 4273408}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def make_system(lib, xi=XI):
    import xmd_x
    box, T = workload()
    s = xmd_x.PimdSystem(lib, N, P, xi, T, box=box)
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


class Runner:
    """Graph capture and per-step CUDA-event timing on the library's stream."""

    def __init__(self, lib, dist, dev, args):
        import torch
        self.torch, self.lib, self.dist, self.dev, self.args = torch, lib, dist, dev, args
        self.stream = torch.cuda.ExternalStream(lib.md_gb300_get_stream_x())
        self.flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def capture(self, step):
        lib = self.lib
        g = C.c_void_p()
        lib.check(lib.md_gb300_capture_begin_x(), "capture begin")
        step()
        lib.check(lib.md_gb300_capture_end_x(C.byref(g)), "capture end")
        return g, lib.md_gb300_graph_kernel_count_x(g)

    def launcher(self, g):
        lib = self.lib
        return lambda: lib.check(lib.md_gb300_graph_launch_x(g, 1))

    def time(self, actions, warm, clocks=True):
        """Per-step CUDA events around each action (one step each); the L2 is
        flushed (256 MB write) before every step, outside the events."""
        torch, lib = self.torch, self.lib
        for a in warm:
            a()
        lib.check(lib.md_gb300_synchronize_x())
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in actions]
        barrier(self.dist)
        torch.cuda.synchronize()
        with Clocks(self.dev) as clk:
            clk.started()
            t0 = time.perf_counter()
            with torch.cuda.stream(self.stream):
                for (e0, e1), act in zip(evs, actions):
                    self.flush.zero_()
                    e0.record(self.stream)
                    act()
                    e1.record(self.stream)
            lib.check(lib.md_gb300_synchronize_x())
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
            # a timed region of a few ms falls between nvidia-smi's 100 ms
            # samples: the same step is replayed (untimed, same flush) until
            # five samples under load exist, at most 3 s
            pad, t1 = 0, time.perf_counter()
            while clocks and clk.proc and clk.fresh() < 5 and time.perf_counter() - t1 < 3.0:
                with torch.cuda.stream(self.stream):
                    for _ in range(16):
                        self.flush.zero_()
                        warm[0]()
                lib.check(lib.md_gb300_synchronize_x())
                pad += 16
        barrier(self.dist)
        self.last_ms = [a.elapsed_time(b) for a, b in evs]
        ms = sum(self.last_ms) / len(evs)
        summ = clk.summary()
        summ["window"] = (f"the {len(actions)} timed steps" if not pad else
                          f"the {len(actions)} timed steps and {pad} untimed replays of the same step after them")
        return max_over_ranks(self.dist, ms), wall, summ

    def profile(self, step, n=2):
        """live per-kernel times of n un-captured steps: {kernel: ms per step}"""
        lib = self.lib
        lib.check(lib.md_gb300_synchronize_x())
        lib.check(lib.md_gb300_profile_x(1))
        for _ in range(n):
            step()
        lib.check(lib.md_gb300_synchronize_x())
        prof = lib.profile_report()
        lib.check(lib.md_gb300_profile_x(0))
        return {k: (v[0] / n, v[1] // n) for k, v in prof.items()}


def roofline(prof, peak, peak_name, unit_nsum=NSUM, split=False):
    """FLOP roofline of the step's dominant arithmetic kernel (the largest
    with a FLOP model) from its live per-launch time; the overall largest
    kernel is named beside it (the exchange recursion is latency-bound: N
    dependent steps, no FLOP or byte roofline applies)"""
    total = sum(v[0] for v in prof.values())
    top_name, (top_ms, _) = max(prof.items(), key=lambda kv: kv[1][0])
    modelled = {k: v for k, v in prof.items() if kernel_flops(k, unit_nsum, split)}
    name, (ms, launches) = max(modelled.items(), key=lambda kv: kv[1][0])
    per_launch_ms = ms / max(launches, 1)
    roof = {"kernel": name, "bound": "fp64" if peak_name == "fp64" else "fp32", "unit": "TFLOP/s",
            "share": ms / total if total else None, "launch_ms": per_launch_ms, "peak": peak,
            "peak_source": f"live {peak_name.upper()} FMA probe on this GPU (md_gb300_{peak_name}_peak_x)",
            "traffic": TRAFFIC.get(name)}
    flops = kernel_flops(name, unit_nsum, split)
    if flops:
        roof["algorithmic_flop_per_launch"] = flops
        roof["achieved"] = flops / (per_launch_ms * 1e-3) / 1e12
        roof["frac"] = roof["achieved"] / peak if peak > 0 else None
    roof["step_top_kernel"] = {"kernel": top_name, "share": top_ms / total if total else None,
                               "ms_per_step": top_ms}
    if "solve" in top_name:
        roof["step_top_kernel"]["bound"] = f"latency: {N} dependent substitution steps, 2 SMs"
    return roof


def judge_fails(j, args):
    """the network is dropped when, on the judged configuration, its force
    error exceeds the truncated sum's own (it would do harm) or its energy
    error per particle exceeds the energy tolerance"""
    return j["force_err"] > args.force_tol * j["force_err_truncated"] or j["energy_err"] > args.energy_tol


def learned_form(lib, R, s, pair, step, args, ws):
    """Truncated Ewald (|n| <= NSUM_CHEAP) + the residual network, FP32 forces.
    Data from plain runs of this system (converged Ewald, mixed forces),
    training on the GPU, then the timed run with the converged sum as judge
    every JUDGE_EVERY steps: after every JUDGE_EVERY-th learned step the
    configuration is judged (converged FP64 reciprocal sums, truncated sums
    and network, compared; inside the timed region).  A failed judgement
    sends the rest of the run to the converged step."""
    import xmd_x
    lib.check(lib.md_gb300_set_precision_x(1))
    box, _ = workload()
    xmd_x.set_potentials(lib, coul_s=1.0, alpha=ALPHA_L / box, nsum=NSUM)
    m = xmd_x.EwaldModel(lib, s, nsum_cheap=NSUM_CHEAP, capacity=args.learn_configs, seed=7)
    t0 = time.perf_counter()
    for _ in range(args.learn_configs):
        step()
        m.collect(s)
    lib.check(lib.md_gb300_synchronize_x())
    t_collect = time.perf_counter() - t0
    t0 = time.perf_counter()
    loss = m.train(args.learn_steps, args.learn_batch, args.learn_lr)
    t_train = time.perf_counter() - t0
    for _ in range(5):
        step()
    first = m.judge(s)
    # graphs: the learned step, and the converged (judge) step
    g_conv, _ = R.capture(step)
    m.attach(s, judge_every=0)
    g_learn, kps = R.capture(step)
    state = {"reverted": False}
    judges = []

    def judge_step():
        lib.check(lib.md_gb300_graph_launch_x(g_conv if state["reverted"] else g_learn, 1))
        if state["reverted"]:
            return
        j = m.judge(s)
        judges.append(j)
        if judge_fails(j, args):
            state["reverted"] = True

    def learned_step():
        lib.check(lib.md_gb300_graph_launch_x(g_conv if state["reverted"] else g_learn, 1))

    # exactly the steps asked for; the judgement follows step 0 and every
    # JUDGE_EVERY-th step after it
    nsteps = args.steps
    actions = [judge_step if i % JUDGE_EVERY == 0 else learned_step for i in range(nsteps)]
    ms, wall, clocks = R.time(actions, [R.launcher(g_learn)] * 3)
    per_step = R.last_ms
    judged_ms = [t for i, t in enumerate(per_step) if i % JUDGE_EVERY == 0]
    plain_ms = [t for i, t in enumerate(per_step) if i % JUDGE_EVERY != 0]
    prof = R.profile(step)
    value = ws * N * P / (ms * 1e-3)
    lib.md_gb300_graph_free_x(g_learn)
    lib.md_gb300_graph_free_x(g_conv)
    keys = ("force_err", "energy_err", "force_err_truncated", "energy_err_truncated")
    all_j = [first] + judges
    form = {"value": value, "ms_per_step": ms, "steps_timed": nsteps, "kernels_per_learned_step": kps,
            "ms_learned_step_median": statistics.median(plain_ms) if plain_ms else None,
            "ms_judged_step": judged_ms, "judgements_timed": len(judged_ms),
            "clocks": clocks, "wall_s_timed": wall, "reverted": state["reverted"],
            "nsum_truncated": NSUM_CHEAP, "nsum_converged": NSUM, "judge_every": JUDGE_EVERY,
            "training": {"configurations": args.learn_configs, "bead_slice_configurations": args.learn_configs * P,
                         "rows": args.learn_configs * N * P, "adam_steps": args.learn_steps,
                         "batch_rows": args.learn_batch * 128, "lr": args.learn_lr, "final_loss": loss,
                         "collect_s": t_collect, "train_s": t_train},
            "judged": {k: [j[k] for j in all_j] for k in keys},
            "delta_E_per_particle_Ha": max(j["energy_err"] for j in all_j),
            "delta_E_per_particle_truncated_only_Ha": max(j["energy_err_truncated"] for j in all_j),
            "force_err_rms_rel": max(j["force_err"] for j in all_j),
            "force_err_rms_rel_truncated_only": max(j["force_err_truncated"] for j in all_j),
            "tolerances": {"force": f"{args.force_tol} x the truncated sum's force error on the same configuration",
                           "energy_per_particle_Ha": args.energy_tol},
            "kernel_ms_per_step": {k: v[0] for k, v in prof.items()}}
    return m, form, prof, kps


# ---------------------------------------------------------------------
# batched ensemble (64 independent systems, one graph launch per step)
# ---------------------------------------------------------------------
ENS_N, ENS_P = (16, 24, 32, 48, 64, 96, 128), (16, 32, 64)


def ensemble_specs(seed=4):
    """8 xi in [0, 1] x 8 beta in 1..8; N and P drawn from the lists; even
    systems 3D traps with Gaussian repulsion, odd ones electron gas"""
    import numpy as np
    rng = np.random.default_rng(seed)
    specs = []
    for a in range(8):
        for b in range(8):
            i = a * 8 + b
            specs.append(("trap" if i % 2 == 0 else "ueg", int(rng.choice(ENS_N)), int(rng.choice(ENS_P)),
                          a / 7.0, b + 1.0))
    return specs


def ensemble_form(lib, R, args):
    import numpy as np
    import xmd_x
    lib.check(lib.md_gb300_set_precision_x(1))  # FP32 forces, FP64 recursion and NHC
    specs = ensemble_specs()
    rng = np.random.default_rng(11)
    systems = []
    for kind, n, p, vi, beta in specs:
        T = 1.0 / beta
        box = (4 * math.pi * n / 3) ** (1 / 3) * 2.0 if kind == "ueg" else 10.0
        s = xmd_x.PimdSystem(lib, n, p, vi, T, box=box)
        if kind == "ueg":
            x = rng.uniform(0, box, (n, 1, 3)) + 0.05 * rng.standard_normal((n, p, 3))
        else:
            x = rng.standard_normal((n, p, 3))
        s.set_state(m=np.ones(n * p), x=x.ravel(), v=rng.standard_normal(n * p * 3) * math.sqrt(T))
        lib.md_init_nhc_x(s.sim, lib.md_get_quick_Q_x(T, s.pimd.contents.omegaP), 0, s.sim.contents.Nf, 0.0)
        systems.append((kind, s, box))
    ewald = lib.fn("md_coulomb_3d_ewald_force_x")
    gauss = lib.fn("md_gaussian_force_x")
    trapf = lib.fn("md_harmonic_trap_force_x")

    def one(i):
        kind, s, box = systems[i]
        if kind == "ueg":
            xmd_x.set_potentials(lib, coul_s=1.0, alpha=5.6 / box, nsum=8)
            xmd_x.md_step(lib, s, 0.05, image=1, pair=ewald, pbc=True)
        else:
            xmd_x.set_potentials(lib, trap_w=1.0, gauss_g=0.75 * math.pi, gauss_s=0.5)
            xmd_x.md_step(lib, s, 0.005, trap=trapf, pair=gauss)

    for _ in range(2):
        for i in range(len(systems)):
            one(i)
    # autotuned tile shapes, one per distinct system shape
    tuned = {}
    for i, (kind, s, box) in enumerate(systems):
        key = (kind, specs[i][1], specs[i][2])
        if key in tuned:
            continue
        if kind == "ueg":
            xmd_x.set_potentials(lib, coul_s=1.0, alpha=5.6 / box, nsum=8)
        else:
            xmd_x.set_potentials(lib, trap_w=1.0, gauss_g=0.75 * math.pi, gauss_s=0.5)
        w = C.c_int()
        lib.check(lib.md_gb300_autotune_pair_x(s.pimd, ewald if kind == "ueg" else gauss, 5, C.byref(w), None))
        tuned[key] = w.value
    step_fn = C.CFUNCTYPE(C.c_int, C.c_int, C.c_void_p)

    def cb(i, ctx):
        try:
            one(i)
            return 0
        except Exception:
            return -1

    fn = step_fn(cb)
    g = C.c_void_p()
    lib.check(lib.md_gb300_capture_ensemble_x(len(systems), C.cast(fn, C.c_void_p), None, C.byref(g)),
              "ensemble capture")
    kernels = lib.md_gb300_graph_kernel_count_x(g)
    beads = sum(n * p for _, n, p, _, _ in specs)
    nst = max(args.steps, 10)
    ms, wall_br, clocks = R.time([R.launcher(g)] * nst, [R.launcher(g)] * 3)
    # the same 64 steps as separate graphs, one after the other
    singles = [R.capture(lambda i=i: one(i))[0] for i in range(len(systems))]

    def seq():
        for gi in singles:
            lib.check(lib.md_gb300_graph_launch_x(gi, 1))

    ms_seq, _, _ = R.time([seq] * nst, [seq] * 3, clocks=False)
    for gi in singles:
        lib.md_gb300_graph_free_x(gi)
    lib.md_gb300_graph_free_x(g)
    # one persistent kernel per step: grid size by the autotuner (which
    # advances the systems by the steps it times), then captured
    ms_br, kernels_br = ms, kernels
    cl, grp, tms = C.c_int(), C.c_int(), C.c_double()
    lib.check(lib.md_gb300_autotune_ensemble_x(len(systems), C.cast(fn, C.c_void_p), None, 3, C.byref(cl),
                                               C.byref(grp), C.byref(tms)), "persistent ensemble autotuning")
    gp = C.c_void_p()
    lib.check(lib.md_gb300_capture_ensemble_persistent_x(len(systems), C.cast(fn, C.c_void_p), None, C.byref(gp)),
              "persistent ensemble capture")
    kernels = lib.md_gb300_graph_kernel_count_x(gp)
    ms, wall, clocks = R.time([R.launcher(gp)] * nst, [R.launcher(gp)] * 3)
    lib.check(lib.md_gb300_ensemble_status_x(gp), "persistent ensemble status")
    ph = (C.c_double * 45)()
    nph = lib.md_gb300_ensemble_phase_times_x(gp, ph, 45)
    group_us = [round(v, 1) for v in ph[13:nph]]
    phase_us = {nm: round(v, 1) for nm, v in zip(
        ("VV3_1", "springs_Eint_tiles_Sk", "prefix_tables", "ENk_recip", "weights_inverses_pairsum", "solves", "G",
         "exch_ends", "VV3_2", "block0_springs", "block0_Eint", "block0_tiles", "block0_Sk"), ph)}
    lib.md_gb300_graph_free_x(gp)
    for _, s, _ in systems:
        s.free()
    lib.check(lib.md_gb300_set_precision_x(0))
    box, _ = workload()  # the ensemble left its last system's parameters in the globals
    xmd_x.set_potentials(lib, coul_s=1.0, alpha=ALPHA_L / box, nsum=NSUM)
    return {"value": beads / (ms * 1e-3), "unit": "bead-steps/s", "ms_per_step": ms, "systems": len(specs),
            "bead_slots": beads, "kernels_per_launch": kernels, "steps_timed": nst,
            "persistent_blocks_per_sm": cl.value, "persistent_groups": grp.value,
            "persistent_phase_us_group0": phase_us, "persistent_group_us": group_us, "autotuned_ms": tms.value, "wall_s_timed": wall,
            "graph_branches_wall_s_timed": wall_br,
            "graph_branches_ms_per_step": ms_br, "graph_branches_kernels": kernels_br,
            "gain_vs_graph_branches": ms_br / ms,
            "sequential_graphs_ms_per_step": ms_seq, "gain_vs_sequential": ms_seq / ms,
            "tile_warps_chosen": {f"{k[0]} N={k[1]} P={k[2]}": v for k, v in sorted(tuned.items())},
            "clocks": clocks,
            "workload": "64 systems: 8 xi in [0,1] x 8 beta in 1..8, N in {16..128}, P in {16,32,64}; "
                        "even: 3D trap + Gaussian repulsion (g=0.75 pi, s=0.5, dt=0.005); odd: electron gas "
                        "rs=2, Ewald alpha=5.6/L |n|<=8, dt=0.05; FP32 forces, FP64 recursion and NHC"}


def two_species_form(lib, R, args, fp64_peak):
    """Spin-unpolarised electron gas through md_pimd_calc_pair_force_2_x:
    N/2 up + N/2 down electrons, P beads, the headline box and density
    (rs=1), theta=0.5 of the unpolarised gas's Fermi temperature.  Each
    species has its own exchange recursion and Ewald pairs, plus the cross
    pairs (real space and structure factors); plain FP64, converged |n|<=10."""
    import xmd_x
    box, _ = workload()
    T = THETA * 0.5 * (3 * math.pi ** 2 * N / box ** 3) ** (2 / 3)
    Na = N // 2
    lib.check(lib.md_gb300_set_precision_x(0))
    xmd_x.set_potentials(lib, coul_s=1.0, alpha=ALPHA_L / box, nsum=NSUM)
    lib.md_set_seed_x(77)
    c = (C.c_double * 3)(box / 2, box / 2, box / 2)
    Lv = (C.c_double * 3)(box, box, box)
    pair_of = []
    for _ in range(2):
        s = xmd_x.PimdSystem(lib, Na, P, XI, T, box=box)
        lib.md_init_particle_mass_x(s.sim, 1.0, 0, Na * P)
        lib.md_pimd_init_particle_uniform_pos_x(s.pimd, c, Lv, 0.05 * RS)
        lib.md_init_maxwell_vel_x(s.sim, T)
        lib.md_init_nhc_x(s.sim, lib.md_get_quick_Q_x(T, s.pimd.contents.omegaP), 0, s.sim.contents.Nf, 0.0)
        pair_of.append(s)
    a, b = pair_of
    pair = lib.fn("md_coulomb_3d_ewald_force_x")
    step = lambda: xmd_x.two_species_step(lib, a, b, DT, image=1, pair=pair, pbc=True)  # noqa: E731
    for _ in range(args.warmup):
        step()
    g, kps = R.capture(step)
    ms, _, clocks = R.time([R.launcher(g)] * args.steps, [R.launcher(g)] * max(3, args.warmup))
    lib.md_gb300_graph_free_x(g)
    prof = R.profile(step)
    out = {"value": N * P / (ms * 1e-3), "unit": "bead-steps/s", "ms_per_step": ms, "kernels_per_step": kps,
           "clocks": clocks, "species": [Na, N - Na], "T": T,
           "kernel_ms_per_step": {k: v[0] for k, v in prof.items()}}
    if "pair_cross" in prof:
        cross_ms, launches = prof["pair_cross"]
        flops = P * Na * (N - Na) * (47.0 * n_images() + 39.0)
        per = cross_ms / max(launches, 1)
        achieved = flops / (per * 1e-3) / 1e12
        out["cross_roofline"] = {"kernel": "pair_cross (Ewald real space, cross pairs)", "bound": "fp64",
                                 "unit": "TFLOP/s", "launch_ms": per, "algorithmic_flop_per_launch": flops,
                                 "achieved": achieved, "peak": fp64_peak,
                                 "frac": achieved / fp64_peak if fp64_peak > 0 else None}
    a.free()
    b.free()
    return out


def recursion_form(lib, R, args):
    """The exchange recursions alone (V_B forward and tmpV backward, weights,
    diagonal-block inverses and the block solve: md_pimd_fill_VB_x) against
    N: microseconds per call, graph-replayed, on electron-gas-like random
    positions (P = 8 beads; the recursion's cost does not depend on P)."""
    import numpy as np
    import xmd_x
    out = {}
    for n in (64, 128, 256, 512, 1024, 2048):
        box = (4 * math.pi * n / 3) ** (1 / 3)
        s = xmd_x.PimdSystem(lib, n, 8, XI, 1.0, box=box)
        rng = np.random.default_rng(n)
        x = (rng.uniform(0, box, (n, 1, 3)) + 0.05 * rng.standard_normal((n, 8, 3))).ravel()
        s.set_state(m=np.ones(n * 8), x=x, v=np.zeros(n * 8 * 3))
        lib.check(lib.md_pimd_fast_fill_ENk_x(s.pimd, 1))
        fill = lambda: lib.check(lib.md_pimd_fill_VB_x(s.pimd))  # noqa: E731
        fill()
        g, _ = R.capture(fill)
        ms, _, _ = R.time([R.launcher(g)] * 10, [R.launcher(g)] * 3, clocks=False)
        lib.md_gb300_graph_free_x(g)
        out[str(n)] = round(ms * 1e3, 1)
        s.free()
    return {"us_per_fill_VB": out,
            "what": "md_pimd_fill_VB_x: both recursions (weights, block inverses, block solve), graph-replayed"}


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
    R = Runner(lib, dist, dev, args)

    def graph_form():
        g, kps = R.capture(step)
        ms, wall, clocks = R.time([R.launcher(g)] * args.steps, [R.launcher(g)] * max(3, args.warmup))
        lib.md_gb300_graph_free_x(g)
        return ms, kps, wall, clocks

    want = set(args.forms.split(","))
    forms = {}
    if "plain" in want:
        # plain FP64: the form that reproduces MD-Lab to 1e-10, with launch
        # shapes chosen by the FP64 autotuner for this system
        lib.check(lib.md_gb300_set_precision_x(0))
        bps, lay, tms = C.c_int(), C.c_int(), C.c_double()
        lib.check(lib.md_gb300_autotune_fp64_x(s.pimd, pair, 3, C.byref(bps), C.byref(lay), C.byref(tms)),
                  "FP64 autotuning")
        step()
        plain_ms, plain_kps, plain_wall, plain_clocks = graph_form()
        plain_prof = R.profile(step)
        fp64_peak = lib.md_gb300_fp64_peak_x()
        # every term in FP64 (MD_GB_PRECISION_FP64_STRICT), for comparison
        lib.check(lib.md_gb300_set_precision_x(2))
        step()
        strict_ms, _, _, strict_clocks = graph_form()
        strict_prof = R.profile(step)
        lib.check(lib.md_gb300_set_precision_x(0))
        step()
        forms["plain_fp64"] = {"value": ws * N * P / (plain_ms * 1e-3), "ms_per_step": plain_ms,
                               "kernels_per_step": plain_kps, "clocks": plain_clocks,
                               "autotuned": {"tile_blocks_per_sm": bps.value, "sk_layout": lay.value},
                               "kernel_ms_per_step": {k: v[0] for k, v in plain_prof.items()},
                               "roofline": roofline(plain_prof, fp64_peak, "fp64", split=True),
                               "arithmetic": "FP64, with the real-space images at alpha R >= 4 and the "
                                             "wave-vector columns of force weight below 1e-7 on the FP32 pipe",
                               "strict_fp64": {"ms_per_step": strict_ms, "clocks": strict_clocks,
                                               "kernel_ms_per_step": {k: v[0] for k, v in strict_prof.items()},
                                               "roofline": roofline(strict_prof, fp64_peak, "fp64")}}
    fp32_peak = lib.md_gb300_fp32_peak_x()
    if "recursion" in want:
        forms["recursion_vs_N"] = recursion_form(lib, R, args)
    if "two" in want:
        forms["two_species_fp64"] = two_species_form(lib, R, args, lib.md_gb300_fp64_peak_x())
        xmd_x.set_potentials(lib, coul_s=1.0, alpha=ALPHA_L / workload()[0], nsum=NSUM)
    if "mixed" in want:
        # mixed precision, converged Ewald
        import numpy as np

        def forces(mode):
            lib.check(lib.md_gb300_set_precision_x(mode))
            lib.check(lib.md_reset_force_x(s.sim))
            lib.check(lib.md_pimd_calc_pair_force_x(s.pimd, pair))
            return s.state()["f"]

        f64, f32 = forces(0), forces(1)
        ferr = float(np.max(np.abs(f32 - f64)) / np.max(np.abs(f64)))
        mixed_ms, mixed_kps, _, mixed_clocks = graph_form()
        mixed_prof = R.profile(step)
        forms["mixed_fp32_forces"] = {"value": ws * N * P / (mixed_ms * 1e-3), "ms_per_step": mixed_ms,
                                      "kernels_per_step": mixed_kps, "force_error_vs_fp64": ferr,
                                      "clocks": mixed_clocks,
                                      "kernel_ms_per_step": {k: v[0] for k, v in mixed_prof.items()}}
    if "truncated" in want:
        # FP32 forces with the reciprocal sum truncated to |n| <= NSUM_CHEAP
        # and no network: what the learned form adds its residual to
        lib.check(lib.md_gb300_set_precision_x(1))
        xmd_x.set_potentials(lib, coul_s=1.0, alpha=ALPHA_L / workload()[0], nsum=NSUM_CHEAP)
        step()  # the truncated sum's tables exist before the capture
        tr_ms, tr_kps, _, tr_clocks = graph_form()
        forms["truncated_fp32"] = {"value": ws * N * P / (tr_ms * 1e-3), "ms_per_step": tr_ms,
                                   "kernels_per_step": tr_kps, "clocks": tr_clocks, "nsum": NSUM_CHEAP}
        xmd_x.set_potentials(lib, coul_s=1.0, alpha=ALPHA_L / workload()[0], nsum=NSUM)
        lib.check(lib.md_gb300_set_precision_x(0))
        step()  # the converged tables back
    if "ensemble" in want:
        forms["ensemble_64"] = ensemble_form(lib, R, args)
    headline = next((k for k in ("plain_fp64", "mixed_fp32_forces", "two_species_fp64", "ensemble_64")
                     if k in forms), None)
    model = None
    if "learned_xi1" in want:
        # the same workload at xi = 1 (bosons): its own system, data and network
        s1 = make_system(lib, xi=1.0)
        step1 = lambda: xmd_x.md_step(lib, s1, DT, image=1, pair=pair, pbc=True)  # noqa: E731
        for _ in range(args.warmup):
            step1()
        m1, f1, p1, _ = learned_form(lib, R, s1, pair, step1, args, ws)
        f1["roofline"] = roofline(p1, fp32_peak, "fp32")
        f1["xi"] = 1.0
        forms["learned_fp32_xi1"] = f1
        m1.free()
        s1.free()
        lib.check(lib.md_gb300_set_precision_x(0))
    if "learned" in want:
        model, lform, lprof, lkps = learned_form(lib, R, s, pair, step, args, ws)
        lform["roofline"] = roofline(lprof, fp32_peak, "fp32")
        if "plain_fp64" in forms:
            lform["speedup_vs_plain_fp64"] = lform["value"] / forms["plain_fp64"]["value"]
        forms["learned_fp32"] = lform
        headline = "learned_fp32"
    H = forms[headline]
    # e2e through the C ABI, host structs authoritative every step: each step
    # the state goes back to page-locked host memory (md_simulation_sync_host_x
    # with read_only = 0) and up again (the step's first call, the periodic
    # wrap, uploads it), the step replays as a captured graph, and the
    # primitive estimator is read back.  The learned headline judges as in its
    # timed run: every JUDGE_EVERY-th step is followed by the FP64 judgement of
    # its configuration, so the e2e run covers JUDGE_EVERY steps.
    wrap = lambda: lib.check(lib.md_periodic_boundary_x(s.sim))  # noqa: E731
    if model is not None:
        model.detach(s)
        g_conv, _ = R.capture(step)
        model.attach(s, judge_every=0)
        g_main, _ = R.capture(step)
        ke = JUDGE_EVERY
    else:
        g_conv, g_main = None, R.capture(step)[0]
        ke = min(args.steps, args.e2e_steps)
    h2d = C.sizeof(lib.Particle) * N * P + C.sizeof(lib.Nhc) * s.sim.contents.Nf
    lib.check(lib.md_gb300_synchronize_x())
    barrier(dist)
    t0 = time.perf_counter()
    dropped = False
    for i in range(ke):
        if not lib.md_simulation_sync_host_x(s.sim, 0):  # device -> host, host authoritative
            raise RuntimeError(lib.err())
        wrap()  # uploads the host state (positions are already inside the box)
        lib.check(lib.md_gb300_graph_launch_x(g_conv if dropped else g_main, 1))
        if g_conv is not None and not dropped and i % JUDGE_EVERY == 0:
            dropped = judge_fails(model.judge(s), args)
        lib.check(lib.md_pimd_calc_VBN_energy_x(s.pimd, s.stats))
        s.take_energy()  # estimator read
    if not lib.md_simulation_sync_host_x(s.sim, 1):
        raise RuntimeError(lib.err())
    e2e_s = max_over_ranks(dist, (time.perf_counter() - t0) / ke)
    for g in (g_conv, g_main):
        if g is not None:
            lib.md_gb300_graph_free_x(g)
    kps = H.get("kernels_per_learned_step", H.get("kernels_per_step", H.get("kernels_per_launch", 0)))
    result = {"metric": METRIC, "value": H["value"], "unit": "bead-steps/s", "n_gpus": ws,
              "steps": H.get("steps_timed", args.steps), "warmup": args.warmup, "ms_per_step": H["ms_per_step"],
              "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
              "dtype": "fp32 forces + bf16/fp32 network (fp64 recursion, NHC, estimators)"
                       if headline == "learned_fp32" else "f64",
              "data": "synthetic (seeded uniform electron-gas configuration from the library's own "
                      "initial-condition routines; training data from plain runs of the same system)",
              "config": config(), "form": "learned+FP32" if headline == "learned_fp32" else "plain FP64",
              "gpu_launches": kps * H.get("steps_timed", args.steps), "forms": forms,
              "e2e": {"value": ws * N * P / e2e_s, "unit": "bead-steps/s", "h2d_bytes_per_step": h2d,
                      "d2h_bytes_per_step": h2d + 8, "steps": ke, "form": headline},
              "roofline": H.get("roofline", forms.get("plain_fp64", {}).get("roofline")),
              "clocks": H["clocks"]}
    if headline == "learned_fp32":
        result["delta_E_per_particle_Ha"] = H["delta_E_per_particle_Ha"]
        result["speedup_vs_plain_fp64"] = H.get("speedup_vs_plain_fp64")
    if rank == 0 and ws == 1 and not args.no_cpu:
        # the same CPU measurement as the reference arm: all host cores
        cores = os.cpu_count() or 1
        st, sample = cpu_step_estimate(cores, args.cpu_budget)
        result["cpu_baseline"] = {"value": N * P / st, "unit": "bead-steps/s", "cores": cores,
                                  "kind": "port", "sample": sample, "form": "plain FP64 (converged Ewald)",
                                  "reference_build": REFERENCE_BUILD}
    if model is not None:
        model.free()
    s.free()
    return result


# MD-Lab's own _nocl library cannot be timed here: its sources are not on
# the measuring host and a build of it from elsewhere does not run on this
# host's architecture, so both CPU figures time the oracle port (MD-Lab's
# _nocl step restated in C, pinned to fixtures recorded from MD-Lab's own
# build); MD-Lab's OpenCL build needs CL headers and a CPU OpenCL runtime,
# which this host lacks as well
REFERENCE_BUILD = ("oracle port timed: MD-Lab's own _nocl sources are not on this host; its POCL OpenCL "
                   "build is unavailable on this box (no CL headers or CPU OpenCL runtime).  Where the sources "
                   "are mounted, oracle/time_reference.py measured the port at 0.82x the _nocl build's time per "
                   "Ewald pair of this workload (one x86 core, identical forces), so the port stands in for the "
                   "reference build with about its speed")


def run_reference(args, rank):
    cores = os.cpu_count() or 1
    vals = []
    sample = ""
    t0 = time.perf_counter()
    for i in range(args.warmup + args.steps):
        st, sample = cpu_step_estimate(cores, args.cpu_budget / 4)
        if i >= args.warmup:
            vals.append(st)
    wall = time.perf_counter() - t0
    step_s = statistics.median(vals)
    v = N * P / step_s
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "bead-steps/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config(), "form": "plain FP64 (CPU oracle port)",
            "cpu_baseline": {"value": v, "unit": "bead-steps/s", "cores": cores, "kind": "port",
                             "sample": sample, "reference_build": REFERENCE_BUILD},
            "e2e": {"value": v, "unit": "bead-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "sampled": {"measured_wall_s": wall,
                        "note": "each step is a bounded sample of the full step (every stage but the Ewald "
                                "pairs on the full system, the Ewald pairs sampled); ms_per_step is the "
                                "full step's time extrapolated from it, so ms_per_step x steps exceeds the "
                                "run's wall time"}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-budget", type=float, default=8.0, help="seconds of CPU sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--forms", default="plain,two,recursion,mixed,truncated,ensemble,learned_xi1,learned",
                    help="forms to run (comma list of plain, two, recursion, mixed, truncated, ensemble, "
                         "learned_xi1, learned)")
    ap.add_argument("--learn-configs", type=int, default=3125,
                    help="configurations collected for training (x P bead slices)")
    ap.add_argument("--learn-steps", type=int, default=3000)
    ap.add_argument("--learn-batch", type=int, default=128, help="tiles of 128 rows per Adam step")
    ap.add_argument("--learn-lr", type=float, default=1e-3)
    ap.add_argument("--force-tol", type=float, default=1.0,
                    help="the judge drops the network when its force error exceeds this multiple of the "
                         "truncated sum's on the same configuration")
    ap.add_argument("--energy-tol", type=float, default=1e-4)
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
