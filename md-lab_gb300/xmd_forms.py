"""The electron-gas step's arithmetic forms, compared with the FP64 form.

Every form keeps positions, the exchange recursion, the springs, the
thermostat and every estimator in FP64; they differ in the pair and Ewald
forces and the pair energy:

  fp64       FP64 real-space tiles and reciprocal sum over |n| <= nsum
  mixed      FP32 real-space tiles and FP32 phase products (double-float
             structure factors), reciprocal sum over |n| <= nsum
  truncated  as mixed, reciprocal sum truncated to |n| <= nsum_cheap
  learned    truncated plus the residual network (md_gb300_ewald_model_*_x),
             trained here on configurations of the system's own runs

Two measurements:

  same_configuration  along one FP64 trajectory, at every `compare_every`-th
      step, each form's forces, pair energy and virial estimator on the same
      configuration against FP64's: largest and mean errors;
  trajectories        each form's own trajectory of `steps` steps from one
      equilibrated configuration, sampled every `every` steps after the
      first `discard` fraction: block averages (mean and standard error over
      `blocks` blocks) of the primitive and virial total-energy estimators
      (exchange estimator plus pair energy; the virial estimator from the
      pair forces) and of the pair energy, and whether each form's mean lies
      within `sigmas` combined standard errors of FP64's.  A second FP64
      run from the same configuration with every position moved by one
      unit in the last place ("fp64_replica") shows how far two runs of the
      same form differ by chaos alone.

The learned trajectory is judged every `judge_every` steps against the
converged FP64 reciprocal sum; a judgement where the network's force error
exceeds the truncated sum's on the same configuration, or its energy error
per particle exceeds `energy_tol`, drops the network for the rest of that
run (the converged mixed form continues).

    python md-lab_gb300/xmd_forms.py [--steps 10000] [--xi 0.5 1.0]

prints one JSON object per xi.  Needs a GPU; the library is loaded from
md-lab_gb300/lib (build it first).
"""
import argparse
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)
import xmd_x  # noqa: E402

FORMS = ("fp64", "mixed", "truncated", "learned")
RUNS = FORMS + ("fp64_replica",)


class Ueg:
    """The spin-polarised electron gas at (N, P, rs, theta, xi) with Ewald
    alpha = alpha_L / L, built by the library's own initial-condition
    routines."""

    def __init__(self, lib, N=512, P=64, rs=1.0, theta=0.5, xi=0.5, nsum=10, nsum_cheap=3, alpha_L=5.6, dt=0.01,
                 seed=2024):
        self.lib, self.N, self.P, self.xi, self.dt = lib, N, P, xi, dt
        self.nsum, self.nsum_cheap = nsum, nsum_cheap
        self.box = (4 * math.pi * N / 3) ** (1 / 3) * rs
        self.T = theta * 0.5 * (6 * math.pi ** 2 * N / self.box ** 3) ** (2 / 3)
        self.alpha = alpha_L / self.box
        s = xmd_x.PimdSystem(lib, N, P, xi, self.T, box=self.box)
        lib.md_set_seed_x(seed)
        lib.md_init_particle_mass_x(s.sim, 1.0, 0, N * P)
        c = (xmd_x.C.c_double * 3)(*([self.box / 2] * 3))
        Lv = (xmd_x.C.c_double * 3)(*([self.box] * 3))
        lib.md_pimd_init_particle_uniform_pos_x(s.pimd, c, Lv, 0.05 * rs)
        lib.md_init_maxwell_vel_x(s.sim, self.T)
        lib.md_init_nhc_x(s.sim, lib.md_get_quick_Q_x(self.T, s.pimd.contents.omegaP), 0, s.sim.contents.Nf, 0.0)
        self.s = s
        self.model = None
        self.pair = lib.fn("md_coulomb_3d_ewald_force_x")
        self.energy_fn = lib.fn("md_coulomb_3d_ewald_energy_x")
        self.set_form("fp64")

    def set_form(self, form):
        lib = self.lib
        if self.model is not None:
            self.model.detach(self.s)
        lib.check(lib.md_gb300_set_precision_x(0 if form == "fp64" else 1))
        xmd_x.set_potentials(lib, coul_s=1.0, alpha=self.alpha,
                             nsum=self.nsum_cheap if form == "truncated" else self.nsum)
        if form == "learned":
            self.model.attach(self.s, judge_every=0)
        self.form = form

    def step(self):
        xmd_x.md_step(self.lib, self.s, self.dt, image=1, pair=self.pair, pbc=True)

    def forces(self):
        """the current form's forces at the current positions, into f"""
        lib, s = self.lib, self.s
        ck = lib.check
        ck(lib.md_reset_force_x(s.sim))
        ck(lib.md_pimd_fast_fill_ENk_x(s.pimd, 1))
        ck(lib.md_pimd_fill_VB_x(s.pimd))
        ck(lib.md_pimd_fast_fill_force_VB_x(s.pimd, 1))
        ck(lib.md_pimd_calc_pair_force_x(s.pimd, self.pair))

    def estimators(self):
        """(primitive exchange estimator, virial exchange estimator, pair
        energy) at the current positions, in the current form.  The virial
        estimator reads the physical (pair) forces alone: f holds only
        them while it runs, and the step's total forces are put back after."""
        lib, s = self.lib, self.s
        ck = lib.check
        ck(lib.md_pimd_calc_VBN_energy_x(s.pimd, s.stats))
        ep = s.take_energy()
        ck(lib.md_pimd_fast_fill_ENk2_x(s.pimd, 1))
        ck(lib.md_reset_force_x(s.sim))
        ck(lib.md_pimd_calc_pair_force_x(s.pimd, self.pair))
        ck(lib.md_pimd_calc_vi_virial_energy_x(s.pimd, s.stats, 1))
        ev = s.take_energy()
        ck(lib.md_pimd_calc_pair_energy_x(s.pimd, self.energy_fn, s.stats))
        epair = s.take_energy()
        self.forces()
        return ep, ev, epair

    def train(self, configs, adam_steps, batch_tiles=128, lr=1e-3, seed=7):
        """collect `configs` configurations of a converged mixed-form run (the
        FP64 converged and truncated sums of each as targets) and train"""
        lib = self.lib
        self.set_form("mixed")
        self.model = xmd_x.EwaldModel(lib, self.s, nsum_cheap=self.nsum_cheap, capacity=configs, seed=seed)
        t0 = time.perf_counter()
        for _ in range(configs):
            self.step()
            self.model.collect(self.s)
        lib.check(lib.md_gb300_synchronize_x())
        t1 = time.perf_counter()
        loss = self.model.train(adam_steps, batch_tiles, lr)
        return {"configurations": configs, "bead_slice_configurations": configs * self.P, "adam_steps": adam_steps,
                "final_loss": loss, "collect_s": t1 - t0, "train_s": time.perf_counter() - t1}

    def save(self):
        return self.s.state()

    def restore(self, st):
        self.s.set_state(x=st["x"], v=st["v"], f=st["f"], theta=st["theta"], vtheta=st["vtheta"])

    def free(self):
        if self.model is not None:
            self.model.free()
        self.s.free()


def block_stats(v, blocks):
    v = np.asarray(v, dtype=np.float64)
    per = len(v) // blocks
    if per < 1:
        return float(v.mean()), float("nan")
    bm = v[:per * blocks].reshape(blocks, per).mean(axis=1)
    return float(v.mean()), float(bm.std(ddof=1) / math.sqrt(blocks))


def same_configuration(u, steps, compare_every):
    """FP64 trajectory; each form's forces, pair energy and virial estimator
    on the same configurations against FP64's"""
    N = u.N
    err = {f: {"force_max": [], "force_rms": [], "pair_energy_per_particle": [], "virial_estimator_rel": [],
               "primitive_estimator_rel": []} for f in FORMS[1:]}
    for it in range(1, steps + 1):
        u.set_form("fp64")
        u.step()
        if it % compare_every:
            continue
        ep0, ev0, epair0 = u.estimators()
        f0 = u.s.state()["f"]
        for form in FORMS[1:]:
            u.set_form(form)
            u.forces()
            f = u.s.state()["f"]
            ep, ev, epair = u.estimators()
            d = f - f0
            e = err[form]
            e["force_max"].append(float(np.abs(d).max() / np.abs(f0).max()))
            e["force_rms"].append(float(np.sqrt((d ** 2).mean() / (f0 ** 2).mean())))
            e["pair_energy_per_particle"].append(abs(epair - epair0) / N)
            e["virial_estimator_rel"].append(abs(ev - ev0) / abs(ev0))
            e["primitive_estimator_rel"].append(abs(ep - ep0) / abs(ep0))
        u.set_form("fp64")
        u.forces()  # the FP64 forces back for the next step's first half kick
    return {f: {k: {"max": max(v), "mean": float(np.mean(v))} for k, v in e.items()} for f, e in err.items()}


def trajectory(u, form, start, steps, every, judge_every, energy_tol, discard):
    if form == "fp64_replica":
        start = dict(start, x=np.nextafter(start["x"], np.inf))
        form = "fp64"
    u.restore(start)
    u.set_form(form)
    u.forces()  # the form's forces at the start, for the first half kick
    samples, judged, reverted_at = [], [], None
    t0 = time.perf_counter()
    for it in range(1, steps + 1):
        u.step()
        if form == "learned" and reverted_at is None and it % judge_every == 0:
            j = u.model.judge(u.s)
            judged.append(j)
            if j["force_err"] > j["force_err_truncated"] or j["energy_err"] > energy_tol:
                reverted_at = it
                u.set_form("mixed")
        if it % every == 0 and it > discard * steps:
            samples.append(u.estimators())
    u.lib.check(u.lib.md_gb300_synchronize_x())
    out = {"steps": steps, "samples": len(samples), "wall_s": time.perf_counter() - t0}
    if form == "learned":
        keys = ("force_err", "energy_err", "force_err_truncated", "energy_err_truncated")
        out["judged"] = len(judged)
        out["judged_force_err"] = [j["force_err"] for j in judged]
        out["judged_energy_err"] = [j["energy_err"] for j in judged]
        out["reverted_at_step"] = reverted_at
        if judged:
            out["judgements"] = {k: {"max": max(j[k] for j in judged), "mean": float(np.mean([j[k] for j in judged]))}
                                 for k in keys}
    return out, np.array(samples)


def validate(lib, xi=0.5, steps=10000, every=10, blocks=10, equil=2000, compare_steps=500, compare_every=50,
             configs=3125, adam_steps=3000, judge_every=50, energy_tol=1e-4, sigmas=3.0, discard=0.2, N=512, P=64,
             seed=2024, runs=RUNS, samples_out=None):
    u = Ueg(lib, N=N, P=P, xi=xi, seed=seed)
    try:
        u.set_form("mixed")
        for _ in range(equil):  # equilibration, converged sum
            u.step()
        training = u.train(configs, adam_steps)
        u.set_form("fp64")
        for _ in range(100):
            u.step()
        start = u.save()
        same = same_configuration(u, compare_steps, compare_every) if compare_steps > 0 else {}
        traj, means, series = {}, {}, {}
        for form in runs:
            info, smp = trajectory(u, form, start, steps, every, judge_every, energy_tol, discard)
            series[form] = smp
            e_prim = smp[:, 0] + smp[:, 2]
            e_vir = smp[:, 1] + smp[:, 2]
            stats = {"E_primitive": block_stats(e_prim, blocks), "E_virial": block_stats(e_vir, blocks),
                     "E_pair": block_stats(smp[:, 2], blocks)}
            info["estimators"] = {k: {"mean": m, "err": e} for k, (m, e) in stats.items()}
            traj[form] = info
            means[form] = stats
        if samples_out:
            np.savez(samples_out, **series)
        for form in [r for r in runs if r != "fp64" and "fp64" in runs]:
            agree = {}
            for k in ("E_primitive", "E_virial", "E_pair"):
                (m, e), (m0, e0) = means[form][k], means["fp64"][k]
                z = abs(m - m0) / math.sqrt(e * e + e0 * e0) if e > 0 or e0 > 0 else float("inf")
                agree[k] = {"difference": m - m0, "sigmas": z, "within": bool(z <= sigmas)}
            traj[form]["vs_fp64"] = agree
        return {"system": {"N": N, "P": P, "rs": 1.0, "theta": 0.5, "xi": xi, "T": u.T, "box": u.box,
                           "ewald_alpha": u.alpha, "nsum": u.nsum, "nsum_cheap": u.nsum_cheap, "dt": u.dt},
                "training": training, "same_configuration": same, "trajectories": traj,
                "settings": {"steps": steps, "every": every, "blocks": blocks, "equil": equil, "discard": discard,
                             "compare_steps": compare_steps, "compare_every": compare_every,
                             "judge_every": judge_every, "energy_tol": energy_tol, "sigmas": sigmas}}
    finally:
        lib.md_gb300_set_precision_x(0)
        u.free()


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--xi", type=float, nargs="+", default=[0.5, 1.0])
    ap.add_argument("--steps", type=int, default=10000)
    ap.add_argument("--every", type=int, default=10)
    ap.add_argument("--blocks", type=int, default=10)
    ap.add_argument("--equil", type=int, default=2000)
    ap.add_argument("--compare-steps", type=int, default=500)
    ap.add_argument("--configs", type=int, default=3125)
    ap.add_argument("--adam-steps", type=int, default=3000)
    ap.add_argument("--runs", default=",".join(RUNS), help="comma list of " + ", ".join(RUNS))
    ap.add_argument("--samples", default=None, help="write each run's samples to this .npz (one file per xi)")
    args = ap.parse_args()
    lib = xmd_x.load(3, 4)
    for xi in args.xi:
        res = validate(lib, xi=xi, steps=args.steps, every=args.every, blocks=args.blocks, equil=args.equil,
                       compare_steps=args.compare_steps, configs=args.configs, adam_steps=args.adam_steps,
                       runs=tuple(args.runs.split(",")),
                       samples_out=args.samples.replace(".npz", f"_xi{xi}.npz") if args.samples else None)
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
