"""Benchmark of the afivo-streamer hot path on one GB300.

Workload (the configuration the headline metric is quoted on): 2D
axisymmetric streamer, r in [0, 1 cm], z in [0, 2 cm], 16x16-cell boxes,
coarse grid 16x32, uniform to level 5 then 4 AMR levels around the streamer
channel (~0.56 M leaf cells, 9 levels); electrons + positive + negative ions
(mobility 0.03 m^2/Vs, diffusion 0.1 m^2/s, alpha(E) = 4.3e5 exp(-2e7/|E|),
eta = 2e3 1/m), 3-term Helmholtz photoionization (lambda 50/150/500 1/m),
applied field 1.5e6 V/m, Heun time steps of 5e-12 s.  A step is one time step
of the reference time loop: photoionization every 5 steps, state copy, two
forward-Euler stages (Koren fluxes + sources), and a Poisson solve to 1e-8
relative residual after each stage.

Metric: cell-updates/s = (smoother cell-updates of all V-cycles + transport
cell-updates) / time, for the mixed-precision path (FP32 V-cycle inside FP64
defect correction); the plain FP64 GPU path is timed beside it.  Inputs are
seeded synthetic data; the L2 cache is flushed between timed steps.

--impl reference times the CPU restatement of the same step (the oracle,
OpenMP on all host cores) on a bounded sample of the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "afivo-streamer_gb300"))

import afivo_gpu as ag  # noqa: E402
import afivo_tree as at  # noqa: E402
import streamer_model as sm  # noqa: E402

METRIC = "cell-updates/s & V-cycle ms at 1e-8 rel. residual, mixed vs FP64 on 1 GB300"
UNIT = "cell-updates/s"
VOLTAGE = -3e4          # 1.5e6 V/m over 2 cm
DT = 5e-12
PHOTOI_LAMBDA = np.array([50.0, 150.0, 500.0])          # 1/m
PHOTOI_COEFFS = np.array([1e-2, 5e-2, 1e-1]) * 1e4       # 1/m^2
PHOTOI_ETA_QUENCH = 0.05 * 0.038


def streamer_refine(base, radii, z_tail, z_head):
    def f(lvl, c, dr):
        if lvl < base:
            return np.ones(len(c), bool)
        R = radii[lvl - base]
        r, z = c[:, 0], c[:, 1]
        return (r < R) & (z > z_tail - R) & (z < z_head + R)
    return f


def workload_tree():
    return at.build_tree(2, 16, [16, 32], [1e-2, 2e-2], coord=ag.AFG_CYL, max_lvl=9,
                         refine=streamer_refine(5, [2e-3, 1e-3, 0.6e-3, 0.35e-3], 0.9e-2, 1.4e-2))


def workload_model():
    return sm.StreamerModel(2, alpha=sm.baseline_alpha, eta=sm.baseline_eta, photoi_modes=3)


def initial_state(tree, model, seed=12345):
    rng = np.random.default_rng(seed)
    cc = ag.new_cc(tree, model.n_var_cell)
    fc = ag.new_fc(tree, model.n_var_face)
    n2 = tree.n_cell + 2
    idx = np.arange(n2) - 0.5
    r = tree.r_min[:, 0][:, None, None] + idx[None, None, :] * tree.dr[:, 0][:, None, None]
    z = tree.r_min[:, 1][:, None, None] + idx[None, :, None] * tree.dr[:, 1][:, None, None]
    seed_n = 1e15 * np.exp(-(r ** 2 + (z - 1.2e-2) ** 2) / (2 * 0.5e-3 ** 2)) + 1e9
    noise = 1 + 1e-3 * rng.standard_normal(seed_n.shape)
    cc[:, model.species_iv[0] - 1] = seed_n * noise
    cc[:, model.species_iv[1] - 1] = seed_n
    cc[:, model.species_iv[2] - 1] = 0.0
    cc[:, model.i_phi - 1] = VOLTAGE * np.broadcast_to(z, seed_n.shape) / 2e-2
    return cc, fc


def work_per_step(ctr0, ctr1):
    return (ctr1["smoother_updates"] - ctr0["smoother_updates"]) + \
        (ctr1["transport_updates"] - ctr0["transport_updates"])


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{os.getpid()}.csv")
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(index), "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm_mhz, sm_max, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 8:
                continue
            try:
                sm_mhz.append(float(p[0]))
                sm_max = max(sm_max, float(p[1]))
            except ValueError:
                continue
            for n, v in zip(names, p[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm_mhz:
            return None
        return {"sm_mhz": float(np.median(sm_mhz)), "sm_max_mhz": sm_max, "reasons": sorted(reasons),
                "samples": len(sm_mhz)}


def run_gpu_arm(args, device):
    tree = workload_tree()
    model = workload_model()
    cc0, fc0 = initial_state(tree, model)
    ctx = ag.Context(device)
    ctx.tree_sync(tree, model.n_var_cell, model.n_var_face)
    results = {}
    for prec_name, prec in (("fp64", ag.FP64), ("mixed", ag.MIXED)):
        ctx.upload(cc0)
        ctx.upload_fc(fc0)
        run = sm.StreamerRun(ctx, tree, model, VOLTAGE, DT, precision=prec, max_rel_residual=1e-8,
                             num_vcycles=30, photoi=(PHOTOI_LAMBDA, PHOTOI_COEFFS, PHOTOI_ETA_QUENCH))
        run.setup()
        run.initial_field()
        for _ in range(args.warmup):
            run.step()
        ctx.sync()
        times, work, vcycles = [], 0, 0
        clocks = Clocks(device) if prec_name == "mixed" else None
        c0 = ctx.counters()
        for _ in range(args.steps):
            ctx.flush_l2(256 << 20)
            ctx.event_record(0)
            run.step()
            ctx.event_record(1)
            times.append(ctx.event_elapsed(0, 1))
            vcycles += run.last["vcycles"]
        c1 = ctx.counters()
        clk = clocks.stop() if clocks else None
        work = work_per_step(c0, c1)
        t_ms = float(np.sum(times))
        res = dict(ms_per_step=t_ms / args.steps, value=work / (t_ms * 1e-3), vcycles_per_step=vcycles / args.steps,
                   launches_per_step=(c1["launches"] - c0["launches"]) / args.steps,
                   vcycle_ms=None, clocks=clk, work_per_step=work / args.steps)
        # V-cycle time: one more solve with the same state, per V-cycle
        ctx.sync()
        ctx.event_record(2)
        n, _ = run.field(0, True)
        ctx.event_record(3)
        res["vcycle_ms"] = ctx.event_elapsed(2, 3) / max(1, n)
        results[prec_name] = (res, run)
    # per-kernel-class device time during one mixed step
    run = results["mixed"][1]
    kstats = {}
    for cls, name in ((ag.KT_GSRB, "gsrb"), (ag.KT_GHOST, "ghost"), (ag.KT_FLUX, "flux"), (ag.KT_UPDATE, "update")):
        ctx.kernel_timing(cls)
        run.step()
        n, ms, by = ctx.kernel_stats()
        kstats[name] = dict(launches=n, ms=ms, bytes=by)
    ctx.kernel_timing(ag.KT_NONE)
    # end to end through the public API: host state in, host state out
    species_ivs = [iv for iv in model.species_iv]
    host = ag.new_cc(tree, model.n_var_cell)
    ctx.download(host)
    out = np.zeros_like(host)
    ctx.sync()
    h2d = d2h = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.upload(host, species_ivs)
        run.step()
        ctx.download(out, species_ivs + [model.i_electric_fld])
    e2e_s = time.perf_counter() - t0
    S = int(np.prod(host.shape[2:]))
    h2d = len(species_ivs) * tree.n_boxes * S * 8
    d2h = (len(species_ivs) + 1) * tree.n_boxes * S * 8
    work_e2e = results["mixed"][0]["work_per_step"] * args.steps
    e2e = dict(value=work_e2e / e2e_s, unit=UNIT, h2d_bytes_per_step=h2d, d2h_bytes_per_step=d2h,
               ms_per_step=1e3 * e2e_s / args.steps)
    launches = ctx.counters()["launches"]
    ctx.close()
    return tree, results, kstats, e2e, launches


def oracle_step_runner(tree, model):
    """CPU restatement of the same step (test/baseline infrastructure)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    o = oracle.Oracle(tree, model.n_var_cell, model.n_var_face)
    o.transport_setup(model.transport_desc())
    D = tree.ndim
    o.set_cc_methods(model.i_electric_fld, *model.electric_fld_gc())
    for s in range(len(model.species)):
        for st in range(model.n_states):
            o.set_cc_methods(model.species_iv[s] + st, [model.bc_species] * (2 * D), None, ag.RB_INTERP_LIM)
    o.set_cc_methods(model.i_photo, *model.photo_gc())
    o.mg_setup(0, model.field_mg(VOLTAGE))
    for n, d in enumerate(model.helmholtz_mg(PHOTOI_LAMBDA)):
        o.mg_setup(1 + n, d)
    L = 2e-2
    min_dr = float(np.min(tree.dr[tree.lvl_ids[-1][0] - 1]))
    leaves = np.concatenate(tree.lvl_leaves) - 1
    n2 = tree.n_cell + 2
    ncell_leaf = len(leaves) * tree.n_cell ** D
    level_cells = [len(tree.lvl_ids[l]) * tree.n_cell ** D for l in range(tree.highest_lvl)]
    vcycle_updates = 4 * sum(level_cells[1:])

    def field(cc, fc, s_in):
        o.field_set_rhs(cc, model.i_rhs, s_in)
        max_rhs = o.maxabs(cc, model.i_rhs)
        thr = max(1e-6, max_rhs * 1e-8, 1e-10 * abs(VOLTAGE) / (L * min_dr))
        n, _ = o.mg_solve(cc, 0, thr, 30)
        o.field_from_potential(cc, fc, model.i_phi)
        return n

    def step(cc, fc, it):
        work = 0
        if it % 5 == 0:
            o.photoi_source(cc, PHOTOI_ETA_QUENCH, model.i_rhs)
            cc[:, model.i_photo - 1] = 0
            max_rhs = max(o.maxabs(cc, model.i_rhs), np.sqrt(np.finfo(float).eps))
            for n in range(3):
                for i in range(10):
                    r = o.mg_fmg(cc, 1 + n, True, True)
                    work += sum(4 * sum(level_cells[1:l]) for l in range(1, tree.highest_lvl + 1))
                    if r / max_rhs < 1e-2:
                        break
                cc[leaves, model.i_photo - 1] -= PHOTOI_COEFFS[n] * cc[leaves, model.i_modes[n] - 1]
        for s in range(len(model.species)):
            cc[:, model.species_iv[s] + model.n_states - 2] = cc[:, model.species_iv[s] - 1]
        o.flux_upwind(cc, fc, 0)
        o.update_densities(cc, fc, DT, 0, [0], [1.0], 1)
        nv = field(cc, fc, 1)
        o.flux_upwind(cc, fc, 1)
        o.update_densities(cc, fc, 0.5 * DT, 1, [0, 1], [0.5, 0.5], 0, True)
        nv += field(cc, fc, 0)
        work += nv * vcycle_updates + 2 * ncell_leaf * len(model.species)
        return work

    def init(cc, fc):
        o.gc(cc, model.i_phi, 0, True)
        o.field_set_rhs(cc, model.i_rhs, 0)
        for _ in range(20):
            r = o.mg_fmg(cc, 0, True, False)
        o.field_from_potential(cc, fc, model.i_phi)

    return init, step


def run_cpu(steps, warmup=1):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    cores = os.cpu_count() or 1
    oracle.set_num_threads(cores)
    tree = workload_tree()
    model = workload_model()
    cc, fc = initial_state(tree, model)
    init, step = oracle_step_runner(tree, model)
    init(cc, fc)
    it = 0
    for _ in range(warmup):
        step(cc, fc, it)
        it += 1
    work, t0 = 0, time.perf_counter()
    for _ in range(steps):
        work += step(cc, fc, it)
        it += 1
    dt = time.perf_counter() - t0
    return work / dt, cores, dt / steps


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=1)
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    config = {"workload": "2D axisymmetric streamer, 16^2 boxes, coarse 16x32, 9 levels (~0.56 M leaf cells), "
                          "3 species, 3 Helmholtz photoionization modes, Heun dt=5e-12 s, Poisson to 1e-8 rel.",
              "l2": "flushed between timed steps (256 MiB write)", "parallelism": "replicas" if world > 1 else "1 GPU"}
    if args.impl == "reference":
        if rank != 0:
            return
        v, cores, sps = run_cpu(max(1, args.steps), warmup=min(1, args.warmup))
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": max(1, args.steps), "warmup": min(1, args.warmup), "ms_per_step": 1e3 * sps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{max(1, args.steps)} full steps of the workload on the CPU oracle"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    tree, results, kstats, e2e, launches = run_gpu_arm(args, local)
    mixed, fp64 = results["mixed"][0], results["fp64"][0]
    ms = mixed["ms_per_step"]
    value = mixed["value"]
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        value = world * mixed["work_per_step"] / (ms * 1e-3)
    peak, peak_kind = peaks()
    dom = max(kstats, key=lambda k: kstats[k]["ms"])
    ks = kstats[dom]
    achieved = ks["bytes"] / (ks["ms"] * 1e-3) / 1e9 if ks["ms"] > 0 else 0.0
    cpu = None
    if rank == 0 and world == 1 and args.cpu_steps > 0:
        v, cores, sps = run_cpu(args.cpu_steps, warmup=0)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{args.cpu_steps} full step(s) of the same workload on the CPU oracle (OpenMP)"}
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic (seeded)", "config": config,
            "precision_split": {
                "mixed": {k: mixed[k] for k in ("ms_per_step", "value", "vcycles_per_step", "vcycle_ms",
                                                "launches_per_step")},
                "fp64": {k: fp64[k] for k in ("ms_per_step", "value", "vcycles_per_step", "vcycle_ms",
                                               "launches_per_step")},
                "speedup_mixed_vs_fp64": fp64["ms_per_step"] / mixed["ms_per_step"]},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": None},
            "kernel_classes": kstats,
            "cpu_baseline": cpu, "e2e": e2e, "clocks": mixed["clocks"],
            "gpu_launches": int(mixed["launches_per_step"] * args.steps),
        }))


if __name__ == "__main__":
    main()
