"""Benchmark of the afivo-streamer hot path on one GB300.

A step is one time step of the reference's time loop over the whole tree:
photoionization every 5 steps (3-term Helmholtz, FMG), copy of the state,
two forward-Euler stages of Heun's method (Koren-limited drift-diffusion
fluxes with consistent coarse fluxes, reaction sources) and a Poisson solve
to 1e-8 relative residual after each stage.

Workloads (seeded synthetic inputs, afivo-streamer_gb300/workloads.py):

* ``3d`` (default; the configuration the headline metric is quoted on): 3D
  streamer in a 3 cm cube, 8^3-cell boxes, 12 levels, 221,129 boxes,
  ~99 M leaf cells / ~113 M cells; 5 species with 8 k13-form reactions;
  applied field 1.5e6 V/m, dt = 5e-12 s.
* ``cyl2d``: 2D axisymmetric streamer, 16^2-cell boxes, 9 levels,
  2,918 boxes, ~0.56 M leaf cells; 3 species with tabulated rates.
* ``cart2d``: the plain 2D Cartesian method on a uniform 256^2 grid (341
  boxes of 16^2 cells), forward Euler, Poisson to 1e-10 relative residual.

Metric: cell-updates/s = (smoother cell-updates of every V-cycle + leaf cells
x species per transport stage) / time.  `value` is the mixed-precision path
(FP32 V-cycles inside FP64 defect correction, FP64 transport) with the state
resident in HBM, CUDA events around each step and a 256 MiB L2 flush between
steps; the plain FP64 path is timed beside it.  `e2e` runs the same steps
through the C-ABI with the state in page-locked host memory: each step
uploads the species densities, advances, and downloads the densities and
|E|, inside the timed region (the densities' download overlaps the step's
final field solve, which does not write them).

`--impl reference` and `cpu_baseline` time the CPU restatement of the same
step (C++/OpenMP on all host cores) on the same tree when the host has the
memory for it (the 3D tree needs ~55 GB on the host), otherwise on the same
construction two levels coarser, stated in `config.workload`.
`error_mixed_vs_fp64` compares the two GPU paths after the same steps from
the same initial state: relative maximum over leaf cells of |mixed - FP64|
divided by the FP64 path's maximum, for phi, |E| and every species.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "afivo-streamer_gb300"))

import afivo_gpu as ag  # noqa: E402
import streamer_model as sm  # noqa: E402
import workloads  # noqa: E402

METRIC = "cell-updates/s & V-cycle ms at 1e-8 rel. residual, mixed vs FP64 on 1 GB300"
UNIT = "cell-updates/s"
CONFIG_TEXT = {
    "3d": "3D streamer, 3 cm cube, 8^3 boxes, 12 levels, 221129 boxes (~99 M leaf / ~113 M cells), 5 species, "
          "8 k13 reactions, 3 Helmholtz photoionization modes, Heun dt=5e-12 s, Poisson to 1e-8 rel.",
    "cyl2d": "2D axisymmetric streamer, 16^2 boxes, 9 levels, 2918 boxes (~0.56 M leaf cells), 3 species, "
             "3 Helmholtz photoionization modes, Heun dt=5e-12 s, Poisson to 1e-8 rel.",
    "cart2d": "2D Cartesian 1 cm^2, uniform 256^2 grid of 16^2 boxes, 5 levels, 341 boxes, electrons + ions, "
              "alpha(E) ionization, forward Euler dt=1e-12 s, Poisson to 1e-10 rel.",
    "poisson3d": "3D Poisson + 3 Helmholtz modes: 2 cm cube, 8^3 boxes, 10 levels (uniform to level 5, 5 AMR "
                 "levels around a sigma=0.3 mm Gaussian seed), 80665 boxes, ~41 M cells; Poisson to 1e-8 rel.",
    "batch": "256 independent 2D axisymmetric Poisson + transport instances (1 cm^2, 16^2 boxes, uniform "
             "grids with sides drawn from {64,128,256,512}, voltages 15-35 kV, seed amplitudes 1e13-1e16), "
             "one forest in one context, 3 species, Heun dt=5e-12 s, Poisson to 1e-8 rel. per instance",
}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix="afg_clocks_", suffix=".csv")
        os.close(fd)
        try:
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
        try:
            os.unlink(self.path)
        except OSError:
            pass
        if not sm_mhz:
            return None
        return {"sm_mhz": float(np.median(sm_mhz)), "sm_max_mhz": sm_max, "reasons": sorted(reasons),
                "samples": len(sm_mhz)}


def work_of(c0, c1):
    return (c1["smoother_updates"] - c0["smoother_updates"]) + (c1["transport_updates"] - c0["transport_updates"])


def initial_host_state(w, tree, model):
    return w.initial_host_state(tree, model)


def cuda_profiler(on):
    """cudaProfilerStart/Stop of the CUDA runtime the library uses (ncu
    --profile-from-start off captures only the bracketed launches)."""
    import ctypes
    rt = ctypes.CDLL("libcudart.so.13")
    rc = rt.cudaProfilerStart() if on else rt.cudaProfilerStop()
    if rc != 0:
        raise RuntimeError(f"cudaProfiler{'Start' if on else 'Stop'} failed: {rc}")


def problem(args, w):
    """(tree, model, host state, its variables, voltage(s), box instances,
    instance trees) of a workload; the batched workload is a forest."""
    if isinstance(w, workloads.BatchCyl2d):
        tree, box_inst, trees = w.forest()
        model = w.model()
        H, ivs = w.initial_host_state(trees, model)
        return tree, model, H, ivs, w.voltages, box_inst, trees
    tree = w.tree(coarsen=args.coarsen)
    model = w.model()
    H, ivs = initial_host_state(w, tree, model)
    return tree, model, H, ivs, w.voltage, None, None


def run_poisson3d(args, device, config):
    """The 3D Poisson + Helmholtz configuration: per precision, a Poisson
    solve from scratch (FMG start + V-cycles to 1e-8 relative residual), K
    further solve iterations timed on their own (V-cycle ms; in the mixed
    path one iteration = FP32 V-cycle + FP64 defect correction), the
    smoother's kernel time and algorithmic GB/s over those iterations, and
    the three Helmholtz modes (photoionization, FMG to 1e-2); the mixed
    results against the FP64 ones (phi, |E| and the photoionization source on
    the leaves)."""
    w = workloads.Poisson3d()
    tree = w.tree(coarsen=args.coarsen)
    model = w.model()
    H, ivs = w.initial_host_state(tree, model)
    ctx = new_context(args, device)
    K = max(3, args.steps)
    lam, coeffs, coeff = w.photoi_lambda, w.photoi_coeffs, w.photoi_eta_quench
    out, fields = {}, {}
    leaves = np.concatenate(tree.lvl_leaves) - 1
    n2 = tree.n_cell + 2
    inner = (slice(None),) + (slice(1, n2 - 1),) * tree.ndim
    for name, prec in (("fp64", ag.FP64), ("mixed", ag.MIXED)):
        ctx.tree_sync(tree, model.n_var_cell, model.n_var_face)
        ctx.upload_vars(H, ivs)
        run = sm.StreamerRun(ctx, tree, model, w.voltage, w.dt, precision=prec, **w.run_kwargs())
        run.setup()
        for _ in range(args.warmup):           # graphs captured, tuning done
            ctx.gc(model.i_phi, 0, True)
            run.field(0, False)
            ctx.photoi_helmh(coeff, run.mode_ids, coeffs, 1e-2, 10)
        ctx.sync()
        ctx.flush_l2(256 << 20)
        ctx.event_record(0)
        n_solve, r_solve = run.field(0, False)
        ctx.event_record(1)
        solve_ms = ctx.event_elapsed(0, 1)
        c0 = ctx.counters()
        ctx.flush_l2(256 << 20)
        ctx.event_record(2)
        ctx.mg_solve(0, 0.0, K, allow_noconv=True)
        ctx.event_record(3)
        it_ms = ctx.event_elapsed(2, 3) / K
        work = ctx.counters()["smoother_updates"] - c0["smoother_updates"]
        ctx.kernel_timing(ag.KT_GSRB)
        ctx.mg_solve(0, 0.0, K, allow_noconv=True)
        gl, gms, gby = ctx.kernel_stats()
        ctx.kernel_timing(ag.KT_NONE)
        ctx.flush_l2(256 << 20)
        ctx.event_record(4)
        ctx.photoi_helmh(coeff, run.mode_ids, coeffs, 1e-2, 10)
        ctx.event_record(5)
        photo_ms = ctx.event_elapsed(4, 5)
        cc = ag.new_cc(tree, model.n_var_cell)
        ctx.download(cc)
        fields[name] = {iv: cc[leaves, iv - 1][inner] for iv in (model.i_phi, model.i_electric_fld, model.i_photo)}
        out[name] = dict(solve_ms=solve_ms, solve_cycles=n_solve, solve_residual=r_solve, vcycle_ms=it_ms,
                         cell_updates_per_s=work / (it_ms * K * 1e-3),
                         smoother=dict(launches=gl, ms_per_vcycle=gms / K, algorithmic_gbs=gby / (gms * 1e-3) / 1e9),
                         photoi_3_modes_ms=photo_ms, tuning=ctx.tuning())
    ctx.close()
    err = {}
    for key, iv in (("phi", model.i_phi), ("E", model.i_electric_fld), ("photoi_source", model.i_photo)):
        a, b = fields["mixed"][iv], fields["fp64"][iv]
        err[key] = float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
    peak, peak_kind = peaks()
    sm32, sm64 = out["mixed"]["smoother"], out["fp64"]["smoother"]
    print(json.dumps({
        "metric": "V-cycle ms & smoother HBM GB/s, FP32 vs FP64 smoothers (3D Poisson + 3 Helmholtz modes)",
        "value": out["mixed"]["vcycle_ms"], "unit": "ms per V-cycle (mixed)", "higher_is_better": False,
        "n_gpus": 1, "steps": K, "warmup": args.warmup, "dtype": "f64+f32", "data": "synthetic (seeded)",
        "config": dict(config, boxes=tree.n_boxes, cells=tree.n_cells(), leaf_cells=tree.n_cells(True),
                       boxes_per_level=[len(x) for x in tree.lvl_ids]),
        "fp64": out["fp64"], "mixed": out["mixed"],
        "speedup_mixed_vs_fp64": {"vcycle": out["fp64"]["vcycle_ms"] / out["mixed"]["vcycle_ms"],
                                  "solve": out["fp64"]["solve_ms"] / out["mixed"]["solve_ms"],
                                  "photoi": out["fp64"]["photoi_3_modes_ms"] / out["mixed"]["photoi_3_modes_ms"]},
        "error_mixed_vs_fp64": err,
        "roofline": {"bound": "hbm", "kernel": "gsrb (FP32 smoother)", "achieved": sm32["algorithmic_gbs"],
                     "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": sm32["algorithmic_gbs"] / peak,
                     "fp64_smoother_frac": sm64["algorithmic_gbs"] / peak, "traffic": None},
    }))


def run_one_at_a_time(args, device, w, trees, model, H, ivs):
    """The batched workload's instances advanced one after another, each in
    its own context (mixed precision, the same steps and L2 flushes as the
    forest); returns cell-updates/s over the summed step times."""
    offs = np.cumsum([0] + [t.n_boxes for t in trees])
    t_ms, work = 0.0, 0
    for q, t in enumerate(trees):
        ctx = new_context(args, device)
        ctx.tree_sync(t, model.n_var_cell, model.n_var_face)
        ctx.upload_vars(H[offs[q]:offs[q + 1]], ivs)
        run = sm.StreamerRun(ctx, t, model, float(w.voltages[q]), w.dt, precision=ag.MIXED, **w.run_kwargs())
        run.setup()
        run.initial_field()
        for _ in range(args.warmup):
            run.step()
        c0 = ctx.counters()
        for _ in range(args.steps):
            ctx.flush_l2(256 << 20)
            ctx.event_record(0)
            run.step()
            ctx.event_record(1)
            t_ms += ctx.event_elapsed(0, 1)
        work += work_of(c0, ctx.counters())
        ctx.close()
    return dict(value=work / (t_ms * 1e-3), ms_per_step=t_ms / args.steps, work_per_step=work / args.steps,
                instances=len(trees))


def leaf_snapshot(ctx, tree, ivs):
    """Leaf-cell interiors of the variables ivs on the device: {iv: array}."""
    nc, D = tree.n_cell, tree.ndim
    leaves = np.concatenate(tree.lvl_leaves).astype(np.int64) - 1
    inner = (slice(None),) + (slice(1, nc + 1),) * D
    h = ag.new_cc(tree, 1)
    out = {}
    for iv in ivs:
        ctx.download_vars(h, [iv])
        out[iv] = np.ascontiguousarray(h[leaves, 0][inner])
    return out


def snapshot_vars(model):
    """(name, variable) pairs compared between the two GPU paths."""
    out = [("phi", model.i_phi), ("E", model.i_electric_fld)]
    out += [(sp.name, model.species_iv[s]) for s, sp in enumerate(model.species)]
    return out


def new_context(args, device):
    ctx = ag.Context(device)
    ctx.set_fp32_layout(getattr(args, "fp32_layout", "compact") == "compact")
    return ctx


def run_gpu_arm(args, device, w):
    tree, model, H, ivs, voltage, box_inst, trees = problem(args, w)
    ctx = new_context(args, device)
    results = {}
    if args.profile:
        arms = (("fp64", ag.FP64),) if args.profile_arm == "fp64" else (("mixed", ag.MIXED),)
    else:
        arms = (("fp64", ag.FP64), ("mixed", ag.MIXED))
    svars = snapshot_vars(model)
    snap64, accuracy = None, None
    for prec_name, prec in arms:
        ctx.tree_sync(tree, model.n_var_cell, model.n_var_face, box_inst=box_inst)     # zeroed pools
        ctx.upload_vars(H, ivs)
        run = sm.StreamerRun(ctx, tree, model, voltage, w.dt, precision=prec, **w.run_kwargs())
        run.setup()
        run.initial_field()
        for _ in range(args.warmup):
            run.step()
        ctx.sync()
        times, vcycles = [], 0
        clocks = Clocks(device) if prec_name == "mixed" or args.profile else None
        c0 = ctx.counters()
        if args.profile:
            cuda_profiler(True)
        photo_steps = []
        for _ in range(args.steps):
            photo_steps.append(run.photoi is not None and run.it % run.photoi_per_steps == 0)
            ctx.flush_l2(256 << 20)
            ctx.event_record(0)
            run.step()
            ctx.event_record(1)
            times.append(ctx.event_elapsed(0, 1))
            vcycles += run.last["vcycles"]
        if args.profile:
            ctx.sync()
            cuda_profiler(False)
        c1 = ctx.counters()
        clk = clocks.stop() if clocks else None
        work = work_of(c0, c1)
        t_ms = float(np.sum(times))
        res = dict(ms_per_step=t_ms / args.steps, value=work / (t_ms * 1e-3), vcycles_per_step=vcycles / args.steps,
                   launches=c1["launches"] - c0["launches"],
                   launches_per_step=(c1["launches"] - c0["launches"]) / args.steps,
                   clocks=clk, work_per_step=work / args.steps,
                   step_ms=[round(x, 3) for x in times],
                   photoi_step_ms=(float(np.mean([x for x, p in zip(times, photo_steps) if p]))
                                   if any(photo_steps) else None),
                   plain_step_ms=(float(np.mean([x for x, p in zip(times, photo_steps) if not p]))
                                  if not all(photo_steps) else None))
        # V-cycle time: one more solve of the current state, per V-cycle
        ctx.sync()
        ctx.event_record(2)
        n, _ = run.field(0, True)
        ctx.event_record(3)
        res["vcycle_ms"] = ctx.event_elapsed(2, 3) / max(1, n)
        results[prec_name] = (res, run)
        # the state after the same steps from the same initial state
        if not args.profile:
            if prec_name == "fp64":
                snap64 = leaf_snapshot(ctx, tree, [iv for _, iv in svars])
            else:
                accuracy = {}
                for name, iv in svars:
                    b = snap64.pop(iv)
                    a = leaf_snapshot(ctx, tree, [iv])[iv]
                    accuracy[name] = float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))
                    del a, b
                accuracy = {"rel_max_over_leaves": accuracy,
                            "after": f"the initial field solve, {args.warmup} warm-up and {args.steps} timed steps "
                                     f"and one more field solve, from the same initial state",
                            "field_target": 1e-6}
    if args.profile:
        tuning = ctx.tuning()
        ctx.close()
        return tree, results, {}, None, tuning, None
    tuning = ctx.tuning()
    # per-kernel-class device time during one mixed step (graphs off while
    # timing, events around every launch), against the device time of the
    # same step measured around it
    run = results["mixed"][1]
    ctx.sync()
    ctx.kernel_timing(ag.KT_ALL)
    ctx.event_record(2)
    run.step()
    ctx.event_record(3)
    step_ms = ctx.event_elapsed(2, 3)
    kstats = {}
    for name, (n, ms, by) in ctx.kernel_stats_all().items():
        kstats[name] = dict(launches=n, ms=ms, bytes=by, gbs=by / (ms * 1e-3) / 1e9 if ms > 0 else 0.0)
    ctx.kernel_timing(ag.KT_NONE)
    covered = sum(v["ms"] for v in kstats.values())
    kstats["_step"] = dict(ms=step_ms, covered_ms=covered, coverage=covered / step_ms if step_ms > 0 else 0.0,
                           note="one mixed step with events around every launch; classes sum to covered_ms")
    # device-side refinement on the state after the timed steps: box flags of
    # default_refinement (reference defaults) and the limited prolongation of
    # one variable into the finest level's boxes
    amr = None
    if trees is None:
        ctx.sync()
        t0 = time.perf_counter()
        flags = ctx.refine_flags(model.refine_desc())
        t_flags = time.perf_counter() - t0
        fine = tree.lvl_ids[-1]
        iv = model.species_iv[0] + model.n_states - 1   # the backup copy: scratch after the step
        ctx.event_record(2)
        ctx.prolong_limit(iv, fine, ag.LIMITER_MC)
        ctx.event_record(3)
        amr = dict(refine_flags_ms=1e3 * t_flags, boxes_do=int(np.sum(flags == ag.REF_DO)),
                   boxes_rm=int(np.sum(flags == ag.REF_RM)), prolong_limit_ms=ctx.event_elapsed(2, 3),
                   prolong_boxes=len(fine),
                   note="refine_flags_ms is wall clock through the C-ABI (list build, upload, kernel, "
                        "flags download); prolong_limit_ms device time for one variable")
    # the batched workload's instances one at a time, from the same initial
    # state (before the end-to-end run below overwrites the host state)
    one = run_one_at_a_time(args, device, w, trees, model, H, ivs) if trees is not None else None
    # end to end through the C-ABI: page-locked host state in, densities and |E| out
    species_ivs = list(model.species_iv)
    cols = list(range(1, 1 + len(species_ivs)))
    Eh = np.empty((tree.n_boxes, 1) + H.shape[2:])
    ctx.host_register(H)
    ctx.host_register(Eh)
    bpH, bpE = ag.box_pointers(H), ag.box_pointers(Eh)
    ctx.download_vars(H, species_ivs, cols=cols, bp=bpH)
    ctx.sync()
    c0 = ctx.counters()
    t_up = t_step = t_down = 0.0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ta = time.perf_counter()
        ctx.upload_vars(H, species_ivs, cols=cols, bp=bpH)
        tb = time.perf_counter()
        # the new densities go down while the field of the new state is solved
        run.step(after_update=lambda: ctx.download_vars_async(H, species_ivs, cols=cols, bp=bpH))
        ctx.sync()
        tc = time.perf_counter()
        ctx.download_vars(Eh, [model.i_electric_fld], bp=bpE)
        ctx.transfers_wait()
        td = time.perf_counter()
        t_up, t_step, t_down = t_up + tb - ta, t_step + tc - tb, t_down + td - tc
    e2e_s = time.perf_counter() - t0
    c1 = ctx.counters()
    ctx.host_unregister(H)
    ctx.host_unregister(Eh)
    S = int(np.prod(H.shape[2:]))
    h2d = len(species_ivs) * tree.n_boxes * S * 8
    d2h = (len(species_ivs) + 1) * tree.n_boxes * S * 8
    e2e = dict(value=work_of(c0, c1) / e2e_s, unit=UNIT, h2d_bytes_per_step=h2d, d2h_bytes_per_step=d2h,
               ms_per_step=1e3 * e2e_s / args.steps,
               upload_ms_per_step=1e3 * t_up / args.steps,
               step_and_species_download_ms_per_step=1e3 * t_step / args.steps,
               field_download_and_wait_ms_per_step=1e3 * t_down / args.steps,
               h2d_gbs=h2d / max(t_up / args.steps, 1e-12) / 1e9,
               transfer_path="zero-copy kernels on host boxes page-locked by afg_host_register; the species "
                             "download overlaps the step's final field solve (afg_cc_download_async)")
    ctx.close()
    if one is not None:
        e2e["one_at_a_time"] = one
    if amr is not None:
        e2e["amr"] = amr
    return tree, results, kstats, e2e, tuning, accuracy


def host_mem_available():
    """Bytes of host memory this process can still use (MemAvailable, capped
    by a cgroup v2 limit), or None if unknown."""
    avail = None
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    avail = int(line.split()[1]) * 1024
    except OSError:
        pass
    try:
        with open("/sys/fs/cgroup/memory.max") as f:
            lim = f.read().strip()
        with open("/sys/fs/cgroup/memory.current") as f:
            cur = int(f.read())
        if lim != "max":
            left = int(lim) - cur
            avail = left if avail is None else min(avail, left)
    except (OSError, ValueError):
        pass
    return avail


def cpu_state_bytes(tree, model):
    """Host bytes the CPU restatement holds for a tree: cell and face pools
    plus the initial-state array, with a quarter in reserve."""
    S = (tree.n_cell + 2) ** tree.ndim
    NF = (tree.n_cell + 1) ** tree.ndim
    cc = tree.n_boxes * model.n_var_cell * S * 8
    fc = tree.n_boxes * model.n_var_face * tree.ndim * NF * 8
    H = tree.n_boxes * (1 + len(model.species)) * S * 8
    return int(1.25 * (cc + fc) + H)


def cpu_tree(name, w, model):
    """The tree the CPU restatement runs: the workload's own when the host
    has the memory, else (3d) the same construction two levels coarser.
    Returns (tree, reduced)."""
    tree = w.tree()
    if name != "3d":
        return tree, False
    avail = host_mem_available()
    if avail is None or avail > cpu_state_bytes(tree, model):
        return tree, False
    del tree
    return w.tree(reduced=True), True


def run_cpu(name, steps, warmup=1, time_limit=None):
    """The CPU restatement of the step (oracle) on all host cores, on the
    workload's tree (cpu_tree).  Returns (cell-updates/s, cores, s/step,
    steps timed, sample text, reduced)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from oracle_streamer import OracleStreamerRun
    cores = os.cpu_count() or 1
    oracle.set_num_threads(cores)
    if name == "batch":
        return run_cpu_batch(steps, warmup, time_limit, cores) + (False,)
    w = workloads.WORKLOADS[name]()
    if name == "poisson3d":
        return run_cpu_poisson3d(w, steps, warmup, time_limit, cores) + (True,)
    model = w.model()
    tree, reduced = cpu_tree(name, w, model)
    cc = ag.new_cc(tree, model.n_var_cell)
    fc = ag.new_fc(tree, model.n_var_face)
    H, ivs = initial_host_state(w, tree, model)
    for v, iv in enumerate(ivs):
        cc[:, iv - 1] = H[:, v]
    del H
    run = OracleStreamerRun(tree, model, w.voltage, w.dt, **w.run_kwargs())
    run.setup()
    run.initial_field(cc, fc)
    for _ in range(warmup):
        run.step(cc, fc)
    work, done, t0 = 0, 0, time.perf_counter()
    while done < steps:
        work += run.step(cc, fc)
        done += 1
        if time_limit is not None and time.perf_counter() - t0 > time_limit:
            break
    dt = time.perf_counter() - t0
    ncells = tree.n_boxes * tree.n_cell ** tree.ndim
    coarser = ", the same construction two levels coarser: the host lacks the memory for the full tree"
    sample = (f"{done} step(s) after {warmup} warm-up step(s) of the {'reduced ' if reduced else ''}{name} tree "
              f"({tree.n_boxes} boxes, {ncells / 1e6:.2f} M cells{coarser if reduced else ''}"
              f") on the CPU restatement (C++/OpenMP, {cores} threads)")
    return work / dt, cores, dt / done, done, sample, reduced


def run_cpu_poisson3d(w, steps, warmup, time_limit, cores):
    """The 3D Poisson configuration on the CPU restatement: FP64 solve
    iterations (V-cycles) on the same construction two levels coarser."""
    from oracle_streamer import OracleStreamerRun
    tree = w.tree(coarsen=2)
    model = w.model()
    cc = ag.new_cc(tree, model.n_var_cell)
    fc = ag.new_fc(tree, model.n_var_face)
    H, ivs = w.initial_host_state(tree, model)
    for v, iv in enumerate(ivs):
        cc[:, iv - 1] = H[:, v]
    kw = w.run_kwargs()
    kw["photoi"] = None
    run = OracleStreamerRun(tree, model, w.voltage, w.dt, **kw)
    run.setup()
    run.initial_field(cc, fc)
    o = run.o
    work, done, t0 = 0, 0, time.perf_counter()
    while done < max(1, steps):
        o.mg_vcycle(cc, 0, True)
        work += run.vcycle_updates(tree.highest_lvl, run.field_desc)
        done += 1
        if time_limit is not None and time.perf_counter() - t0 > time_limit:
            break
    dt = time.perf_counter() - t0
    sample = (f"{done} FP64 V-cycle(s) of the poisson3d tree two levels coarser ({tree.n_boxes} boxes, "
              f"{tree.n_cells() / 1e6:.2f} M cells) on the CPU restatement (C++/OpenMP, {cores} threads)")
    return work / dt, cores, dt / done, done, sample


def run_cpu_batch(steps, warmup, time_limit, cores):
    """The batched workload on the CPU restatement: instances one after
    another (as the reference runs them), `steps` steps each, until the time
    bound is spent."""
    from oracle_streamer import OracleStreamerRun
    b = workloads.BatchCyl2d()
    model = b.model()
    work, t_run, done_inst, done_steps = 0, 0.0, 0, 0
    t_all = time.perf_counter()
    for q, w in enumerate(b.instances):
        tree = w.tree()
        H, ivs = w.initial_host_state(tree, model, seed=12345 + q)
        cc = ag.new_cc(tree, model.n_var_cell)
        fc = ag.new_fc(tree, model.n_var_face)
        for v, iv in enumerate(ivs):
            cc[:, iv - 1] = H[:, v]
        run = OracleStreamerRun(tree, model, w.voltage, b.dt, **b.run_kwargs())
        run.setup()
        run.initial_field(cc, fc)
        for _ in range(warmup):
            run.step(cc, fc)
        t0 = time.perf_counter()
        for _ in range(steps):
            work += run.step(cc, fc)
            done_steps += 1
        t_run += time.perf_counter() - t0
        done_inst += 1
        if time_limit is not None and time.perf_counter() - t_all > time_limit:
            break
    sample = (f"the first {done_inst} of {len(b.instances)} batched instances, one after another, {steps} step(s) "
              f"each after {warmup} warm-up step(s), on the CPU restatement (C++/OpenMP, {cores} threads)")
    return work / t_run, cores, t_run / max(1, done_steps), done_steps, sample


def combine_replicas(ms, work_per_step, world):
    """Whole-job figures of N independent replicas (one rank per GPU, an
    initialised process group): the step time is the maximum over the ranks
    and the value counts the work of all of them."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    return ms, world * work_per_step / (ms * 1e-3)


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
    ap.add_argument("--config", default="3d", choices=sorted(workloads.WORKLOADS) + ["batch"])
    ap.add_argument("--cpu-steps", type=int, default=10, help="CPU baseline sample steps (0 = skip)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="CPU baseline time bound")
    ap.add_argument("--coarsen", type=int, default=0,
                    help="3d only: the same tree construction this many levels coarser (smaller profiling cases)")
    ap.add_argument("--fp32-layout", default="compact", choices=["compact", "ghosted"],
                    help="layout of the FP32 correction buffers of the mixed solves")
    ap.add_argument("--profile", action="store_true",
                    help="one arm only (--profile-arm), timed steps bracketed by cudaProfilerStart/Stop; "
                         "no e2e or CPU baseline")
    ap.add_argument("--profile-arm", default="mixed", choices=["mixed", "fp64"],
                    help="the arm --profile runs")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    config = {"workload": CONFIG_TEXT[args.config] if args.coarsen == 0 else
              f"{CONFIG_TEXT[args.config]} -- coarsened by {args.coarsen} level(s)", "name": args.config,
              "fp32_layout": args.fp32_layout,
              "l2": "flushed between timed steps (256 MiB write)",
              "parallelism": "replicas" if world > 1 else "1 GPU"}
    if args.impl == "reference":
        if rank != 0:
            return
        warm = max(0, args.warmup)
        v, cores, sps, done, sample, reduced = run_cpu(args.config, max(1, args.steps), warmup=warm,
                                                       time_limit=300.0)
        if reduced:
            config["workload"] = f"{config['workload']} -- CPU sample: {sample}"
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": done, "warmup": warm, "ms_per_step": 1e3 * sps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "config": config,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.config == "poisson3d":
        if rank == 0:
            run_poisson3d(args, local, config)
        return
    w = workloads.BatchCyl2d() if args.config == "batch" else workloads.WORKLOADS[args.config]()
    tree, results, kstats, e2e, tuning, accuracy = run_gpu_arm(args, local, w)
    one = e2e.pop("one_at_a_time", None) if e2e else None
    amr = e2e.pop("amr", None) if e2e else None
    if args.profile:
        if rank == 0:
            print(json.dumps({"profile": True, "config": config,
                              args.profile_arm: results[args.profile_arm][0]}))
        return
    mixed, fp64 = results["mixed"][0], results["fp64"][0]
    ms = mixed["ms_per_step"]
    value = mixed["value"]
    if world > 1:
        ms, value = combine_replicas(ms, mixed["work_per_step"], world)
    peak, peak_kind = peaks()
    dom = max((k for k in kstats if not k.startswith("_")), key=lambda k: kstats[k]["ms"])
    ks = kstats[dom]
    achieved = ks["bytes"] / (ks["ms"] * 1e-3) / 1e9 if ks["ms"] > 0 else 0.0
    cpu = None
    if rank == 0 and world == 1 and args.cpu_steps > 0:
        v, cores, sps, done, sample, reduced = run_cpu(args.config, args.cpu_steps, warmup=1,
                                                       time_limit=args.cpu_seconds)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
               "ms_per_step": 1e3 * sps, "same_tree": not reduced}
    if rank == 0:
        keys = ("ms_per_step", "value", "vcycles_per_step", "vcycle_ms", "launches_per_step", "work_per_step",
                "photoi_step_ms", "plain_step_ms", "step_ms")
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic (seeded)", "config": config,
            "precision_split": {
                "mixed": {k: mixed[k] for k in keys},
                "fp64": {k: fp64[k] for k in keys},
                "speedup_mixed_vs_fp64": fp64["ms_per_step"] / mixed["ms_per_step"]},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                         "traffic_note": ("DRAM bytes are not measured inside the timed run (no profiler there); "
                                          "every kernel's DRAM bytes for the same workload under ncu are in "
                                          "profiles/dram_per_kernel_streamer_steps.md (2026-12-04)"),
                         "algorithmic_bytes_per_launch": ks["bytes"] / max(1, ks["launches"]),
                         "avg_launch_us": 1e3 * ks["ms"] / max(1, ks["launches"])},
            "kernel_classes": kstats, "tuning": tuning,
            **({"error_mixed_vs_fp64": accuracy} if accuracy else {}),
            **({"one_at_a_time": dict(one, speedup_batched=value / one["value"])} if one else {}),
            **({"amr": amr} if amr else {}),
            "cpu_baseline": cpu, "e2e": e2e, "clocks": mixed["clocks"],
            "gpu_launches": int(mixed["launches"]),
        }))


if __name__ == "__main__":
    main()
