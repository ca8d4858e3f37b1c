"""Benchmark of the D2Q9 step: GLUPS and the fraction of the HBM roofline.

Workload (one GPU): the plain FP32 channel -- 4096 x 4096 cells, Zou-He parabolic inlet
(peak u = 0.05), zero-gradient outflow, bounce-back walls top and bottom, seeded
non-overlapping disks (radius U[8, 32], 5 % solid), tau = 0.56, equilibrium start.  A
bench step is one LBM time step over the whole lattice.  The working set (2 x 604 MB of
populations) is larger than L2, so no flush is needed between steps.

Output: one JSON line.  value = cell updates / s / 1e9 of K steps (device time, CUDA events
on the library's stream), the median over `repeats` back-to-back intervals of exactly K
steps (repeated until about --min-seconds of device time, so that the clock samples see the
load; `spread` gives the slowest and fastest interval); e2e = the same metric for the whole
job through the public API (create from host parameters, scene mask built on the device
from the uploaded disk list, K steps, macro field read back to page-locked host memory);
roofline = 72 algorithmic bytes per cell update over the measured HBM copy bandwidth;
cpu_baseline = the oracle (the CPU restatement of the reference path) on the host cores,
full workload, about 15 s of steps.  `reference_mode_glups` / `reference_mode_exact_glups`:
the reference's own rules (its Poiseuille scene) at the same size, in the fast and the exact
arithmetic.  `extras`: the precision form's 8192^2 lattice in FP32, the reference's rules,
FP16 / BF16 storage, and the batched form (256 seeded domains), each with its roofline
fraction.

--impl reference times that CPU restatement alone (all host threads) on the full workload,
the reference having no CPU implementation of its own (its path is WGSL run by wgpu, which
needs a graphics API these machines do not have).

Multi-GPU: replicas only -- each rank advances its own copy of the workload; no
collectives touch the data path.
"""
import argparse
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_VALUE = {"f32": 4, "f16": 2, "bf16": 2, "f64": 8}  # 9 loads + 9 stores per cell update
METRIC = "D2Q9 GLUPS (FP32 channel 4096^2), % HBM roofline"
UNIT = "GLUPS"
E2E_REPEATS = 5  # end-to-end runs (create + K steps + read-back); the median is reported


def workload_params(args):
    return dict(nx=args.nx, ny=args.ny, mode="physics", dtype=args.dtype, scene="channel", tau=0.56,
                inlet_speed=0.05, solid_fraction=0.05, disk_radius=(8.0, 32.0), seed=1234, kernel=args.kernel,
                rounding=args.rounding)


def config_dict(args):
    return {"workload": "channel %dx%d %s, Zou-He inlet u=0.05 parabolic, outflow, walls, disks r 8-32 5%% solid, "
                        "tau 0.56, equilibrium start" % (args.nx, args.ny, args.dtype),
            "cells": args.nx * args.ny, "steps_per_bench_step": 1, "l2_flush": "none: working set 1.2 GB > L2",
            "parallelism": "replicas" if args.gpus > 1 else "single GPU", "kernel": args.kernel,
            "rounding": args.rounding}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(pg, x: float, device) -> float:
    """The largest x over the ranks of pg (x itself without a process group)."""
    if pg is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def replica_glups(world: int, cells: int, steps: int, seconds_max: float) -> float:
    """Whole-job GLUPS of `world` independent replicas of `cells` cells, each stepped
    `steps` times, timed by the slowest replica (weak scaling: no data is exchanged)."""
    return world * cells * steps / seconds_max / 1e9


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.3)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def effective_kernel(args):
    """The step kernel LBM_KERNEL_AUTO runs for this configuration."""
    if args.kernel != "auto":
        return args.kernel
    if args.dtype in ("f32", "f64"):
        return "cell"
    return "tiled" if args.nx % 64 == 0 else "vec2"


def committed_traffic(args):
    """DRAM bytes per launch of the step kernel from a committed ncu summary of this exact
    configuration (dtype, size, kernel, rounding), or None."""
    path = os.path.join(ROOT, "profiles", "channel_step_traffic.json")
    try:
        with open(path) as f:
            entries = json.load(f)["entries"]
    except (OSError, ValueError, KeyError):
        return None
    key = (args.dtype, args.nx, args.ny, effective_kernel(args), args.rounding)
    for e in entries:
        if (e["dtype"], e["nx"], e["ny"], e["kernel"], e["rounding"]) == key:
            return e
    return None


def cpu_baseline_sample(args, seconds_cap=15.0):
    """The oracle's FP32 physics step on the full channel workload (all host threads), as
    many steps as fit in seconds_cap after two warm-up steps."""
    import numpy as np

    import oracle

    info, _ = oracle.mask_physics_channel(args.nx, args.ny, 0.05, 1234, 0.05, 8.0, 32.0)
    sim = oracle.PhysOracle(info, 0.56, np.float32)
    sim.step(2)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while True:
        sim.step(1)
        steps += 1
        el = time.perf_counter() - t0
        if el > seconds_cap or steps >= 5000:
            break
    glups = args.nx * args.ny * steps / el / 1e9
    return {"value": glups, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
            "sample": "oracle FP32 physics step on the full %dx%d channel workload, %d steps after 2 warm-up "
                      "steps, %.1f s" % (args.nx, args.ny, steps, el)}


def run_reference(args):
    """CPU restatement of the reference path (the oracle) on the full workload, all host
    threads: W warm-up steps, then K timed steps."""
    import numpy as np

    import oracle

    world, rank, _ = dist_env()
    if rank != 0:
        return
    info, _ = oracle.mask_physics_channel(args.nx, args.ny, 0.05, 1234, 0.05, 8.0, 32.0)
    sim = oracle.PhysOracle(info, 0.56, np.float32)
    sim.step(args.warmup)
    t0 = time.perf_counter()
    sim.step(args.steps)
    el = time.perf_counter() - t0
    glups = args.nx * args.ny * args.steps / el / 1e9
    cores = oracle.num_threads()
    line = {"impl": "reference", "metric": METRIC, "value": glups, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded channel mask)", "config": config_dict(args),
            "cpu_baseline": {"value": glups, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "oracle FP32 physics step on the full %dx%d channel workload, %d steps"
                                       % (args.nx, args.ny, args.steps)},
            "e2e": {"value": glups, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def timed_intervals(step_k, stream, steps, min_seconds, min_repeats=10, max_repeats=20000):
    """Device milliseconds of R back-to-back intervals of `steps` steps (step_k(steps) queues
    one interval), each bracketed by CUDA events on `stream`.  R >= min_repeats and large
    enough that the intervals together last about min_seconds, estimated from a first
    interval; one host synchronisation at the end."""
    import torch

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    step_k(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    est = max(e0.elapsed_time(e1), 1e-3)
    reps = int(min(max_repeats, max(min_repeats, round(min_seconds * 1e3 / est))))
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for a, b in evs:
        a.record(stream)
        step_k(steps)
        b.record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in evs]


def median(xs):
    ys = sorted(xs)
    n = len(ys)
    return ys[n // 2] if n % 2 else 0.5 * (ys[n // 2 - 1] + ys[n // 2])


def glups_of(cells, steps, ms):
    return cells * steps / (ms * 1e-3) / 1e9


def measure_sim(sim, stream, cells, bytes_per_cell, peak, steps=100, warmup=5, min_seconds=0.5):
    """GLUPS (median over repeated intervals) and roofline fraction of one simulator."""
    import torch

    sim.set_stream(stream.cuda_stream)
    sim.step(warmup)
    torch.cuda.synchronize()
    ms = timed_intervals(sim.step, stream, steps, min_seconds, min_repeats=3)
    g = glups_of(cells, steps, median(ms))
    return {"glups": g, "gb_per_s": g * bytes_per_cell, "roofline_frac": g * bytes_per_cell / peak,
            "bytes_per_cell": bytes_per_cell, "steps_per_interval": steps, "intervals": len(ms),
            "spread_glups": [glups_of(cells, steps, max(ms)), glups_of(cells, steps, min(ms))]}


def run_extras(args, stream, peak):
    """The other forms of the step at the precision form's size (8192^2), each timed on its own
    lattice: the FP32 channel (the size the 80 % target is stated for), the reference's own
    rules (its Poiseuille scene) in the fast and the exact arithmetic, 16-bit storage of the
    channel (FP16 and BF16, round-to-nearest and stochastic rounding), and the batched form
    (256 seeded domains, autotuned persistent launch against the per-domain loop)."""
    import torch

    from simuverse_gb300 import BatchSimulator, FluidSimulator, generate_domains

    n = args.extras_size
    cells = n * n
    chan = dict(mode="physics", scene="channel", inlet_speed=0.05, solid_fraction=0.05, disk_radius=(8.0, 32.0),
                seed=1234)
    out = {"size": [n, n]}
    forms = [("fp32", dict(chan, tau=0.56), 72),
             ("reference_rules_fast", dict(mode="reference", scene="poiseuille", tau=0.56, arith="fast"), 72),
             ("reference_rules_exact", dict(mode="reference", scene="poiseuille", tau=0.56, arith="exact"), 72),
             ("f16", dict(chan, tau=0.6, dtype="f16"), 36),
             ("f16_stochastic", dict(chan, tau=0.6, dtype="f16", rounding="stochastic"), 36),
             ("bf16_stochastic", dict(chan, tau=0.6, dtype="bf16", rounding="stochastic"), 36)]
    for name, kw, bpc in forms:
        sim = FluidSimulator(n, n, **kw)
        out[name] = measure_sim(sim, stream, cells, bpc, peak)
        sim.close()
        torch.cuda.synchronize()
    for name in ("f16", "f16_stochastic", "bf16_stochastic"):
        out[name]["over_fp32"] = out[name]["glups"] / out["fp32"]["glups"]

    doms = generate_domains(256, 1234)
    b = BatchSimulator(doms)
    b.set_stream(stream.cuda_stream)
    t0 = time.perf_counter()
    tuned = b.tune(trial_steps=10)
    res = {"domains": len(doms), "cells": b.cells, "tune_seconds": time.perf_counter() - t0, "tuned": tuned}
    for method, steps in (("persistent", 200), ("domain_loop", 50)):
        b.configure(method=method)
        b.step(3)
        b.status()
        ms = timed_intervals(b.step, stream, steps, 0.3, min_repeats=3)
        b.status()
        g = glups_of(b.cells, steps, median(ms))
        res[method] = {"glups": g, "gb_per_s": 72 * g, "roofline_frac": 72 * g / peak, "steps_per_interval": steps,
                       "intervals": len(ms)}
    res["persistent_over_loop"] = res["persistent"]["glups"] / res["domain_loop"]["glups"]
    b.close()
    out["batch"] = res
    out["closure"] = closure_speed(stream)
    return out


def closure_speed(stream, nf=4096, factor=4, k_coarse=4):
    """Speed of the learned-closure form: periodic decaying turbulence, fine lattice nf^2 at tau
    0.5005 against the coarse lattice (nf / factor)^2 at the acoustically scaled tau with the
    closure (fused tcgen05 kernel, stress form) applied every k_coarse coarse steps, KBC
    on both.  Device time per fine step, per coarse step and per closure application (median of
    repeated intervals); the coarse run covers factor fine steps per coarse step, so its speed-up
    for the same span is factor * t_fine / (t_coarse + t_closure / k_coarse).  The speed does not
    depend on the network's weights (seeded initial weights here)."""
    import numpy as np

    from simuverse_gb300 import FluidSimulator
    from simuverse_gb300.closure import Closure
    from simuverse_gb300.turbulence import random_velocity

    nc = nf // factor
    tau_f = 0.5005
    tau_c = 0.5 + (tau_f - 0.5) / factor
    out = {"fine": nf, "coarse": nc, "k_coarse": k_coarse, "collision": "kbc"}
    sims = {}
    for name, n, tau in (("fine", nf, tau_f), ("coarse", nc, tau_c)):
        s = FluidSimulator(n, n, mode="physics", scene="periodic", tau=tau, collision="kbc")
        ux, uy = random_velocity(n, 9001, 8.0, 0.04)
        s.init_equilibrium(None, ux.astype(np.float32), uy.astype(np.float32))
        s.set_stream(stream.cuda_stream)
        s.step(3)
        sims[name] = s
    t_fine = median(timed_intervals(sims["fine"].step, stream, 20, 0.3, min_repeats=3)) / 20
    t_coarse = median(timed_intervals(sims["coarse"].step, stream, 80, 0.3, min_repeats=3)) / 80
    c = Closure(nc, nc, seed=1, s_in=20.0, s_out=1e6, inputs="eq", target="stress", projection="cell")
    c.set_kernel("fused")

    def apply_k(k):
        for _ in range(k):
            c.apply(sims["coarse"])

    apply_k(3)
    t_closure = median(timed_intervals(apply_k, stream, 20, 0.3, min_repeats=3)) / 20
    c.status()
    c.close()
    for s in sims.values():
        s.close()
    out.update({"fine_step_ms": t_fine, "coarse_step_ms": t_coarse, "closure_apply_ms": t_closure,
                "speedup_plain_coarse": factor * t_fine / t_coarse,
                "speedup_with_closure": factor * t_fine / (t_coarse + t_closure / k_coarse)})
    return out


def run_gpu(args):
    import numpy as np
    import torch

    from simuverse_gb300 import FluidSimulator

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist

    params = workload_params(args)
    cells = args.nx * args.ny
    sim = FluidSimulator(**params)
    # a real stream (not the legacy default, whose handle is 0): the library launches on
    # it and the CUDA events below are recorded on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sim.set_stream(stream.cuda_stream)
    sim.step(args.warmup)
    torch.cuda.synchronize()

    # ---- timed region: R intervals of exactly K steps each, device time on the launching
    # stream; R repeats the interval until about --min-seconds of load, so the clock samples
    # see the kernel running
    clocks = ClockSampler(local)
    clocks.start()
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    launches0 = sim.kernel_launches
    ms_list = timed_intervals(sim.step, stream, args.steps, args.min_seconds)
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    gpu_launches = sim.kernel_launches - launches0
    clk = clocks.stop()
    ms = median(ms_list)
    ms_max = max_over_ranks(pg, ms, "cuda")
    value = replica_glups(world, cells, args.steps, ms_max * 1e-3)
    per_launch_s = ms * 1e-3 / args.steps
    bytes_per_cell = 18 * BYTES_PER_VALUE[args.dtype]
    achieved = bytes_per_cell * cells / per_launch_s / 1e9
    peak, peak_kind = measured_peak()
    tr = committed_traffic(args)

    # ---- macro every step (the reference's behaviour), reported separately
    sim_m = FluidSimulator(macro_every_step=True, **params)
    sim_m.set_stream(stream.cuda_stream)
    sim_m.step(args.warmup)
    torch.cuda.synchronize()
    glups_macro = glups_of(cells, args.steps, median(timed_intervals(sim_m.step, stream, args.steps, 0.3,
                                                                        min_repeats=3)))
    sim_m.close()
    sim.close()
    torch.cuda.synchronize()

    # ---- the reference's own rules (reference mode, its Poiseuille scene) at the same size
    glups_ref_mode = {}
    if args.dtype == "f32":
        for arith in ("fast", "exact"):
            sim_r = FluidSimulator(args.nx, args.ny, mode="reference", scene="poiseuille", tau=0.56, arith=arith)
            glups_ref_mode[arith] = measure_sim(sim_r, stream, cells, 72, peak, steps=args.steps, warmup=args.warmup,
                                                min_seconds=0.3)["glups"]
            sim_r.close()

    # ---- end to end through the public API, host buffers
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    # the result lands in page-locked host buffers allocated before the timed region
    pinned = torch.empty((3, args.ny, args.nx), dtype=torch.float32, pin_memory=True).numpy()
    e2e_runs = []
    for _ in range(E2E_REPEATS):
        t0 = time.perf_counter()
        s2 = FluidSimulator(**params)
        t1 = time.perf_counter()
        s2.step(args.steps)
        rho, ux, uy = s2.read_macro(out=(pinned[0], pinned[1], pinned[2]))
        t2 = time.perf_counter()
        s2.close()
        assert np.isfinite(rho).all()
        e2e_runs.append((t2 - t0, t1 - t0))
    t_e2e, t_create = sorted(e2e_runs)[len(e2e_runs) // 2]
    e2e_glups = replica_glups(world, cells, args.steps, max_over_ranks(pg, t_e2e, "cuda"))
    from simuverse_gb300.fluid import scene_disks

    h2d = 24 * len(scene_disks(**params))  # the channel's disk list; the mask is built on the device
    d2h = cells * 12  # rho, ux, uy read back

    extras = None
    if world == 1 and not args.no_extras:
        extras = run_extras(args, stream, peak)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": args.dtype,
            "data": "synthetic (seeded channel mask, equilibrium start)", "config": config_dict(args),
            "repeats": len(ms_list),
            "spread": {"glups_min": glups_of(cells, args.steps, max(ms_list)),
                       "glups_max": glups_of(cells, args.steps, min(ms_list)),
                       "what": "value is the median over `repeats` back-to-back intervals of `steps` steps"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": (tr or {}).get("bytes_per_launch_scaled"),
                         "traffic_source": (tr or {}).get("source"),
                         "algorithmic_bytes_per_launch": bytes_per_cell * cells},
            "macro_every_step_glups": glups_macro,
            "reference_mode_glups": glups_ref_mode.get("fast"),
            "reference_mode_exact_glups": glups_ref_mode.get("exact"),
            "e2e": {"value": e2e_glups, "unit": UNIT, "h2d_bytes_per_step": h2d / args.steps,
                    "d2h_bytes_per_step": d2h / args.steps, "create_ms": t_create * 1e3,
                    "repeats": E2E_REPEATS,
                    "glups_min": glups_of(cells, args.steps, 1e3 * max(r[0] for r in e2e_runs)),
                    "glups_max": glups_of(cells, args.steps, 1e3 * min(r[0] for r in e2e_runs)),
                    "what": "create (disk list upload, scene mask built on the device; buffers from the "
                            "library's memory pool, which the lattices closed before left reserved) + K steps "
                            "+ macro read-back into page-locked host buffers, wall clock; median of the repeats"},
            "gpu_launches": gpu_launches,
            "gpu_launches_per_interval": gpu_launches // max(1, len(ms_list) + 1),
            "clocks": clk,
        }
        if extras is not None:
            line["extras"] = extras
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline_sample(args)
        print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()


def run_reference_rules(args):
    """The reference's own rules (reference mode, its Poiseuille scene at args.nx x args.ny,
    tau 0.56) in one arithmetic (--arith): GLUPS over K steps, median of repeated intervals,
    and the fraction of the HBM roofline at 72 B per cell update."""
    import torch

    from simuverse_gb300 import FluidSimulator

    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    peak, peak_kind = measured_peak()
    sim = FluidSimulator(args.nx, args.ny, mode="reference", scene="poiseuille", tau=0.56, arith=args.arith)
    r = measure_sim(sim, stream, args.nx * args.ny, 72, peak, steps=args.steps, warmup=args.warmup,
                    min_seconds=args.min_seconds)
    sim.close()
    r.update({"workload": "reference rules, Poiseuille %dx%d, tau 0.56, arith %s" % (args.nx, args.ny, args.arith),
              "peak_gbs": peak, "peak_source": peak_kind})
    print(json.dumps(r), flush=True)


def run_precision(args):
    """Precision form at 8192^2: GLUPS of FP32 / FP16 / BF16 storage with each kernel
    variant, and the error of each against an FP64 run of the same channel at checkpoints up
    to args.steps steps (rel L2 of rho and u; the open channel's mass change, for
    comparison with FP64's)."""
    import torch

    from simuverse_gb300 import FluidSimulator

    nx = ny = args.nx
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    out = {"workload": "precision", "nx": nx, "ny": ny, "glups": {}, "errors": {}}
    base = dict(mode="physics", scene="channel", inlet_speed=0.05, solid_fraction=0.05, disk_radius=(8.0, 32.0),
                seed=1234)
    for dtype in () if args.skip_glups else ("f32", "f16", "bf16"):
        for kernel in ("cell", "vec2", "vec4", "bulk") + (("tiled", "tiled+sr", "vec2+sr") if dtype != "f32" else ()):
            rounding = "stochastic" if kernel.endswith("+sr") else "nearest"
            sim = FluidSimulator(nx, ny, dtype=dtype, tau=0.6, kernel=kernel.split("+")[0], rounding=rounding, **base)
            sim.set_stream(stream.cuda_stream)
            sim.step(args.warmup)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            sim.step(args.timing_steps)
            e1.record(stream)
            torch.cuda.synchronize()
            g = nx * ny * args.timing_steps / (e0.elapsed_time(e1) * 1e-3) / 1e9
            out["glups"]["%s/%s" % (dtype, kernel)] = g
            sim.close()
    # error study: all four storage forms step in lockstep; errors against FP64 at every
    # checkpoint.  BGK is unstable for this channel at tau 0.51 (FP64 included), so taus
    # below 0.55 use the KBC collision for every form.
    checkpoints = sorted(set([c for c in args.checkpoints if c < args.steps] + [args.steps]))
    for tau in args.taus:
        coll = args.error_collision if args.error_collision != "auto" else ("kbc" if tau < 0.55 else "bgk")
        # f16sr / bf16sr: the same storage with stochastic rounding
        forms = ("f64", "f32", "f16", "bf16", "f16sr", "bf16sr")
        sims = {d: FluidSimulator(nx, ny, dtype=d[:-2] if d.endswith("sr") else d, tau=tau, collision=coll,
                                  rounding="stochastic" if d.endswith("sr") else "nearest", **base) for d in forms}
        m0 = {d: s.conservation()[0] for d, s in sims.items()}
        rows, done = [], 0
        for cp in checkpoints:
            for s in sims.values():
                s.step(cp - done)
            done = cp
            ref = sims["f64"]
            row = {"step": cp, "fp64_mass_change": (ref.conservation()[0] - m0["f64"]) / m0["f64"],
                   "fp64_nonfinite": ref.nonfinite_count()}
            for d in forms[1:]:
                err = sims[d].macro_error(ref)
                row[d] = {"rel_l2_rho": err[0], "rel_l2_u": err[1], "max_du": err[2],
                          "mass_change": (sims[d].conservation()[0] - m0[d]) / m0[d],
                          "nonfinite": sims[d].nonfinite_count()}
            rows.append(row)
        for s in sims.values():
            s.close()
        out["errors"]["tau=%g" % tau] = {"collision": coll, "checkpoints": rows}
    out["steps"] = args.steps
    print(json.dumps(out), flush=True)


def run_batch(args):
    """Batched form: seeded list of 256 cavities and channels; aggregate GLUPS of the
    persistent CUDA-graph launch (autotuned) against a per-domain launch loop."""
    import torch

    from simuverse_gb300 import BatchSimulator, generate_domains

    doms = generate_domains(args.domains, args.seed)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    out = {"workload": "batch", "domains": len(doms)}
    b = BatchSimulator(doms)
    b.set_stream(stream.cuda_stream)
    out["cells"] = b.cells
    t0 = time.perf_counter()
    out["tuned"] = b.tune(trial_steps=10)
    out["tune_seconds"] = time.perf_counter() - t0
    res = {}
    for method, steps in (("persistent", args.steps), ("tile_launches", args.steps), ("domain_loop", args.loop_steps)):
        b.configure(method=method)
        b.step(3)
        b.status()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        b.step(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        b.status()
        ms = e0.elapsed_time(e1)
        res[method] = {"steps": steps, "ms_per_step": ms / steps, "glups": b.cells * steps / (ms * 1e-3) / 1e9,
                       "gb_per_s": 72 * b.cells * steps / (ms * 1e-3) / 1e9}
    out["methods"] = res
    out["persistent_over_loop"] = res["persistent"]["glups"] / res["domain_loop"]["glups"]
    print(json.dumps(out), flush=True)


def run_closure(args):
    """Learned closure on periodic decaying turbulence: fine 4096^2 (tau 0.5005) against a
    4x-coarsened 1024^2 lattice corrected by the trained BF16 network every k coarse steps.
    Pairs from args.train_seeds seeds x args.snapshots snapshots x (fresh, rollout); with
    --dagger N, N more rounds regenerate the pairs from closure-corrected rollouts and
    continue training.  Evaluation on unseen seeds."""
    import torch

    import numpy as np

    from simuverse_gb300.closure import Closure, TurbulenceSetup, evaluate, generate_pairs, time_runs

    setup = TurbulenceSetup(nf=args.nx, factor=4, tau_f=0.5005, k_coarse=args.k_coarse, collision=args.collision)
    out = {"workload": "closure", "fine": args.nx, "coarse": setup.nc, "tau_f": setup.tau_f, "tau_c": setup.tau_c,
           "k_coarse": setup.k_coarse, "collision": args.collision}
    c = Closure(setup.nc, setup.nc, seed=args.seed, inputs=args.inputs, target=args.target, projection=args.projection)
    window = args.window or args.k_coarse
    if args.target == "stress":
        c.set_stress_factor(window / (2.0 * args.k_coarse))
    out["form"] = {"inputs": args.inputs, "target": args.target, "projection": args.projection, "window": window}
    out["sources"] = list(args.sources)
    seeds = list(range(1000, 1000 + args.train_seeds))
    npairs = args.train_seeds * args.snapshots * len(args.sources)
    curve = []
    out["datagen_s"] = 0.0
    out["train_s"] = 0.0
    for rnd in range(1 + args.dagger):
        c.reserve(npairs + 64, args.crop, 8)
        t0 = time.perf_counter()
        generate_pairs(c, setup, seeds, snapshots=args.snapshots, interval=args.interval, crop=args.crop,
                       rng_seed=args.seed + rnd, sources=tuple(args.sources), corrected=c if rnd > 0 else None,
                       calibrate=rnd == 0, window=window)
        out["datagen_s"] += time.perf_counter() - t0
        hold = max(1, c.npairs // 20)
        if rnd == 0:
            out["pairs"] = c.npairs
            out["scales"] = [c.s_in, c.s_out]
            p0 = c.params
            c.params = np.zeros_like(p0)
            out["loss_zero_output"] = c.eval(c.npairs - hold, c.npairs)
            c.params = p0
            out["loss_initial"] = c.eval(c.npairs - hold, c.npairs)
        t0 = time.perf_counter()
        iters = args.train_iters if rnd == 0 else args.train_iters // 2
        for block in range(args.train_blocks):
            last = block >= args.train_blocks - 2
            lt = c.train(iters // args.train_blocks, lr=args.lr / 4 if last else args.lr, seed=args.seed + 97 * rnd + block)
            curve.append({"round": rnd, "iter": (block + 1) * (iters // args.train_blocks), "train_loss": lt,
                          "heldout_loss": c.eval(c.npairs - hold, c.npairs)})
        torch.cuda.synchronize()
        out["train_s"] += time.perf_counter() - t0
    out["training_curve"] = curve
    # correction strength: chosen on a validation seed (neither a training nor an evaluation
    # seed) by the final velocity error, then used on the evaluation seeds next to strength 1
    best = 1.0
    if len(args.strengths) > 1:
        rows = evaluate(c, setup, args.val_seed, fine_steps=args.fine_steps, check_every=args.fine_steps,
                        strengths=tuple(args.strengths))
        last = rows[-1]
        best = min(args.strengths, key=lambda a: last["err_closure" if a == 1.0 else "err_closure@%g" % a])
        out["validation"] = {"seed": args.val_seed, "rows": rows, "strength": best}
    out["strength"] = best
    out["eval"] = {}
    for seed in args.eval_seeds:
        rows = evaluate(c, setup, seed, fine_steps=args.fine_steps, check_every=args.check_every,
                        strengths=tuple(sorted({1.0, best})))
        out["eval"][str(seed)] = rows
    out["timing"] = time_runs(c, setup, args.eval_seeds[0], fine_steps=args.fine_steps, strength=best)
    print(json.dumps(out), flush=True)


def run_view(args):
    """Consumers of the macro field on a physics channel of args.nx x args.ny cells drawn on
    a canvas of 2 pixels per cell: the reference frame (two steps, each followed by a
    particle update; then the canvas present), the curl field and the curl colour map.
    Device time per operation (CUDA events on the lattice's stream), and the bandwidth of the
    canvas-sized kernels against the HBM roofline (algorithmic bytes: present 12 B read +
    16 B RGBA write + 4 B alpha write per lit pixel; curl 8 B read + 4 B write per cell;
    colour map 16 B write per pixel + the field and curl planes once)."""
    import numpy as np
    import torch

    from simuverse_gb300 import FluidSimulator
    from simuverse_gb300 import _native as nat
    from simuverse_gb300.view import Particles

    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    nx, ny = args.nx, args.ny
    sim = FluidSimulator(nx, ny, mode="physics", scene="channel", tau=0.56, inlet_speed=0.05, solid_fraction=0.05,
                         seed=args.seed, pixel_size=2)
    sim.set_stream(stream.cuda_stream)
    ps = Particles(sim, count=args.particles, life_time=60.0, point_size=2, seed=1, color_ty=1)
    cw, ch = ps.canvas_w, ps.canvas_h
    out = {"workload": "view", "nx": nx, "ny": ny, "canvas": [cw, ch], "particles": ps.count}
    lib = nat.load()
    curl_buf = torch.empty(nx * ny, dtype=torch.float32, device="cuda")
    rgba = torch.empty(cw * ch * 4, dtype=torch.float32, device="cuda")
    import ctypes

    def op_curl():
        nat.check(lib.lbm_curl(sim.handle, ctypes.c_void_p(curl_buf.data_ptr())))

    def op_colorize():
        nat.check(lib.lbm_colorize(sim.handle, 0, ctypes.c_void_p(curl_buf.data_ptr()), cw, ch,
                                   ctypes.c_void_p(rgba.data_ptr())))

    def timed(fn, reps):
        for _ in range(3):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    # warm the field and the canvas with a few frames
    for _ in range(50):
        ps.compute()
        ps.present()
    peak = measured_peak()[0]
    ms = {}
    ms["step"] = timed(lambda: sim.step(1), args.timing_steps // 10)
    ms["particles_update"] = timed(ps.update, 200)
    lit = float(np.mean(ps.canvas()[..., 0] > 0.001))
    ms["present"] = timed(ps.present, 50)
    ms["curl"] = timed(op_curl, 50)
    ms["colorize"] = timed(op_colorize, 50)

    def frame():
        ps.compute()
        ps.present()

    ms["frame"] = timed(frame, 50)
    out["ms"] = ms
    out["lit_fraction"] = lit
    npix = cw * ch
    bytes_present = npix * (12 + 16) + lit * npix * 4
    bytes_curl = nx * ny * 12
    bytes_color = npix * 16 + nx * ny * 16
    out["gb_per_s"] = {"present": bytes_present / (ms["present"] * 1e-3) / 1e9,
                       "curl": bytes_curl / (ms["curl"] * 1e-3) / 1e9,
                       "colorize": bytes_color / (ms["colorize"] * 1e-3) / 1e9}
    out["roofline_frac"] = {k: v / peak for k, v in out["gb_per_s"].items()}
    out["particles_per_s"] = ps.count / (ms["particles_update"] * 1e-3)
    out["peak_gbs"] = peak
    print(json.dumps(out), flush=True)
    ps.close()
    sim.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nx", type=int, default=4096)
    ap.add_argument("--ny", type=int, default=4096)
    ap.add_argument("--dtype", default="f32", choices=["f32", "f16", "bf16", "f64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the 8192^2 forms and the batched form")
    ap.add_argument("--extras-size", type=int, default=8192)
    ap.add_argument("--min-seconds", type=float, default=2.0,
                    help="repeat the K-step interval until about this much device time is timed")
    ap.add_argument("--kernel", default="auto", choices=["auto", "cell", "vec4", "bulk", "vec2", "tiled", "ring"])
    ap.add_argument("--rounding", default="nearest", choices=["nearest", "stochastic"],
                    help="rounding of 16-bit population stores")
    ap.add_argument("--workload", default="channel",
                    choices=["channel", "reference", "precision", "batch", "closure", "closure_speed", "view"])
    ap.add_argument("--arith", default="fast", choices=["fast", "exact"],
                    help="--workload reference: arithmetic of the reference-rule step")
    ap.add_argument("--train-seeds", type=int, default=8)
    ap.add_argument("--snapshots", type=int, default=125)
    ap.add_argument("--interval", type=int, default=512)
    ap.add_argument("--dagger", type=int, default=0)
    ap.add_argument("--inputs", default="eq", choices=["eq", "neq"])
    ap.add_argument("--target", default="stress", choices=["momentum", "equilibrium", "populations", "stress"])
    ap.add_argument("--window", type=int, default=128, help="coarse steps per training pair (0: --k-coarse)")
    ap.add_argument("--crop", type=int, default=256, help="training crop side (coarse cells)")
    ap.add_argument("--projection", default="cell", choices=["domain", "cell"])
    ap.add_argument("--sources", nargs="+", default=["fresh"], choices=["fresh", "rollout"])
    ap.add_argument("--k-coarse", type=int, default=4)
    ap.add_argument("--train-iters", type=int, default=8000)
    ap.add_argument("--train-blocks", type=int, default=10)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--eval-seeds", type=int, nargs="*", default=[9001, 9002])
    ap.add_argument("--strengths", type=float, nargs="*", default=[1.0, 0.5, 0.35, 0.25],
                    help="closure correction strengths tried on the validation seed")
    ap.add_argument("--val-seed", type=int, default=7001)
    ap.add_argument("--check-every", type=int, default=2000)
    ap.add_argument("--fine-steps", type=int, default=20000, help="--workload closure: fine-equivalent steps evaluated")
    ap.add_argument("--collision", default="kbc", choices=["bgk", "kbc", "mrt", "regularized"])
    ap.add_argument("--taus", type=float, nargs="*", default=[0.51, 0.6, 0.9])
    ap.add_argument("--checkpoints", type=int, nargs="*", default=[1000, 5000])
    ap.add_argument("--error-collision", default="auto", choices=["auto", "bgk", "kbc"])
    ap.add_argument("--skip-glups", action="store_true")
    ap.add_argument("--timing-steps", type=int, default=500)
    ap.add_argument("--domains", type=int, default=256)
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--loop-steps", type=int, default=200)
    ap.add_argument("--particles", type=int, default=205000)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "reference":
        run_reference_rules(args)
    elif args.workload == "closure_speed":
        import torch

        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        print(json.dumps(closure_speed(stream, nf=args.nx)), flush=True)
    elif args.workload == "precision":
        run_precision(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "closure":
        run_closure(args)
    elif args.workload == "view":
        run_view(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
