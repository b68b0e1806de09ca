"""Benchmark: cell-updates/s of the force-free SSP-RK3 step on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--size S] [--precision fp32c|fp32|fp32cd|fp64] [--no-cpu-baseline]

Workload (the single-grid benchmark configuration): a periodic S^3 grid
(S = 512), Bz = 1 plus 32 seeded Alfven and fast modes with integer
wavevectors |k| <= 8 and amplitudes U[0, 0.02], c = 0.45, FP32 fields.
The timed mode is FP32C (float storage, the increment form of the RK
combination), the one that stays within 1e-5 of FP64; plain FP32 (the
reference's arithmetic in float), FP32CD and FP64 are timed beside it.
A step is one full main-loop body: three SSP-RK3 stages, each with its E
cleaning and ghost fills.  One cell-update = one interior cell advanced one
step.  Inputs are 3.3 GB per field set, far larger than the 129 MB L2, so no
flush is needed between steps.

Reported numbers:
  value   : cell-updates/s with the fields resident in HBM (CUDA events on the
            library's stream around K steps; max over ranks).
  e2e     : the same metric through the C ABI from pinned host buffers:
            upload of E,B, K steps, download of E,B, all inside the timed region
            (median of three runs).
  roofline: the fused stage kernel (3 launches per step, the whole step):
            algorithmic bytes = 54 words per cell-update (18 per stage launch:
            E,B in and out plus the step-start E,B) / step time, against the
            measured HBM copy bandwidth; `frac_fused_words` restates it with
            the 48 words the fused path must move (no step-start copy).
  accuracy: relative L2 and L-infinity error of E and B of the timed mode
            against the FP64 path after --accuracy-line-steps steps of the
            same workload, and of the FP64 GPU path against the CPU oracle
            (FP64) after --oracle-check-steps steps.
  cpu_baseline: the CPU restatement (oracle/, OpenMP, all host cores) on a
            bounded sample of the same workload (the same grid, a few steps),
            in the timed mode and in FP64, with the host's CPU model.
Multi-GPU: replicas only (one independent grid per rank, no collective in the
data path); value sums all ranks' cell-updates over the slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "tristan-ff_gb300"))

# Algorithmic words per cell-update: 3 stages x 18 (stage 1 reads E,B and
# writes E,B and the step-start copy En,Bn; stages 2-3 read E,B,En,Bn and
# write E,B), the compulsory traffic of a fully fused stage.  The fused path
# keeps the step-start set in place (a set rotation) and so moves 48.
WORDS_PER_CELL_STEP = 54
WORDS_FUSED_PATH = 48
HBM_FALLBACK_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--precision", default="fp32c", choices=["fp32", "fp32c", "fp32cd", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-other-precisions", action="store_true",
                    help="skip the FP32C and FP64 timings added to the line (single GPU)")
    ap.add_argument("--cpu-sample", type=int, default=0, help="edge of the CPU sample grid (0 = auto)")
    ap.add_argument("--accuracy-steps", type=int, default=0,
                    help="instead of timing: run FP64, FP32 and FP32C for N steps and report their errors")
    ap.add_argument("--workload", default="grid", choices=["grid", "batch", "serve", "psr", "psr-accuracy"],
                    help="grid: the single 512^3 grid (default line); batch: 64 uneven boxes, batched vs "
                         "one grid at a time; serve: a Poisson stream of pulsar runs, continuous batching "
                         "vs one grid at a time; psr: the 512^3 pulsar magnetosphere (rate and error vs FP64)")
    ap.add_argument("--batch-steps", type=int, default=500, help="batch: steps of every box")
    ap.add_argument("--psr-marks", default="50,100,200,400",
                    help="psr: step counts at which the error against FP64 is stated")
    ap.add_argument("--batch-boxes", type=int, default=64)
    ap.add_argument("--batch-kind", default="mixed", choices=["mixed", "packet"],
                    help="batch: half packets and half flux tubes (which carry a B0 field), or packets only")
    ap.add_argument("--tile-y", type=int, default=0, choices=[0, 8, 16],
                    help="batch: fixed tile height instead of the autotuned tiling (0: autotune)")
    ap.add_argument("--requests", type=int, default=32, help="serve: number of requests")
    ap.add_argument("--budget-gb", type=float, default=180.0, help="serve: HBM admission budget")
    ap.add_argument("--epoch-steps", type=int, default=32, help="serve: steps per batched epoch at most")
    ap.add_argument("--max-active-cells", type=float, default=64 * 2 ** 20,
                    help="serve: cells of the admitted runs at most")
    ap.add_argument("--fp64-checks", type=int, default=2, help="serve: runs re-done in FP64 for the error")
    ap.add_argument("--oracle-steps", type=int, default=0,
                    help="with --accuracy-steps: also check the FP64 GPU path against the CPU oracle "
                         "after this many steps")
    ap.add_argument("--accuracy-line-steps", type=int, default=100,
                    help="steps of the accuracy check added to the line (timed mode vs FP64; 0: none)")
    ap.add_argument("--oracle-check-steps", type=int, default=10,
                    help="steps of the FP64 GPU path vs the CPU oracle check added to the line (0: none)")
    ap.add_argument("--cpu-steps", type=int, default=0,
                    help="steps of the CPU baseline sample (0: 3 at 512^3, more on smaller grids)")
    return ap.parse_args()


def accuracy(args):
    """Relative L2 and L-infinity error of E and B of the FP32 and FP32C fused
    paths against the FP64 fused path after N steps of the benchmark workload.
    The FP64 GPU path stands in for the CPU oracle at this size; it is first
    checked against the oracle (FP64, OpenMP) over `--oracle-steps` steps."""
    import numpy as np
    import torch
    import ffe
    import build as ffe_build
    torch.cuda.set_device(0)
    ffe_build.build()
    S = args.size
    size = (S, S, S)
    bg, modes = workload(S)
    names = ("ex", "ey", "ez", "bx", "by", "bz")

    def run(prec, steps):
        g = ffe.Solver(ffe.make_desc(size, precision=prec))
        g.init_waves(bg, modes)
        g.mainloop_prologue()
        init = None
        if prec == ffe.FP64 and args.oracle_steps:
            init = {n: g.download(n) for n in names}
        t0 = time.perf_counter()
        g.mainloop(steps, 0)
        g.synchronize()
        dt = time.perf_counter() - t0
        out = {n: ffe.interior(g.download(n)) for n in names}
        g.close()
        return out, dt, init

    def errors(a, b):
        res = {}
        for grp, comps in (("E", names[:3]), ("B", names[3:])):
            num2 = den2 = linf = dmax = 0.0
            for n in comps:
                x = a[n].astype(np.float64)
                y = b[n]
                d = x - y
                num2 += float(np.vdot(d, d).real)
                den2 += float(np.vdot(y, y).real)
                linf = max(linf, float(np.max(np.abs(d))))
                dmax = max(dmax, float(np.max(np.abs(y))))
            res[grp] = {"rel_l2": (num2 / den2) ** 0.5 if den2 else None, "rel_linf": linf / dmax if dmax else None}
        return res

    N = args.accuracy_steps
    ref, t64, init = run(ffe.FP64, N)
    line = {"metric": "relative error vs the FP64 path after %d steps" % N, "grid": [S] * 3,
            "workload": "random Alfven+fast modes, periodic", "fp64_seconds": t64}
    for name, prec in (("fp32", ffe.FP32), ("fp32c", ffe.FP32C), ("fp32cd", ffe.FP32CD)):
        out, dt, _ = run(prec, N)
        line[name] = errors(out, ref)
        line[name]["seconds"] = dt
        del out
    if args.oracle_steps:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build()
        k = args.oracle_steps
        g = ffe.Solver(ffe.make_desc(size, precision=ffe.FP64))
        g.set_fields(init)
        g.mainloop(k, 0)
        gpu = {n: ffe.interior(g.download(n)) for n in names}
        g.close()
        o = O.Oracle(ffe.make_desc(size, precision=ffe.FP64), threads=os.cpu_count() or 1, loop_order=1)
        o.set_fields(init)
        t0 = time.perf_counter()
        o.mainloop(k, 0)
        cpu = {n: ffe.interior(o.download(n)) for n in names}
        line["fp64_gpu_vs_cpu_oracle"] = errors(gpu, cpu)
        line["fp64_gpu_vs_cpu_oracle"]["steps"] = k
        line["fp64_gpu_vs_cpu_oracle"]["oracle_seconds"] = time.perf_counter() - t0
    print(json.dumps(line), flush=True)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, world):
    """The largest x over all ranks (the slowest rank's time); x itself on one rank."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(cells_per_rank, steps, world, seconds):
    """Whole-job cell-updates/s: every rank advances its own grid (replicas)."""
    return cells_per_rank * steps * world / seconds


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", HBM_FALLBACK_GBS)), "measured"
    return HBM_FALLBACK_GBS, "fallback"


def traffic_from_profile(precision, size):
    """DRAM bytes per fused-stage launch from the committed ncu summary, scaled to `size`."""
    p = os.path.join(ROOT, "profiles", "fused_stage_traffic.json")
    if not os.path.exists(p):
        return None
    try:
        with open(p) as f:
            d = json.load(f)
        e = d.get(precision)
        if not e:
            return None
        return e["bytes_per_cell_per_launch"] * size ** 3
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None
        self.path = os.environ.get("FFE_CLOCKS_LOG") or os.path.join(
            tempfile.gettempdir(), "ffe_clocks_rank%d_%d.csv" % (index, os.getpid()))

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines()]
            rows = [[c.strip() for c in r] for r in rows if len(r) >= 9]
            sm = [float(r[1]) for r in rows]
            mx = max(float(r[2]) for r in rows)
            reasons = set()
            names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
            for r in rows:
                for n, v in zip(names, r[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
            return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                    "samples": len(rows)}
        except Exception as e:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "error": str(e)[:80]}


def workload(size):
    from ffe.workloads import random_modes
    bg, modes, meta = random_modes((size, size, size), seed=1, n=32, kmax=8, amax=0.02)
    return bg, modes


def cpu_model():
    """The host CPU's model name (lscpu), or the platform string."""
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, timeout=10).stdout
        for line in out.decode(errors="replace").splitlines():
            if line.strip().startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


def time_oracle(size, prec, steps, threads, warm=1):
    """Seconds per step of the oracle (CPU restatement, OpenMP, x-innermost
    loops) on the random-mode workload of `size`, after `warm` untimed steps."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import ffe
    import oracle as O
    from ffe.workloads import random_modes
    O.build()
    bg, modes, _ = random_modes(size, seed=1, n=32, kmax=8, amax=0.02)
    o = O.Oracle(ffe.make_desc(size, precision=prec), threads=threads, loop_order=1)
    o.init_waves(bg, modes)
    o.mainloop_prologue()
    if warm:
        o.mainloop(warm, 0)  # warm caches and pages
    t0 = time.perf_counter()
    o.mainloop(steps, warm)
    dt = time.perf_counter() - t0
    o.close()
    return dt / steps


def cpu_baseline(args, edge=None, steps=None, threads=None):
    """Time the oracle (CPU restatement) on a bounded sample of the workload:
    the same grid, a few steps, in the timed mode and in FP64."""
    import ffe
    threads = threads or os.cpu_count() or 1
    edge = edge or args.cpu_sample or args.size
    steps = steps or args.cpu_steps or max(2, min(50, int(3 * (512.0 / edge) ** 3)))
    size = (edge, edge, edge)
    prec = ffe.PRECISIONS[args.precision]
    s_step = time_oracle(size, prec, steps, threads)
    s64 = time_oracle(size, ffe.FP64, max(1, steps // 2), threads)
    return {"value": edge ** 3 / s_step, "unit": "cell-updates/s", "cores": threads, "kind": "port",
            "cpu": cpu_model(),
            "sample": "%d^3 grid of the same random-mode workload, %d steps after 1 warm-up, %s, x-innermost "
                      "loops, OpenMP %d threads, %.1f s" % (edge, steps, args.precision, threads, s_step * steps),
            "fp64": {"value": edge ** 3 / s64, "unit": "cell-updates/s", "steps": max(1, steps // 2)}}


def rel_errors(a, b):
    """Relative L2 and L-infinity error of E and B of a against b (dicts of
    interior arrays)."""
    import numpy as np
    names = ("ex", "ey", "ez", "bx", "by", "bz")
    res = {}
    for grp, comps in (("E", names[:3]), ("B", names[3:])):
        num2 = den2 = linf = dmax = 0.0
        for n in comps:
            x = a[n].astype(np.float64)
            y = b[n].astype(np.float64)
            d = x - y
            num2 += float(np.vdot(d, d).real)
            den2 += float(np.vdot(y, y).real)
            linf = max(linf, float(np.max(np.abs(d))))
            dmax = max(dmax, float(np.max(np.abs(y))))
        res[grp] = {"rel_l2": (num2 / den2) ** 0.5 if den2 else None, "rel_linf": linf / dmax if dmax else None}
    return res


def line_accuracy(args, size, bg, modes, stream):
    """Accuracy of the timed mode, stated beside the timed number: relative L2
    and L-infinity of E and B after --accuracy-line-steps steps against the
    FP64 path from the same initial fields; and the FP64 GPU path against
    the CPU oracle (FP64, OpenMP) after --oracle-check-steps steps.  The FP64
    GPU path stands in for the oracle over the longer run once it matches
    it over the short one."""
    import ffe
    names = ("ex", "ey", "ez", "bx", "by", "bz")
    prec = ffe.PRECISIONS[args.precision]
    n_acc, n_ora = args.accuracy_line_steps, args.oracle_check_steps
    out = {}
    g64 = ffe.Solver(ffe.make_desc(size, precision=ffe.FP64, stream=stream))
    g64.init_waves(bg, modes)
    g64.mainloop_prologue()
    done = 0
    if n_ora:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build()
        init = g64.fields()
        o = O.Oracle(ffe.make_desc(size, precision=ffe.FP64), threads=os.cpu_count() or 1, loop_order=1)
        o.set_fields(init)
        del init
        g64.mainloop(n_ora, 0)
        done = n_ora
        t0 = time.perf_counter()
        o.mainloop(n_ora, 0)
        t_ora = time.perf_counter() - t0
        cpu = {n: ffe.interior(o.download(n)) for n in names}
        o.close()
        gpu = {n: ffe.interior(a) for n, a in g64.fields().items()}
        out["fp64_gpu_vs_cpu_oracle"] = dict(rel_errors(gpu, cpu), steps=n_ora, oracle_seconds=round(t_ora, 1))
        del cpu, gpu
    if n_acc and prec != ffe.FP64:
        g = ffe.Solver(ffe.make_desc(size, precision=prec, stream=stream))
        g.init_waves(bg, modes)
        g.mainloop_prologue()
        g.mainloop(n_acc, 0)
        mine = {n: ffe.interior(a) for n, a in g.fields().items()}
        g.close()
        g64.mainloop(n_acc - done, done)
        ref = {n: ffe.interior(a) for n, a in g64.fields().items()}
        out["vs_fp64"] = dict(rel_errors(mine, ref), steps=n_acc, mode=args.precision,
                              reference="the FP64 GPU path from the same initial fields")
    g64.close()
    return out


def run_reference(args):
    """The reference's CPU path: its Fortran build is unavailable (no Fortran
    compiler, MPI or HDF5 in this image or on the GPU hosts), so the CPU
    restatement of the same procedures (oracle/) runs on all host cores, on
    the benchmark grid itself (--size, 512^3 by default), in the reference's
    arithmetic (FP32: its default real)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import ffe
    edge = args.cpu_sample or args.size
    threads = os.cpu_count() or 1
    size = (edge, edge, edge)
    s_step = time_oracle(size, ffe.FP32, args.steps, threads, warm=args.warmup)
    v = edge ** 3 / s_step
    cfg = {"workload": "random Alfven+fast modes, periodic %d^3" % edge
                       + ("" if edge == args.size else " (CPU sample of the %d^3 grid)" % args.size),
           "grid": [args.size] * 3, "modes": 32, "kmax": 8, "amax": 0.02, "cc": 0.45,
           "boundary": "periodic", "parallelism": "replicas" if world > 1 else "single grid"}
    line = {"metric": "cell-updates/s per RK3 step", "value": v, "unit": "cell-updates/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * s_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic", "config": cfg, "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                             "cpu": cpu_model(),
                             "sample": "%d^3 grid, %d steps after %d warm-up, fp32 (the reference's real); the "
                                       "reference's Fortran build is unavailable (no Fortran compiler, MPI, "
                                       "HDF5), so its CPU restatement runs" % (edge, args.steps, args.warmup)},
            "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def bench_batch(args):
    """Batched workload: `--batch-boxes` boxes with sides U[48, 160] per axis
    (half Alfven packets, half twisted flux tubes; `--batch-kind packet`:
    packets only), `--steps` steps.  Times the batch (autotuned tiling or
    `--tile-y`, one launch per stage and variant for all boxes, CUDA graph)
    and the plain path that runs the same boxes one grid at a time, from the
    same initial state; reports both rates, time-to-result percentiles and the
    largest relative L2 difference between the two results."""
    import numpy as np
    import torch
    import ffe
    import build as ffe_build
    from ffe import workloads
    torch.cuda.set_device(0)
    ffe_build.build()
    prec = ffe.PRECISIONS[args.precision]
    specs = workloads.batch_boxes(args.batch_boxes, kind=args.batch_kind)
    cells = [s["size"][0] * s["size"][1] * s["size"][2] for s in specs]
    K = args.batch_steps
    # one grid at a time: each box runs all K steps, then the next box
    seq = [workloads.build_solver(sp, prec) for sp in specs]
    for g in seq:
        g.mainloop(args.warmup, 0)
    for g in seq:
        g.synchronize()
    done = []
    t0 = time.perf_counter()
    for g in seq:
        g.mainloop(K, args.warmup)
        g.synchronize()
        done.append(time.perf_counter() - t0)
    t_seq = time.perf_counter() - t0
    # batched
    bat = [workloads.build_solver(sp, prec) for sp in specs]
    b = ffe.Batch(bat)
    b.step(args.warmup)
    b.synchronize()
    if args.tile_y:
        b.set_tiling(args.tile_y, 0, False)
        tune_ms = None
    else:
        tune_ms = b.autotune(reps=3)
    tiling = b.tiling()
    t0 = time.perf_counter()
    b.step(K, step0=[args.warmup] * len(bat))
    b.synchronize()
    t_bat = time.perf_counter() - t0
    diff = 0.0
    for gs, gb in zip(seq, bat):
        for grp in (("ex", "ey", "ez"), ("bx", "by", "bz")):
            x = np.concatenate([ffe.interior(gs.download(k)).ravel().astype(np.float64) for k in grp])
            y = np.concatenate([ffe.interior(gb.download(k)).ravel().astype(np.float64) for k in grp])
            diff = max(diff, float(np.linalg.norm(x - y) / max(np.linalg.norm(x), 1e-300)))
    launches = b.launches()
    b.close()
    for g in seq + bat:
        g.close()
    total = float(sum(cells)) * K
    pct = lambda v, q: float(np.percentile(np.asarray(v), q))
    print(json.dumps({
        "metric": "aggregate cell-updates/s, batched uneven boxes", "value": total / t_bat,
        "unit": "cell-updates/s", "n_gpus": 1, "steps": K, "warmup": args.warmup,
        "higher_is_better": True, "dtype": args.precision, "data": "synthetic",
        "one_grid_at_a_time": total / t_seq, "speedup_vs_one_at_a_time": t_seq / t_bat,
        "time_to_result_s": {"batched_all_boxes": t_bat,
                             "one_at_a_time": {"p50": pct(done, 50), "p99": pct(done, 99), "last": t_seq},
                             "note": "the batch advances every box in one call, so all its results arrive "
                                     "together; one at a time, box i's result arrives after boxes 0..i"},
        "max_rel_l2_batched_vs_single": diff, "tiling": tiling, "autotune_ms_per_stage": tune_ms,
        "gpu_launches": launches * K,
        "config": {"workload": "%d boxes, sides U[48,160], %s"
                               % (len(specs), "Alfven packets" if args.batch_kind == "packet"
                                  else "half Alfven packets, half twisted flux tubes"),
                   "cells": int(sum(cells)),
                   "timing": "host clock around synchronised runs (includes launch overhead of both paths)"},
    }))


def bench_psr(args):
    """The pulsar magnetosphere at --size^3 (512^3): user_psr with a rotating
    conducting sphere of radius 24 cells at the centre, inclination 30
    degrees, light cylinder at 120 cells (period 2 pi 120 / c steps), the
    dipole scaled to B = 1e3 at the stellar surface, an absorbing shell 48
    cells thick (user/user_psr.F90:72-383, src/algorithms/field_solver.F90:
    198-268).  The reference's shell (jg = i + y0, clamped, TINY in the
    cleaning) and the true-y shell, one line each: the step rate of FP32C and
    of FP32CD (B^2 denominators in double) with the roofline at 54 words per
    cell-update, and their relative L2 / L-infinity error of E and B against
    the FP64 path at the step counts of --psr-marks."""
    import math
    import torch
    import ffe
    import build as ffe_build
    torch.cuda.set_device(0)
    ffe_build.build()
    S = args.size
    cc = 0.45
    params = (24.0 * S / 512, 30.0, 2.0 * math.pi * (120.0 * S / 512) / cc, 1000.0)
    buff = int(round(48 * S / 512))
    marks = [int(m) for m in args.psr_marks.split(",") if m]
    peak, peak_kind = peaks()
    names = ("ex", "ey", "ez", "bx", "by", "bz")
    base = ffe.FLAG_ABSORB_CLAMP | ffe.FLAG_CLEAN_TINY
    stream = torch.cuda.Stream()

    def make(prec, flags):
        d = ffe.make_desc((S,) * 3, precision=prec, boundary=(ffe.ABSORB,) * 3, absorb_buff=buff, cc=cc,
                          setup=ffe.SETUP_PSR, params=params, flags=flags, stream=stream.cuda_stream)
        g = ffe.Solver(d)
        g.userInitialize()
        g.mainloop_prologue()
        return g

    for label, flags in (("reference shell (jg = i + y0), clamped", base),
                         ("true-y shell, clamped", base | ffe.FLAG_ABSORB_TRUE_Y)):
        rates = {}
        for pn in ("fp32c", "fp32cd"):
            g = make(ffe.PRECISIONS[pn], flags)
            g.mainloop(args.warmup, 0)
            g.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            k = args.steps if pn == "fp32c" else max(2, args.steps // 5)
            e0.record(stream)
            g.mainloop(k, args.warmup)
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1) / k
            ach = S ** 3 * WORDS_PER_CELL_STEP * 4 / (ms / 1e3) / 1e9
            rates[pn] = {"value": S ** 3 / (ms / 1e3), "ms_per_step": ms, "steps": k,
                         "roofline_frac": ach / peak, "finite": g.check_finite()}
            g.close()
        runs = {pn: make(ffe.PRECISIONS[pn], flags) for pn in ("fp64", "fp32c", "fp32cd")}
        errs, done = [], 0
        t0 = time.perf_counter()
        for m in marks:
            for g in runs.values():
                g.mainloop(m - done, done)
            done = m
            ref = {n: ffe.interior(a) for n, a in runs["fp64"].fields().items()}
            row = {"step": m}
            for pn in ("fp32c", "fp32cd"):
                row[pn] = rel_errors({n: ffe.interior(a) for n, a in runs[pn].fields().items()}, ref)
            errs.append(row)
        for g in runs.values():
            g.close()
        print(json.dumps({
            "metric": "cell-updates/s per RK3 step, pulsar magnetosphere", "value": rates["fp32c"]["value"],
            "unit": "cell-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": rates["fp32c"]["ms_per_step"], "higher_is_better": True, "dtype": "fp32c",
            "data": "synthetic", "shell": label, "rates": rates,
            "roofline": {"bound": "hbm", "peak": peak, "unit": "GB/s", "words_per_cell_update": WORDS_PER_CELL_STEP,
                         "peak_source": peak_kind},
            "error_vs_fp64": errs, "error_seconds": time.perf_counter() - t0,
            "config": {"workload": "pulsar magnetosphere %d^3" % S, "psr_radius": params[0],
                       "inclination_deg": 30.0, "light_cylinder": 120.0 * S / 512, "period_steps": params[2],
                       "surface_b": 1000.0, "absorb_buff": buff, "cc": cc,
                       "stopped_at_step": marks[-1] if marks else 0}}), flush=True)


def psr_accuracy(args):
    """Sensitivity of the served pulsar configuration (cubic side --size,
    inclination 30 degrees, R = side/10, absorbing shell of ceil(side*48/512)
    cells with the clamp and cleaning TINY): relative L2 of E and B of FP32,
    FP32C and of the FP64 staged path against the FP64 fused path at several
    step counts, with the reference's shell and with FFE_FLAG_ABSORB_TRUE_Y."""
    import numpy as np
    import torch
    import ffe
    import build as ffe_build
    from ffe import workloads
    torch.cuda.set_device(0)
    ffe_build.build()
    side = args.size
    marks = [25, 50, 100, 200, 400]
    names = ("ex", "ey", "ez", "bx", "by", "bz")

    def err(a, b):
        out = {}
        for n, grp in (("E", names[:3]), ("B", names[3:])):
            x = np.concatenate([ffe.interior(a[k]).ravel().astype(np.float64) for k in grp])
            y = np.concatenate([ffe.interior(b[k]).ravel().astype(np.float64) for k in grp])
            out[n] = float(np.linalg.norm(x - y) / np.linalg.norm(x))
        return out

    def make(prec, flags, path=ffe.PATH_AUTO):
        d = ffe.make_desc((side,) * 3, precision=prec, boundary=(ffe.ABSORB,) * 3,
                          absorb_buff=int(np.ceil(side * 48 / 512)), setup=ffe.SETUP_PSR,
                          params=workloads.psr_params(side, 30.0), path=path, flags=flags)
        s = ffe.Solver(d)
        s.userInitialize()
        s.mainloop_prologue()
        return s

    base = ffe.FLAG_ABSORB_CLAMP | ffe.FLAG_CLEAN_TINY
    for label, flags in (("reference shell (jg = i + y0)", base), ("true-y shell", base | ffe.FLAG_ABSORB_TRUE_Y)):
        ref = make(ffe.FP64, flags)
        cand = {"fp32": make(ffe.FP32, flags), "fp32c": make(ffe.FP32C, flags),
                "fp64_staged": make(ffe.FP64, flags, ffe.PATH_STAGED)}
        done = 0
        for m in marks:
            for s in [ref] + list(cand.values()):
                s.mainloop(m - done, done)
            done = m
            fr = ref.fields()
            row = {"workload": "psr-accuracy", "shell": label, "side": side, "step": m}
            for n, s in cand.items():
                row[n] = err(fr, s.fields())
            print(json.dumps(row), flush=True)
        for s in [ref] + list(cand.values()):
            s.close()


def bench_serve(args):
    """Served workload: `--requests` pulsar runs arriving as a Poisson stream
    (20 per second; cubic sides U[96, 256], inclination U[0, 90] degrees,
    R = side/10, light cylinder 5R, steps U[200, 2000]) served by continuous
    batching under the HBM budget, then by the one-grid-at-a-time path on the
    same stream.  Reports aggregate cell-updates/s and time-to-result
    percentiles of both, and the relative L2 error of E and B of the
    `--fp64-checks` smallest runs against the same runs in FP64."""
    import numpy as np
    import torch
    import ffe
    import build as ffe_build
    from ffe import serve, workloads
    torch.cuda.set_device(0)
    ffe_build.build()
    prec = ffe.PRECISIONS[args.precision]
    reqs = workloads.served_requests(args.requests)
    check = sorted(reqs, key=lambda q: q["size"][0] ** 3 * q["steps"])[:args.fp64_checks]
    keep = {q["id"] for q in check}
    srv = serve.Server(precision=prec, hbm_budget=args.budget_gb * 1e9, epoch_steps=args.epoch_steps,
                       keep_results=keep, max_active_cells=int(args.max_active_cells))
    recs = srv.serve(reqs)
    served = serve.report(recs)
    plain = serve.report(serve.serve_plain(reqs, precision=prec))
    sjf = serve.Server(precision=prec, hbm_budget=args.budget_gb * 1e9, epoch_steps=args.epoch_steps,
                       policy="sjf", max_active_cells=int(args.max_active_cells))
    served_sjf = serve.report(sjf.serve(reqs))
    plain_sjf = serve.report(serve.serve_plain(reqs, precision=prec, policy="sjf"))
    def rel(ref, f):
        e = {}
        for name, grp in (("E", ("ex", "ey", "ez")), ("B", ("bx", "by", "bz"))):
            x = np.concatenate([ffe.interior(ref[k]).ravel() for k in grp])
            y = np.concatenate([ffe.interior(f[k]).ravel().astype(np.float64) for k in grp])
            e[name] = float(np.linalg.norm(x - y) / np.linalg.norm(x))
        return e

    errs = []
    for q in check:
        r = next(x for x in recs if x.id == q["id"])
        out = {}
        for path in (ffe.PATH_FUSED, ffe.PATH_STAGED):  # the FP64 fused path, and its own spread
            g = workloads.build_solver(q, ffe.FP64, path=path)
            g.mainloop(q["steps"], 0)
            g.synchronize()
            out[path] = g.fields()
            g.close()
        errs.append({"id": q["id"], "side": q["size"][0], "steps": q["steps"],
                     "rel_l2_vs_fp64": rel(out[ffe.PATH_FUSED], r.result),
                     "fp64_staged_vs_fp64_fused": rel(out[ffe.PATH_FUSED], out[ffe.PATH_STAGED])})
    print(json.dumps({
        "metric": "served aggregate cell-updates/s; p50/p99 time-to-result", "value": served["cell_updates_per_s"],
        "unit": "cell-updates/s", "n_gpus": 1, "higher_is_better": True, "dtype": args.precision,
        "data": "synthetic", "served": served, "one_grid_at_a_time": plain, "served_sjf": served_sjf,
        "one_grid_at_a_time_sjf": plain_sjf,
        "speedup_vs_one_at_a_time": served["cell_updates_per_s"] / plain["cell_updates_per_s"],
        "scheduler": {"epochs": srv.epochs, "batches_built": srv.batches_built, "peak_runs": srv.peak_runs,
                      "peak_bytes": srv.peak_bytes, "budget_bytes": srv.budget,
                      "host_s": {"wait": srv.t_wait, "admit": srv.t_admit, "build": srv.t_build,
                                 "finish": srv.t_finish}},
        "fp64_error": errs, "gpu_launches": srv.launches,
        "config": {"workload": "%d pulsar runs, Poisson 20/s, sides U[96,256], steps U[200,2000]" % len(reqs),
                   "epoch_steps": args.epoch_steps, "max_active_cells": int(args.max_active_cells)},
    }))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.accuracy_steps:
        accuracy(args)
        return
    if args.workload == "batch":
        bench_batch(args)
        return
    if args.workload == "psr-accuracy":
        psr_accuracy(args)
        return
    if args.workload == "psr":
        bench_psr(args)
        return
    if args.workload == "serve":
        if args.precision == "fp32":
            args.precision = "fp32c"  # the served runs are quoted at <= 1e-5 against FP64
        bench_serve(args)
        return
    import numpy as np
    import torch
    import ffe
    import build as ffe_build

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    if rank == 0:
        ffe_build.build()
    if world > 1:
        dist.barrier()

    S = args.size
    size = (S, S, S)
    prec = ffe.PRECISIONS[args.precision]
    stream = torch.cuda.Stream()
    desc = ffe.make_desc(size, precision=prec, stream=stream.cuda_stream)
    g = ffe.Solver(desc)
    bg, modes = workload(S)
    g.init_waves(bg, modes)
    g.mainloop_prologue()
    g.synchronize()
    launches_per_step = g.step_launches()
    path_name = "fused" if g.step_path() != ffe.PATH_STAGED else "staged"

    # ---- device-resident timing -------------------------------------------
    step = 0
    g.mainloop(args.warmup, step)
    step += args.warmup
    g.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        g.mainloop(args.steps, step)
        ev1.record(stream)
        ev1.synchronize()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
    step += args.steps
    t_ms = max_over_ranks(ev0.elapsed_time(ev1), world)
    ok = g.check_finite()
    cells = S ** 3
    ms_per_step = t_ms / args.steps
    value = job_rate(cells, args.steps, world, t_ms / 1e3)

    # ---- end to end through the C ABI from pinned host buffers ------------
    names = ("ex", "ey", "ez", "bx", "by", "bz")
    dt = np.float64 if prec == ffe.FP64 else np.float32
    host = {}
    for n in names:
        t = torch.empty(g.shape, dtype=torch.float64 if dt == np.float64 else torch.float32, pin_memory=True)
        a = t.numpy()
        host[n] = (t, a)
    g2 = ffe.Solver(ffe.make_desc(size, precision=prec, stream=stream.cuda_stream))
    g2.init_waves(bg, modes)
    for n in names:
        host[n][1][...] = g2.download(n)
    # two untimed copy passes: the first makes the staging buffers; the second
    # gives the copy rates of this host (they differ from host to host)
    arr_bytes = host["ex"][1].nbytes
    for _ in range(2):
        torch.cuda.synchronize()
        ta = time.perf_counter()
        g2.set_fields({n: host[n][1] for n in names})
        g2.synchronize()
        tb = time.perf_counter()
        g2.download_into({n: host[n][1] for n in names})
        g2.synchronize()
        tc = time.perf_counter()
    h2d_gbs, d2h_gbs = 6 * arr_bytes / (tb - ta) / 1e9, 6 * arr_bytes / (tc - tb) / 1e9
    # three timed runs, the median reported: the device-to-host rate of these
    # hosts varies from run to run (pinned-host writes at ~25 to ~190 GB/s)
    runs = []
    for _ in range(3):
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g2.set_fields({n: host[n][1] for n in names})        # ffe_upload_many
        g2.mainloop_prologue()
        g2.mainloop(args.steps, 0)
        g2.download_into({n: host[n][1] for n in names})     # ffe_download_many
        g2.synchronize()
        runs.append(max_over_ranks(time.perf_counter() - t0, world))
    e2e_s = sorted(runs)[1]
    e2e = {"value": job_rate(cells, args.steps, world, e2e_s), "unit": "cell-updates/s",
           "h2d_bytes_per_step": 6 * arr_bytes / args.steps, "d2h_bytes_per_step": 6 * arr_bytes / args.steps,
           "runs_s": runs, "h2d_gbs": h2d_gbs, "d2h_gbs": d2h_gbs,
           "note": "upload E,B + %d steps + download E,B per run, from pinned host memory; median of 3 runs; "
                   "h2d_gbs / d2h_gbs: the copy rates of an untimed pass on this host" % args.steps}
    g2.close()

    if rank != 0:
        if world > 1:
            dist.barrier()
        return
    peak, peak_kind = peaks()
    es = 8 if prec == ffe.FP64 else 4
    alg_bytes_step = cells * WORDS_PER_CELL_STEP * es
    achieved = alg_bytes_step / (ms_per_step / 1e3) / 1e9
    traffic = traffic_from_profile(args.precision, S)
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic,
            "kernel": "k_fused (3 fused stage launches per step) with the ghost fills after them: the whole "
                      "step, %d launches" % launches_per_step,
            "alg_bytes_per_launch": alg_bytes_step / 3, "words_per_cell_update": WORDS_PER_CELL_STEP,
            "frac_fused_words": achieved / peak * WORDS_FUSED_PATH / WORDS_PER_CELL_STEP,
            "peak_source": peak_kind + " copy bandwidth (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
            else "fallback 6800 GB/s"}
    others = {}
    if world == 1 and not args.no_other_precisions:
        # the same workload in the other precisions, for the FP32-vs-FP64 comparison of the metric
        g.close()
        for name, k, w in (("fp32", 10, 2), ("fp32c", 10, 2), ("fp32cd", 4, 1), ("fp64", 4, 1)):
            if name == args.precision:
                continue
            h = ffe.Solver(ffe.make_desc(size, precision=ffe.PRECISIONS[name], stream=stream.cuda_stream))
            h.init_waves(bg, modes)
            h.mainloop_prologue()
            h.mainloop(w, 0)
            h.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            h.mainloop(k, w)
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1) / k
            others[name] = {"value": cells / (ms / 1e3), "ms_per_step": ms, "steps": k, "warmup": w}
            h.close()
    acc = None
    if world == 1 and (args.accuracy_line_steps or args.oracle_check_steps):
        try:
            g.close()
            acc = line_accuracy(args, size, bg, modes, stream.cuda_stream)
        except Exception as e:
            acc = {"error": str(e)[:200]}
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        try:
            cpu = cpu_baseline(args)
        except Exception as e:
            cpu = {"value": None, "error": str(e)[:200]}
    clocks = clk.summary()
    cfg = {"workload": "random Alfven+fast modes, periodic %d^3, %s" % (S, args.precision),
           "grid": [S, S, S], "modes": 32, "kmax": 8, "amax": 0.02, "cc": 0.45, "boundary": "periodic",
           "l2": "inputs (3.3 GB per field set) larger than L2; no flush",
           "parallelism": "replicas x%d" % world if world > 1 else "single grid",
           "path": path_name}
    line = {"metric": "cell-updates/s per RK3 step", "value": value, "unit": "cell-updates/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.precision,
            "data": "synthetic", "config": cfg, "e2e": e2e, "roofline": roof, "cpu_baseline": cpu,
            "clocks": clocks, "gpu_launches": launches_per_step * args.steps, "finite": ok,
            "accuracy": acc, "other_precisions": others}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
