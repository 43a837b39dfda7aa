#!/usr/bin/env python
"""Benchmark of the GB300 W-projection gridder.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload cfg2|cfg2b|cfg2s|cfg1|cfg0]

Prints one JSON line (rank 0).  The default workload is the SKA-LOW
EL56-82-shaped snapshot (cfg2: 31,395,840 visibilities, 8192^2 grid, 601
w-planes, support 4..72), the configuration the metric is stated on.  A step
is one gridding call over the whole workload (placement, binning, sort, tile gridding, partial reduction) onto a
complex64 grid that stays in HBM; inputs are resident on the device when the
timed region starts (``value``).  ``e2e`` is the same metric through the
reference-facing drop-in (oskar_grid_wproj_f, host buffers) with every host
to device and device to host copy inside the timed region.

``--impl reference`` times the reference's serial algorithm on the host
cores instead: the CPU restatement in oracle/ (bit-identical to the
reference's compiled oskar_grid_wproj_f, as the tests check), spread over all
host threads by grid-row bands so each cell is still accumulated in the
serial order.

Multi-GPU: the gridding call has no exchange step; under torchrun each rank
grids its own replica of the workload ("replicas only"), value = all ranks'
visibilities / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = ("Mvis/s & GFLOP/s on 1 GB300, batched vs plain, grid err "
          "≤1e-5 vs FP64 oracle")
UNIT = "Mvis/s"
GRID_TOL = 1e-5     # max |grid - FP64 oracle| / max |FP64 oracle|
PUBLISHED_P100_MVIS = {"cfg1": 2152800 / 0.074 / 1e6,
                       "cfg2": 31395840 / 0.781 / 1e6,
                       "cfg2b": 31395840 / 0.553 / 1e6}
WORKLOAD_TEXT = {
    "cfg0": "plain 200,000 vis on a 2048^2 grid, 128 w-planes, support "
            "4..24, oversample 4",
    "cfg1": "synthetic-challenge shape: 2,152,800 vis on an 8192^2 grid, "
            "714 w-planes, support 4..36, oversample 4",
    "cfg2": "SKA-LOW EL56-82 shape: 31,395,840 vis, 8192^2 grid, 601 "
            "w-planes, support 4..72",
    "cfg2b": "SKA-LOW EL82-70 shape: 31,395,840 vis, 8192^2 grid, 339 "
             "w-planes, support 8..44",
    "cfg2s": "SKA-LOW EL56-82 array with 60 time samples (7,848,960 vis), "
             "8192^2 grid, 601 w-planes, support 4..72 (profiling size)",
    "cfg4s": "64 channels (100-200 MHz, 0-60% flagged) of a 128-station "
             "SKA-LOW-like array, 120 times, 64 grids of 4096^2, 339 "
             "w-planes, support 8..44",
    "cfg4": "64 channels (100-200 MHz, 0-60% flagged) of the 512-station "
            "SKA-LOW array, 240 times, 64 grids of 4096^2, 339 w-planes, "
            "support 8..44",
}


def measure_batched(pkg, torch, steps, warmup=2, tune=None, name="cfg4",
                    threads=None):
    """Batched (one call for all channels) vs plain (one call per channel)
    on the 64-channel workload; both device-resident, CUDA-event timed,
    plus the batched call's replay on the kept geometry captured in a CUDA
    graph.  tune: a TuningCache -- the batched plan is tuned on the first
    six channels, the plain plan on channel 0's single calls -- or None for
    the per-call heuristics.  After the timing every channel's batched grid
    is compared with its plain grid on the device, and two channels (the
    first and the last) with the FP64 oracle on the host."""
    wl = load_workload(name)
    dev = torch.device("cuda", torch.cuda.current_device())
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    uu, vv, ww, vis, weight = (to(wl.uu), to(wl.vv), to(wl.ww), to(wl.vis),
                               to(wl.weight))
    C, G = wl.num_grids, wl.grid_size
    offs = [int(x) for x in wl.channel_offsets]
    grids = torch.zeros((C, G, G, 2), dtype=torch.float32, device=dev)
    plain_grids = torch.zeros((C, G, G, 2), dtype=torch.float32, device=dev)
    norms = torch.zeros(C, dtype=torch.float64, device=dev)
    skips = torch.zeros(C, dtype=torch.int64, device=dev)
    pnorms = torch.zeros(C, dtype=torch.float64, device=dev)
    pskips = torch.zeros(C, dtype=torch.int64, device=dev)
    stack = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    plain_plan = pkg.Plan()
    cell, wsc = np.float32(wl.cell_size_rad), np.float32(wl.w_scale)
    stream = torch.cuda.current_stream()
    tuning = None
    if tune is not None:
        from importlib import import_module
        at = import_module(pkg.__name__ + ".autotune")
        k = min(6, C)
        e, a, b = offs[k], offs[0], offs[1]
        sub_plan = pkg.Plan()
        tuning = {
            "batched": at.autotune(pkg, sub_plan, stack, uu[:e], vv[:e],
                                   ww[:e], vis[:e], weight[:e], cell, wsc, G,
                                   offsets=offs[:k + 1], cache=tune),
            "plain": at.autotune(pkg, plain_plan, stack, uu[a:b], vv[a:b],
                                 ww[a:b], vis[a:b], weight[a:b], cell, wsc,
                                 G, cache=tune)}
        plan.set_tuning(sub_plan.tuning())
        del sub_plan

    def batched():
        pkg.grid_wproj_batched_device(plan, stack, offs, uu, vv, ww, vis,
                                      weight, cell, wsc, G, grids, norms,
                                      skips, stream)

    def plain():
        for c in range(C):
            a, b = offs[c], offs[c + 1]
            pkg.grid_wproj_device(plain_plan, stack, uu[a:b], vv[a:b], ww[a:b],
                                  vis[a:b], weight[a:b], cell, wsc, G,
                                  plain_grids[c], pnorms[c:c + 1],
                                  pskips[c:c + 1], stream)

    out = {}
    for key, fn in (("plain", plain), ("batched", batched)):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(steps):
            fn()
        t1.record(stream)
        torch.cuda.synchronize()
        ms = t0.elapsed_time(t1) / steps
        out[key] = {"ms_per_step": ms,
                    "mvis_s": wl.num_points / (ms * 1e-3) / 1e6}
    out["speedup"] = out["plain"]["ms_per_step"] / out["batched"]["ms_per_step"]
    out["workload"] = f"{name}: {WORKLOAD_TEXT[name]}"
    out["num_vis"] = wl.num_points
    st = plan.stats()
    out["macs_per_step"] = st["num_macs"]
    out["records_per_step"] = st["num_records"]
    out["gflops_batched"] = 8.0 * out["macs_per_step"] / (
        out["batched"]["ms_per_step"] * 1e-3) / 1e9

    # Replay of the kept geometry (fixed uvw, new amplitudes each major
    # cycle) captured once in a CUDA graph and launched per step.
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        pkg.grid_wproj_batched_replay(plan, stack, vis, weight, grids, norms,
                                      skips)
    for _ in range(warmup):
        graph.replay()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(steps):
        graph.replay()
    t1.record(stream)
    torch.cuda.synchronize()
    pkg.check_plan(plan)
    ms = t0.elapsed_time(t1) / steps
    out["replay_graph"] = {"ms_per_step": ms,
                           "mvis_s": wl.num_points / (ms * 1e-3) / 1e6}
    out["replay_speedup_vs_plain"] = out["plain"]["ms_per_step"] / ms
    out["tuning"] = tuning or plan.tuning()
    del graph

    # Accuracy: one clean batched call and one clean plain pass.
    grids.zero_(); norms.zero_(); plain_grids.zero_(); pnorms.zero_()
    batched()
    plain()
    torch.cuda.synchronize()
    worst = 0.0
    for c in range(C):
        ref = plain_grids[c].double()
        scale = ref.abs().max().item()
        if scale > 0:
            worst = max(worst, (grids[c].double() - ref).abs().max().item()
                        / scale)
    acc = {"batched_vs_plain_max_rel": worst,
           "skips_equal": bool(torch.equal(skips, pskips)),
           "norm_max_rel": float(((norms - pnorms).abs() /
                                  pnorms.abs().clamp_min(1e-300)).max())}
    oracle = load_oracle()
    for c in sorted({0, C - 1}):
        ch = wl.channel(c)
        g64, ns64, nm64 = oracle.grid_f_fp64acc_mt(ch, threads=threads)
        e = error_vs(grids[c].cpu().numpy(), g64)
        acc[f"channel{c}_vs_fp64"] = dict(e, skips_equal=int(skips[c]) == ns64)
        del g64
    acc["ok"] = bool(acc["skips_equal"] and
                     all(acc[k]["max_rel"] <= GRID_TOL and
                         acc[k]["skips_equal"] for k in acc
                         if k.startswith("channel")))
    out["accuracy"] = acc
    del grids, plain_grids
    return out


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="cfg2",
                    choices=sorted(WORKLOAD_TEXT))
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the grid-error check against the FP64 "
                         "oracle (runs after the timed region)")
    ap.add_argument("--tile-shape", type=int, default=0,
                    help="force the tile width (32, 16, 8); 0 = automatic")
    ap.add_argument("--staging", type=int, default=-1,
                    help="kernel-slice staging: -1 automatic, 0 off, 1 on")
    ap.add_argument("--no-autotune", action="store_true",
                    help="use the per-call heuristics instead of tuning the "
                         "plans (tuning runs before the timed region)")
    ap.add_argument("--tuning", default=None,
                    help="plan settings as JSON (gg_tuning fields), applied "
                         "instead of tuning")
    ap.add_argument("--tune-cache", default=None,
                    help="autotuner cache file (default: $GPUGRID_TUNE_CACHE "
                         "or ~/.cache/gpugrid/tuning.json)")
    ap.add_argument("--batched-steps", type=int, default=3,
                    help="steps of the batched-vs-plain comparison on the "
                         "64-channel workload (0 = skip)")
    ap.add_argument("--batched-workload", default="cfg4",
                    choices=["cfg4", "cfg4s"],
                    help="the 64-channel workload of that comparison")
    return ap.parse_args()


def rank_info():
    return (int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def max_over_ranks(x, dist=None, device="cpu"):
    """The largest x over the ranks of the process group (x itself when
    dist is None): the job's step time is its slowest replica's."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world, units_per_rank, seconds):
    """Whole-job rate in millions of units per second: every one of the
    world replicas processed units_per_rank in (at most) seconds."""
    return world * units_per_rank / seconds / 1e6


def load_workload(name):
    synthetic = importlib.import_module("gpu-gridding_gb300.synthetic")
    return synthetic.WORKLOADS[name]()


L2_BYTES = 129 * 2 ** 20


def grid_exceeds_l2(wl):
    return 8 * wl.grid_size ** 2 > L2_BYTES


def workload_config(name, wl, extra=None):
    gmb = 8 * wl.grid_size ** 2 / 1e6
    l2 = (f"inputs larger than L2: the {wl.grid_size}^2 complex64 grid "
          f"({gmb:.0f} MB) is read and written every step"
          if grid_exceeds_l2(wl) else
          "L2 flushed between timed steps (256 MB write outside the "
          "per-step events)")
    cfg = {"workload": f"{name}: {WORKLOAD_TEXT[name]}",
           "num_vis": wl.num_points, "grid_size": wl.grid_size,
           "num_w_planes": wl.num_w_planes,
           "support": [int(wl.support.min()), int(wl.support.max())],
           "oversample": wl.oversample, "l2": l2,
           "parallelism": "replicas (no exchange step)"}
    if extra:
        cfg.update(extra)
    return cfg


# ---------------------------------------------------------------------------
# Clock sampling (nvidia-smi) during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id=None):
        self.gpu_id = gpu_id
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}",
               "--format=csv,noheader,nounits", "-lms", "200"]
        if self.gpu_id:
            cmd += ["-i", self.gpu_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=open(self.path, "w"),
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows
                          for i, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows),
                "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def gpu_uuid(torch, dev):
    try:
        u = torch.cuda.get_device_properties(dev).uuid
        s = str(u)
        return s if s.startswith("GPU-") else "GPU-" + s
    except Exception:
        return None


# ---------------------------------------------------------------------------
# CPU runs (reference algorithm on the host cores)
# ---------------------------------------------------------------------------
def load_oracle():
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle
    return oracle


def cpu_run(wl, threads, keep=False):
    """Seconds for one host-threaded oskar_grid_wproj_f pass over the
    workload; with keep, also the grid, skip count and norm."""
    oracle = load_oracle()
    grid = np.zeros((wl.grid_size, wl.grid_size, 2), np.float32)
    t0 = time.perf_counter()
    _, ns, nm = oracle.grid_f_mt(wl, grid, 0.0, threads=threads)
    t = time.perf_counter() - t0
    return (t, grid, ns, nm) if keep else t


def _err_sums(a, ref, rows=512):
    """(max |a - ref|, sum |a - ref|^2, max |ref|, sum |ref|^2) in FP64 over
    complex grids [G, G, 2], by bands of rows (no whole-grid temporaries)."""
    a = np.asarray(a)
    ref = np.asarray(ref)
    a2 = a.reshape(-1, *a.shape[-2:]) if a.ndim >= 2 else a.reshape(1, -1)
    r2 = ref.reshape(a2.shape)
    emax = esq = rmax = rsq = 0.0
    for i in range(0, a2.shape[0], rows):
        x = np.asarray(a2[i:i + rows], np.float64)
        y = np.asarray(r2[i:i + rows], np.float64)
        d = x - y
        if d.size:
            emax = max(emax, float(np.abs(d).max()))
            rmax = max(rmax, float(np.abs(y).max()))
        esq += float((d * d).sum())
        rsq += float((y * y).sum())
    return emax, esq, rmax, rsq


def max_rel_err(a, ref):
    """max |a - ref| / max |ref|, in FP64."""
    emax, _, rmax, _ = _err_sums(a, ref)
    return emax / rmax if rmax > 0 else emax


def error_vs(a, ref):
    """Max and RMS relative error of grid a against grid ref:
    max |a - ref| / max |ref| and sqrt(sum |a - ref|^2 / sum |ref|^2)."""
    emax, esq, rmax, rsq = _err_sums(a, ref)
    return {"max_rel": emax / rmax if rmax > 0 else emax,
            "rms_rel": float(np.sqrt(esq / rsq)) if rsq > 0 else
                float(np.sqrt(esq))}


def rel(x, ref):
    return abs(x - ref) / abs(ref) if ref else abs(x - ref)


def accuracy_vs_fp64(wl, grid, nskip, norm, threads, cpu_result=None,
                     with_d=True):
    """The measured workload's grid, skip count and norm against the
    oracles, after the timed region:

    * `vs_fp64`: the FP64-accumulation oracle with the FP32 placement of
      oskar_grid_wproj_f (the yardstick of the 1e-5 bound);
    * `vs_reference_d`: the reference's own FP64 gridder oskar_grid_wproj_d
      on the inputs promoted to FP64 (FP64 placement), with the count of
      visibilities whose FP32 and FP64 placements differ
      (`placement_disagreements`), which that comparison includes;
    * `vs_reference_f` (when the reference's FP32 gridder ran on the host,
      cpu_result): the GPU grid against it, with the stated tolerance
      max(1e-5, the reference _f's own max-rel error against the FP64
      oracle + 1e-6), and the reference _f's own errors beside ours.

    All errors are max |a - ref| / max |ref| and
    sqrt(sum |a - ref|^2 / sum |ref|^2)."""
    oracle = load_oracle()
    t0 = time.perf_counter()
    g64, ns64, nm64 = oracle.grid_f_fp64acc_mt(wl, threads=threads)
    e64 = error_vs(grid, g64)
    out = {"tolerance": GRID_TOL,
           "grid_max_rel_err": e64["max_rel"],
           "grid_rms_rel_err": e64["rms_rel"],
           "num_skipped": int(nskip), "num_skipped_fp64": ns64,
           "norm_rel_err": rel(norm, nm64),
           "vs_fp64": dict(e64, norm_rel=rel(norm, nm64),
                           oracle="FP64 sums, FP32 placement")}
    ok = e64["max_rel"] <= GRID_TOL and int(nskip) == ns64
    gref = None
    if cpu_result is not None:
        _, gref, ns_ref, nm_ref = cpu_result
        ef = error_vs(gref, g64)
        out["reference_f_max_rel_err"] = ef["max_rel"]
        out["reference_f_num_skipped"] = int(ns_ref)
        out["reference_f_norm_rel_err"] = rel(nm_ref, nm64)
        tol_f = max(GRID_TOL, ef["max_rel"] + 1e-6)
        eg = error_vs(grid, gref)
        out["vs_reference_f"] = dict(
            eg, tolerance=tol_f, norm_rel=rel(norm, nm_ref),
            num_skipped_equal=int(nskip) == int(ns_ref),
            reference_f_vs_fp64=ef)
        ok = ok and eg["max_rel"] <= tol_f and int(nskip) == int(ns_ref)
    del g64
    if with_d:
        gd, nsd, nmd = oracle.grid_d_promoted_mt(wl, threads=threads)
        dis, dis_gridded = oracle.placement_disagreements(wl)
        out["vs_reference_d"] = dict(
            error_vs(grid, gd), norm_rel=rel(norm, nmd),
            num_skipped_d=nsd, placement_disagreements=dis,
            placement_disagreements_gridded=dis_gridded,
            oracle="oskar_grid_wproj_d on the inputs promoted to FP64")
        if gref is not None:
            out["vs_reference_d"]["reference_f_vs_d"] = error_vs(gref, gd)
        del gd
    out["ok"] = bool(ok)
    out["oracle_seconds"] = time.perf_counter() - t0
    return out


# Visibilities per CPU step of the reference arm: a strided sample keeps a
# step to a few seconds on the host cores while holding the workload's own
# uv, w and support distribution.
CPU_SAMPLE_VIS = 8_000_000
# Visibilities of the single-thread figure (a strided sample again).
CPU_SAMPLE_VIS_1T = 1_000_000


def cpu_sample(wl, target):
    k = max(1, -(-wl.num_points // target))
    return wl.strided(k), k


def ordinal(k):
    """1st, 2nd, 3rd, 4th, ..., 11th, 12th, 13th, 21st, 32nd, ..."""
    if 10 <= k % 100 <= 20:
        return f"{k}th"
    return f"{k}" + {1: "st", 2: "nd", 3: "rd"}.get(k % 10, "th")


def single_thread_rate(wl):
    """Mvis/s of the serial restatement of oskar_grid_wproj_f on one host
    thread, on a strided sample of about CPU_SAMPLE_VIS_1T visibilities."""
    sample, k = cpu_sample(wl, CPU_SAMPLE_VIS_1T)
    oracle = load_oracle()
    grid = np.zeros((wl.grid_size, wl.grid_size, 2), np.float32)
    t0 = time.perf_counter()
    oracle.grid_f(sample, grid)
    t = time.perf_counter() - t0
    return {"value": sample.num_points / t / 1e6, "unit": UNIT, "cores": 1,
            "kind": "port",
            "sample": ("every visibility" if k == 1 else
                       f"every {ordinal(k)} visibility")
                      + f" ({sample.num_points} vis), "
                      "serial restatement of oskar_grid_wproj_f, one run"}


def run_reference(args):
    rank, _, world = rank_info()
    if rank != 0:
        return 0
    wl = load_workload(args.workload)
    sample, k = cpu_sample(wl, CPU_SAMPLE_VIS)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_run(sample, threads)
    times = [cpu_run(sample, threads) for _ in range(args.steps)]
    t = statistics.mean(times)
    value = sample.num_points / t / 1e6
    what = ("whole workload" if k == 1 else
            f"every {ordinal(k)} visibility of the workload")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "impl": "reference",
        "config": workload_config(args.workload, wl),
        "cpu_baseline": {
            "value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{what} ({sample.num_points} vis) per step; the "
                      "oracle's restatement of oskar_grid_wproj_f "
                      "(bit-identical to the reference build), grid rows "
                      f"split over {threads} host threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU run
# ---------------------------------------------------------------------------
def read_traffic(kernel, workload):
    """DRAM bytes of `kernel` per gridding step (all its plane-group passes)
    from the committed ncu summary (profiles/<kernel>_<workload>.txt, line
    'dram_bytes_per_step: X')."""
    path = os.path.join(HERE, "profiles", f"{kernel}_{workload}.txt")
    if not os.path.isfile(path):
        return None
    for line in open(path):
        if line.startswith("dram_bytes_per_step:"):
            try:
                return float(line.split(":", 1)[1])
            except ValueError:
                return None
    return None


def measured_peaks():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.isfile(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0}, "fallback"


def run_ours(args):
    import torch
    rank, local_rank, world = rank_info()
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl", device_id=torch.device(
            "cuda", local_rank))
    else:
        torch.cuda.set_device(0)
    pkg = importlib.import_module("gpu-gridding_gb300")
    if not os.path.isfile(pkg.LIB_PATH):
        pkg.build()
    wl = load_workload(args.workload)
    dev = torch.device("cuda", torch.cuda.current_device())

    def to_dev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    stack = pkg.KernelStack.from_workload(wl, "f")
    plan = pkg.Plan()
    uu, vv, ww = to_dev(wl.uu), to_dev(wl.vv), to_dev(wl.ww)
    vis, weight = to_dev(wl.vis), to_dev(wl.weight)
    G = wl.grid_size
    tune_cache, tuning = None, None
    if args.tuning:
        plan.set_tuning(json.loads(args.tuning))
    elif args.no_autotune or args.tile_shape or args.staging >= 0:
        plan.set_tile_shape(args.tile_shape)
        plan.set_slice_staging(args.staging)
    else:
        at = importlib.import_module(pkg.__name__ + ".autotune")
        tune_cache = at.TuningCache(args.tune_cache)
        tuning = at.autotune(pkg, plan, stack, uu, vv, ww, vis, weight,
                             np.float32(wl.cell_size_rad),
                             np.float32(wl.w_scale), G, cache=tune_cache)
    # The host-pointer entry points (the e2e leg) grid with the same
    # settings as the device-pointer plan.
    pkg.set_host_tuning(plan.tuning())
    grid = torch.zeros((G, G, 2), dtype=torch.float32, device=dev)
    norm = torch.zeros(1, dtype=torch.float64, device=dev)
    nskip = torch.zeros(1, dtype=torch.int64, device=dev)
    cell, wsc = np.float32(wl.cell_size_rad), np.float32(wl.w_scale)
    stream = torch.cuda.current_stream()

    def step():
        pkg.grid_wproj_device(plan, stack, uu, vv, ww, vis, weight, cell,
                              wsc, G, grid, norm, nskip, stream)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(max(args.warmup, 3)):
        step()
    barrier()
    clocks = ClockSampler(gpu_uuid(torch, dev))
    clocks.start()
    barrier()
    if grid_exceeds_l2(wl):
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(args.steps):
            step()
        t1.record(stream)
        barrier()
        ms = t0.elapsed_time(t1) / args.steps
    else:
        flush = torch.empty(256 * 2 ** 20, dtype=torch.uint8, device=dev)
        evs = [(torch.cuda.Event(enable_timing=True),
                torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        for a, b in evs:
            flush.fill_(1)
            a.record(stream)
            step()
            b.record(stream)
        barrier()
        ms = sum(a.elapsed_time(b) for a, b in evs) / args.steps
    clk = clocks.stop()
    ms_max = max_over_ranks(ms, dist, dev)
    stats = plan.stats()
    num_vis = wl.num_points
    value = replica_throughput(world, num_vis, ms_max * 1e-3)
    macs = stats["num_macs"]
    gflops = world * 8.0 * macs / (ms_max * 1e-3) / 1e9

    # Phase times of the same call, CUDA events on the launching stream.
    plan.set_profiling(True)
    phases = []
    for _ in range(max(3, min(args.steps, 10))):
        step()
        torch.cuda.synchronize()
        phases.append(plan.phase_ms())
    plan.set_profiling(False)
    phase_ms = {k: statistics.mean(p[k] for p in phases) for k in phases[0]}
    grid_ms = phase_ms["grid_tiles"]
    fma_peak = pkg.measure_fp32_fma_tflops()
    achieved = 8.0 * macs / (grid_ms * 1e-3) / 1e12
    peaks, peak_kind = measured_peaks()
    traffic = read_traffic("k_grid_tiles", args.workload)
    # Algorithmic bytes of one gridding-kernel launch: placed visibility
    # (cell, meta, weighted vis: 16 B) once per visibility, one 4-byte record
    # index per (visibility, tile), each re-laid kernel tap once (8 B), and
    # the grid read and written once (16 B per cell).
    stack_taps = int(sum(wl.oversample ** 2 *
                         (((wl.oversample + 1) // 2 + int(s) * wl.oversample)
                          // wl.oversample + 1) ** 2 for s in wl.support))
    alg_bytes = (16 * num_vis + 4 * stats["num_records"] + 8 * stack_taps +
                 16 * G * G)

    # End to end through the drop-in with pinned host buffers.
    def pinned(a):
        t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)),
                        pin_memory=True)
        t.numpy()[...] = a
        return t.numpy()

    h = {k: pinned(getattr(wl, k)) for k in
         ("support", "conv_func", "uu", "vv", "ww", "vis", "weight")}
    h_grid = pinned(np.zeros((G, G, 2), np.float32))

    def e2e_step():
        pkg.oskar_grid_wproj_f(wl.num_w_planes, h["support"], wl.oversample,
                               wl.conv_size_half, h["conv_func"], num_vis,
                               h["uu"], h["vv"], h["ww"], h["vis"],
                               h["weight"], cell, wsc, G, h_grid, 0.0)

    e2e = None
    host_tuning = None
    if args.e2e_steps > 0:
        # The host calls start from the plan's settings; the tile order and
        # plane groups are re-timed on the host buffers themselves, where
        # the grid is used in place (outside the timed region).
        if not args.tuning:
            at = importlib.import_module(pkg.__name__ + ".autotune")
            host_tuning = at.autotune_host(pkg, e2e_step, plan.tuning())
        e2e_step()
        barrier()
        call_ms, inside_ms = [], []
        te = time.perf_counter()
        for _ in range(args.e2e_steps):
            t_call = time.perf_counter()
            e2e_step()
            call_ms.append((time.perf_counter() - t_call) * 1e3)
            inside_ms.append(pkg.host_last_call_ms()["return"])
        te = (time.perf_counter() - te) / args.e2e_steps
        te = max_over_ranks(te, dist, dev)
        # Bytes the drop-in copied in its last call (every step copies the
        # same): the grid comes back only where tiles hold records.
        h2d, d2h = pkg.host_last_transfer()
        # One more call with phase events (not timed above).
        pkg.set_host_profiling(True)
        e2e_step()
        host_phases = pkg.host_phase_ms()
        pkg.set_host_profiling(False)
        e2e = {"value": replica_throughput(world, num_vis, te), "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "host_buffers": "page-locked",
               "grid_access": ["copy", "pinned", "pageable"][
                   pkg.host_grid_access()],
               "host_tuning": host_tuning or pkg.host_tuning(),
               "call_ms": [round(t, 3) for t in call_ms],
               "call_ms_in_library": [round(t, 3) for t in inside_ms],
               "phase_ms": host_phases}
        # The same call on pageable (malloc) buffers, as a numpy caller
        # passes them (the grid's pages already touched).
        hp = {k: np.ascontiguousarray(v).copy() for k, v in h.items()}
        gp = np.zeros((G, G, 2), np.float32)
        gp[...] = 0.0

        def e2e_pageable():
            pkg.oskar_grid_wproj_f(wl.num_w_planes, hp["support"],
                                   wl.oversample, wl.conv_size_half,
                                   hp["conv_func"], num_vis, hp["uu"],
                                   hp["vv"], hp["ww"], hp["vis"],
                                   hp["weight"], cell, wsc, G, gp, 0.0)

        e2e_pageable()
        barrier()
        call_ms_p = []
        tp = time.perf_counter()
        for _ in range(args.e2e_steps):
            t_call = time.perf_counter()
            e2e_pageable()
            call_ms_p.append((time.perf_counter() - t_call) * 1e3)
        tp = (time.perf_counter() - tp) / args.e2e_steps
        tp = max_over_ranks(tp, dist, dev)
        h2d_p, d2h_p = pkg.host_last_transfer()
        e2e["pageable"] = {"value": replica_throughput(world, num_vis, tp),
                           "unit": UNIT, "h2d_bytes_per_step": h2d_p,
                           "d2h_bytes_per_step": d2h_p,
                           "call_ms": [round(t, 3) for t in call_ms_p]}
        del hp, gp

    # The operations either side of the gridder on the same workload: the
    # adjoint (degridding) and the uniform-weighting pair (density grid,
    # re-weighting), device-resident, CUDA-event timed.
    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    out_vis = torch.empty((num_vis, 2), dtype=torch.float32, device=dev)
    dens = torch.zeros((G, G), dtype=torch.float32, device=dev)
    w_out = torch.empty_like(weight)
    ms_degrid = timed(lambda: pkg.degrid_wproj_device(
        plan, stack, uu, vv, ww, cell, wsc, G, grid, out_vis, stream))
    ms_wwrite = timed(lambda: pkg.grid_weights_write_device(
        plan, uu, vv, weight, cell, G, dens, nskip, stream))
    ms_wread = timed(lambda: pkg.grid_weights_read_device(
        plan, uu, vv, weight, w_out, cell, G, dens, nskip, stream))
    # One training step of the autograd binding: the forward gridding into
    # a new grid, then the backward (the degridding kernel and the vis /
    # weight gradients) for dL/dgrid = a fixed random array.
    vis_req = vis.clone().requires_grad_(True)
    w_req = weight.clone().requires_grad_(True)
    target = torch.randn((G, G, 2), dtype=torch.float32, device=dev,
                         generator=torch.Generator(device=dev).manual_seed(5))

    def fwd_bwd():
        vis_req.grad = None
        w_req.grad = None
        g = pkg.GridWproj.apply(vis_req, w_req, uu, vv, ww, stack, plan, cell,
                                wsc, G)
        g.backward(target)

    with torch.cuda.stream(stream):
        ms_fb = timed(fwd_bwd)
    neighbours = {
        "degrid": {"ms_per_step": ms_degrid,
                   "mvis_s": num_vis / (ms_degrid * 1e-3) / 1e6,
                   "gflops": 8.0 * macs / (ms_degrid * 1e-3) / 1e9},
        "weights_write": {"ms_per_step": ms_wwrite,
                          "mvis_s": num_vis / (ms_wwrite * 1e-3) / 1e6},
        "weights_read": {"ms_per_step": ms_wread,
                         "mvis_s": num_vis / (ms_wread * 1e-3) / 1e6},
        "forward_backward": {"ms_per_step": ms_fb,
                             "mvis_s": num_vis / (ms_fb * 1e-3) / 1e6},
    }
    del out_vis, dens, w_out

    batched = None
    if args.batched_steps > 0 and world == 1:
        batched = measure_batched(pkg, torch, args.batched_steps,
                                  tune=tune_cache,
                                  name=args.batched_workload,
                                  threads=os.cpu_count() or 1)

    cpu, cpu_result = None, None
    threads = os.cpu_count() or 1
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu_result = cpu_run(wl, threads, keep=True)
        tc = cpu_result[0]
        cpu = {"value": num_vis / tc / 1e6, "unit": UNIT, "cores": threads,
               "kind": "port",
               "sample": f"whole workload ({num_vis} vis), one run; the "
                         "oracle's restatement of oskar_grid_wproj_f "
                         "(bit-identical to the reference build), grid rows "
                         f"split over {threads} host threads",
               "single_thread": single_thread_rate(wl)}

    accuracy = None
    if rank == 0 and not args.no_accuracy:
        # One clean call on the same inputs and plan, outside the timed
        # region, checked against the FP64 oracle.
        grid.zero_()
        norm.zero_()
        nskip.zero_()
        step()
        torch.cuda.synchronize()
        accuracy = accuracy_vs_fp64(wl, grid.cpu().numpy(),
                                    int(nskip.item()), float(norm.item()),
                                    threads, cpu_result)
    cpu_result = None

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": max(args.warmup, 3),
            "ms_per_step": ms_max, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded PCG64, shape-matched to the "
                    "reference's dataset)",
            "config": workload_config(args.workload, wl, {
                "macs_per_step": macs, "records_per_step":
                    stats["num_records"], "tile": [stats["tile_u"],
                                                    stats["tile_v"]],
                "slice_staging": stats["slice_staging"],
                "gridding_ctas": stats["num_ctas"],
                "chunk_records": stats["chunk_records"],
                "tuning": tuning or plan.tuning()}),
            "gflops": gflops,
            "phase_ms": phase_ms,
            "roofline": {
                "bound": "fp32_fma", "kernel": "k_grid_tiles",
                "achieved": achieved, "peak": fma_peak, "unit": "TFLOP/s",
                "frac": achieved / fma_peak if fma_peak else None,
                "peak_source": "measured in this run (FP32 FMA probe "
                               "kernel, gg_measure_fp32_fma_tflops)",
                "traffic": traffic,
                "algorithmic_bytes": alg_bytes,
                "hbm_achieved_gbs": alg_bytes / (grid_ms * 1e-3) / 1e9,
                "hbm_peak_gbs": peaks.get("hbm_gbs"),
                "hbm_peak_source": peak_kind},
            "cpu_baseline": cpu,
            "accuracy": accuracy,
            "e2e": e2e,
            "gpu_launches": args.steps * stats["num_launches"],
            "clocks": clk,
            "published_p100_mvis": PUBLISHED_P100_MVIS.get(args.workload),
            "batched_vs_plain": batched,
            "neighbours": neighbours,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
