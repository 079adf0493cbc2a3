#!/usr/bin/env python3
"""Benchmark: primary protons per second of the GB300 proton transport (one JSON line).

Default workload (the configuration the headline metric is quoted on): a 256^3 phantom of 1 mm
voxels -- water with a 30 mm lung slab and a 15 mm bone slab -- and one 150 MeV Gaussian spot
(sigma 4 mm), 1e6 histories per step, FP32 stepping, FP64 dose tally.  A step transports the
1e6 histories; the tally accumulates over steps.  Inputs (density 67 MB, vertices 28 MB, dose
tally 134 MB) exceed the 129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mqi|reference] [--workload c2|c1]

The line also carries plan-level sections measured on rank 0 (skip with --no-plan): "plan" -- the
synthetic CT with 2000 spots, one batched call vs one call per spot, and the time to the
reference's 1% criterion in the >50% dose region; "robust" -- 21 setup/density scenarios in one
queue drain; "dij" -- the Dij of the plan, its products and 100 optimisation iterations with a
finite-difference check of the gradient.  "robust_full" (only with --sections robust_full) -- the
whole c4 configuration, 2000 spots x 21 scenarios, autotuned, to the 1% criterion.

--impl reference times the reference's own CPU implementation (the staged reference build in
oracle/_ref) on the host cores for the same workload and metric.

Under torchrun (N > 1) every rank runs an independent replica with its own seed ("replicas only":
histories shard with no exchange inside the step); value = histories on all ranks / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "primary protons/s"
BYTES_PER_STEP_DOSE = 4 + 16   # density read + one FP64 tally read-modify-write per transport step


def dist_env():
    from moquimc_gb300 import replicas

    return replicas.world()


class ClockSampler:
    """nvidia-smi clock/throttle sampler run during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def stop(self, t0: float = None, t1: float = None) -> dict:
        """Summary of the samples read between t0 and t1 (perf_counter seconds, the timed region;
        a sample is read up to one interval after it is taken); all samples when none fell there."""
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        inside = [ln for t, ln in self.lines if t0 is not None and t0 <= t <= t1 + 0.1]
        for ln in inside or [ln for _, ln in self.lines]:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "window": "timed region" if inside else "whole sampling run (no sample inside the timed region)"}


def measured_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def fp64_atomic_peak(torch, device) -> float:
    """Measured rate of FP64 atomic adds to distinct addresses of an L2-resident array (random
    indices into 2^21 doubles = 16 MB), through torch's index_add_ (one atomicAdd per element):
    the denominator of the tally-update roofline.  Median of three timed runs of 2^26 adds."""
    n, m = 1 << 21, 1 << 26
    t = torch.zeros(n, dtype=torch.float64, device=device)
    idx = torch.randint(0, n, (m,), device=device, generator=torch.Generator(device=device).manual_seed(5))
    src = torch.ones(m, dtype=torch.float64, device=device)
    t.index_add_(0, idx, src)
    rates = []
    for _ in range(3):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        t.index_add_(0, idx, src)
        ev1.record()
        torch.cuda.synchronize()
        rates.append(m / (ev0.elapsed_time(ev1) / 1e3))
    return float(sorted(rates)[1])


def wave_traffic_per_step() -> float | None:
    """DRAM bytes per transport step of the wave kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "k_wave_traffic.txt")
    if os.path.exists(path):
        with open(path) as f:
            return float(json.load(f)["dram_bytes_per_step"])
    return None


# ------------------------------------------------------------------------------------------
# CPU baselines: the reference's own CPU build (oracle/_ref), run as P processes
# ------------------------------------------------------------------------------------------

def reference_cpu_sample(wl, histories_each: int, n_proc: int, seed0: int) -> dict:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import mqo  # noqa: E402  (the oracle is the checker / CPU baseline only)

    if not mqo.ref_available():
        raise RuntimeError("reference CPU build unavailable (no staged reference sources)")
    with tempfile.TemporaryDirectory(prefix="mqi_cpu_") as td:
        t0 = time.time()
        _, recs, _ = mqo.ref_phantom_parallel(wl.physics_debug, wl.lxyz, wl.pxyz, wl.nxyz, wl.energy,
                                              wl.spot_position, wl.spot_size, histories_each, n_proc, wl.hu, seed0,
                                              beam=wl.beam, workdir=td)
        wall = time.time() - t0
    slowest = max(r["transport_seconds"] for r in recs)
    total = histories_each * n_proc
    return {"value": total / slowest, "transport_seconds": slowest, "wall_seconds": wall, "histories": total}


def run_reference(args, wl):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    n_proc = os.cpu_count() or 1
    each = args.ref_histories
    for w in range(args.warmup):
        reference_cpu_sample(wl, max(each // 10, 50), n_proc, 7000 + w)
    vals, secs = [], []
    for k in range(args.steps):
        r = reference_cpu_sample(wl, each, n_proc, 9000 + 97 * k)
        vals.append(r["value"])
        secs.append(r["transport_seconds"])
    value = float(np.sum([each * n_proc for _ in vals]) / np.sum(secs))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "primaries/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(secs)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(wl, each * n_proc, "reference CPU build, one process per host core"),
        "cpu_baseline": {"value": value, "unit": "primaries/s", "cores": n_proc, "kind": "reference",
                         "sample": f"{each} histories per process x {n_proc} processes per step"},
        "e2e": {"value": value, "unit": "primaries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(wl, histories, note=""):
    return {"workload": wl.name, "voxels": list(wl.nxyz), "voxel_mm": [wl.lxyz[i] / wl.nxyz[i] for i in range(3)],
            "energy_MeV": wl.energy, "beam": f"{wl.beam} {wl.spot_size[0]} mm", "histories_per_step": histories,
            "physics_debug": bool(wl.physics_debug), "scorer": "dose_to_water (FP64 tally)",
            "l2": "inputs larger than L2 (density 4 B/voxel + FP64 tally 8 B/voxel)", **wl.meta,
            **({"note": note} if note else {})}


# ------------------------------------------------------------------------------------------
# Plan-level measurements (synthetic CT, 2000 spots): batched vs plain, time to 1% sigma, the Dij
# and its optimisation loop, robust scenarios.  Rank 0 only.
# ------------------------------------------------------------------------------------------

def _cuda_time(torch, fn):
    torch.cuda.synchronize()
    t = time.perf_counter()
    r = fn()
    torch.cuda.synchronize()
    return time.perf_counter() - t, r


def plan_section(torch, capi, workloads, args) -> dict:
    """C3: one batched plan call vs one call per spot (identical tracks and tallies), and the time
    to the reference's 1% criterion (mean sigma/mean over voxels above 50% of the maximum) by
    whole plan passes."""
    wl = workloads.c3()
    c = capi.Context(0)
    c.set_physics(False)
    cid = c.add_child(*wl.edges())
    c.set_hu(cid, wl.hu)
    sid = c.add_scorer(cid, capi.DOSE_W)
    d1, d2 = c.add_stat_scorers(cid)
    N = c.set_spot_plan(wl.spots)
    cum = c.plan_cum
    # the batched form runs with the launch shape, queue size and launch mode the tuner picks on a
    # sample of the plan (8e6 histories per candidate -- several queue loads, so that the launch
    # modes' behaviour at load boundaries shows -- with the dose and statistics scorers as timed)
    t_tune, tune = _cuda_time(torch, lambda: c.autotune(0, min(N, 8_000_000), 11, plan=True))
    best = tune[np.argmax(tune["histories_per_s"])]
    c.transport_plan(0, min(N, 200_000), 1)                       # warm-up
    c.reset()
    t_b, _ = _cuda_time(torch, lambda: c.transport_plan(0, N, 2))
    est1, nv = c.stat_uncertainty(d1, d2, N, 0.5)
    st = c.stats()
    c.reset()
    # the plain path: one mqi_transport_plan call per spot over the whole plan, in its best launch
    # mode (queue generations: no graph is captured per call); the streamed mode, which captures
    # and instantiates a graph on every call, is timed on a sample of spots beside it
    sub = list(range(0, len(wl.spots), args.plain_stride))
    h_sub = int(sum(int(cum[s + 1] - cum[s]) for s in sub))

    def plain(spots):
        for s in spots:
            c.transport_plan(int(cum[s]), int(cum[s + 1]), 2)

    t_ps, _ = _cuda_time(torch, lambda: plain(sub))
    c.set_launch_mode(streamed=0)
    plain(sub[:20])                                                 # warm-up in this mode
    c.reset()
    t_p, _ = _cuda_time(torch, lambda: plain(range(len(wl.spots))))
    c.set_launch_mode(streamed=int(best["streamed"]))               # back to the tuned batched form
    c.reset()
    t_s, (passes, achieved) = _cuda_time(
        torch, lambda: c.run_plan_until_stat(d1, d2, 0.01, 0.5, args.max_passes, 0x5EED))
    # the per-history batch estimator over the same number of passes, one batch per pass
    c.reset()
    for p in range(int(passes)):
        c.transport_plan(0, N, 0x5EED + 1000 + p)
        c.batch_accumulate(sid)
    batch_est, batch_vox, n_batches = c.batch_uncertainty(sid, 0.5) if passes >= 2 else (float("nan"), 0, passes)
    batched = N / t_b
    plain_rate = N / t_p
    out = {
        "workload": wl.name, "voxels": list(wl.nxyz), "voxel_mm": [0.98, 0.98, 2.0], "spots": len(wl.spots),
        "histories_per_pass": N, "physics_debug": False,
        "batched": {"primaries_per_s": batched, "seconds_per_pass": t_b, "steps_per_primary": st["steps"] / N,
                    "waves": st["waves"], "estimate_after_one_pass": est1, "voxels_above_50pct": nv,
                    "tuning": {"seconds": t_tune, "candidates": int(len(tune)),
                               "chosen": {"block": int(best["block"]), "blocks_per_sm": int(best["blocks_per_sm"]),
                                          "streamed": int(best["streamed"]),
                                          "primary_chunk": int(best["primary_chunk"])}}},
        "plain_per_spot": {"primaries_per_s": plain_rate, "seconds_per_pass": t_p, "spots_timed": len(wl.spots),
                           "histories_timed": N, "launch_mode": "queue generations",
                           "sample": "the whole plan, one mqi_transport_plan call per spot",
                           "streamed_with_graph_per_call": {"primaries_per_s": h_sub / t_ps, "spots": len(sub),
                                                            "sample": f"every {args.plain_stride}th spot"}},
        "batched_over_plain": batched / plain_rate,
        "time_to_1pct_sigma": {"criterion": "reference estimator <= 1% over voxels > 50% of max dose",
                               "batched_s": t_s, "passes": passes, "achieved": achieved,
                               "histories": passes * N,
                               "plain_s": passes * t_p,
                               "plain_note": "measured seconds of one full per-spot pass x the passes: the per-spot "
                                             "calls run the same histories and streams, so the tallies and the "
                                             "estimate after each pass are the batched run's",
                               "batch_estimator_same_passes": {"mean_rel_sigma": batch_est, "voxels": batch_vox,
                                                               "batches": n_batches}},
    }
    c.close()
    return out


def dij_section(torch, capi, workloads, optimize, stride: int = 1) -> dict:
    """C3 Dij (one batched pass) and C5: 100 projected-gradient iterations, FD check on 64 spots.
    stride > 1 keeps every stride-th spot (a smaller matrix, e.g. for a profiler capture)."""
    wl = workloads.c3()
    if stride > 1:
        wl.spots = wl.spots[::stride].copy()
    dev = torch.device("cuda:0")
    c = capi.Context(0)
    c.set_physics(False)
    cid = c.add_child(*wl.edges())
    c.set_hu(cid, wl.hu)
    cap = 1 << 31
    while stride > 1 and cap > (1 << 26) and cap // 2 >= 4 * int(wl.spots["histories"].sum()) * 16:
        cap //= 2   # ~16 entries per history at most, the table at most half full
    sid = c.add_dij_scorer(cid, capacity=cap)
    N = c.set_spot_plan(wl.spots)
    t_tr, _ = _cuda_time(torch, lambda: c.transport_plan(0, N, 7))
    t_bd, op = _cuda_time(torch, lambda: c.dij_build(sid, scale=1.0))
    target, organ, _ = workloads.c5_structures(wl)
    tgt = torch.from_numpy(target).to(dev)
    org = torch.from_numpy(organ).to(dev)
    d1 = op.matvec(torch.ones(op.n_spots, device=dev, dtype=torch.float64))
    op = c.dij_build(sid, scale=2.0 / float(d1[tgt].mean()))    # w = 1: 2 Gy mean target dose
    obj = optimize.make_objective(torch, tgt, org)
    lip = optimize.lipschitz(op, tgt, org)
    # warm-up: the first autograd pass of a process loads (and on a new architecture JIT-compiles)
    # torch's own kernels for the objective, which took ~10 s once on the box
    optimize.projected_gradient(op, obj, torch.ones(op.n_spots, device=dev), 3, lip=lip)
    t_opt, (w, hist) = _cuda_time(
        torch, lambda: optimize.projected_gradient(op, obj, torch.ones(op.n_spots, device=dev), 100, lip=lip))
    # where an iteration's time goes: the forward product alone, then forward + objective + backward
    w1 = torch.ones(op.n_spots, device=dev)
    t_f, _ = _cuda_time(torch, lambda: [op.matvec(w1) for _ in range(10)])

    def fwd_bwd():
        for _ in range(10):
            wv = w1.detach().requires_grad_(True)
            obj(optimize.dijmod.dose(op, wv)).backward()

    t_fb, _ = _cuda_time(torch, fwd_bwd)
    spots = np.random.default_rng(8).choice(op.n_spots, min(64, op.n_spots), replace=False)
    rel32, _, fd = optimize.fd_check(op, obj, w, spots, dtype=torch.float32)
    rel64, _, _ = optimize.fd_check(op, obj, w, spots, dtype=torch.float64)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = {}
    for name, fn, arg in (("forward", op.matvec, w), ("backward", op.rmatvec, torch.rand(op.n_voxels, device=dev))):
        fn(arg)
        ev0.record()
        for _ in range(10):
            fn(arg)
        ev1.record()
        torch.cuda.synchronize()
        times[name] = ev0.elapsed_time(ev1) / 10
    vr = c.dij_info(sid)["voxel_rows"]
    # algorithmic bytes: what each product must move at least.  D.w: spot + value per entry, row
    # voxel + indptr per voxel row, the dose zeroed and written.  D^T.g: voxel + value per entry,
    # g read once per voxel that has an entry, the gradient and its FP64 partials per spot.
    fwd_bytes = op.nnz * 8 + vr * 12 + op.n_voxels * 8
    bwd_bytes = op.nnz * 8 + vr * 4 + op.n_spots * 16
    hbm = measured_peaks()["hbm_gbs"]
    out = {
        "workload": "c3 Dij + c5 objective" + (f" (every {stride}th spot)" if stride > 1 else ""),
        "histories": N, "nnz": op.nnz, "voxel_rows": vr,
        "transport_primaries_per_s": N / t_tr, "build_s": t_bd,
        "forward_ms": times["forward"], "backward_ms": times["backward"],
        "forward_frac_hbm": fwd_bytes / (times["forward"] / 1e3) / 1e9 / hbm,
        "backward_frac_hbm": bwd_bytes / (times["backward"] / 1e3) / 1e9 / hbm,
        "optimisation": {"iterations": 100, "ms_per_iteration": t_opt * 10, "objective_first": float(hist[0]),
                         "objective_last": float(hist[-1]), "forward_call_ms": t_f * 100,
                         "forward_objective_backward_ms": t_fb * 100},
        "fd_check": {"spots": len(spots), "h": 1e-3, "nonzero": int((np.abs(fd) > 0).sum()),
                     "max_rel_err_fp32_grad": float(rel32.max()), "max_rel_err_fp64_grad": float(rel64.max())},
    }
    c.close()
    return out


def robust_section(torch, capi, workloads, args) -> dict:
    """C4 sample: 21 scenarios x every 20th spot of the plan in one queue drain."""
    wl = workloads.c3()
    scen = workloads.c4_scenarios()
    sub = wl.spots[::args.robust_stride].copy()
    c = capi.Context(0)
    c.set_physics(False)
    cid = c.add_child(*wl.edges())
    c.set_density(cid, c.hu_to_density(wl.hu.ravel()))
    c.add_scorer(cid, capi.DOSE_W)
    d1, d2 = c.add_stat_scorers(cid)
    es = [workloads.scenario_edges(wl, sh) for sh, _ in scen]
    c.set_scenarios(cid, [e[0] for e in es], [e[1] for e in es], [e[2] for e in es], [k for _, k in scen])
    N = c.set_spot_plan(sub)
    tune = c.autotune(0, min(N, 500_000), 11, plan=True)        # on the scenario workload itself
    best = tune[np.argmax(tune["histories_per_s"])]
    c.transport_plan(0, min(N, 50_000), 1)
    c.reset()
    t, _ = _cuda_time(torch, lambda: c.transport_plan(0, N, 2))
    est, _ = c.stat_uncertainty(d1, d2, N, 0.5)
    c.close()
    return {"scenarios": len(scen), "spots": len(sub), "histories": N, "instances": N * len(scen),
            "instance_primaries_per_s": N * len(scen) / t, "seconds": t, "worst_scenario_estimate": est,
            "sample": f"every {args.robust_stride}th spot of the c3 plan",
            "tuned": {"block": int(best["block"]), "blocks_per_sm": int(best["blocks_per_sm"]),
                      "streamed": int(best["streamed"]), "primary_chunk": int(best["primary_chunk"])}}


def robust_full_section(torch, capi, workloads, args) -> dict:
    """C4 as specified: the c3 CT and its whole 2000-spot plan x 21 scenarios (setup shifts 0 and
    +-3 mm on x, y and z, each with DensityScaling 1, 1.035 and 0.965) in one queue drain per pass,
    tuned by mqi_autotune on a sample of the plan, statistical stopping at 1% (the reference
    estimator over voxels above 50% of the maximum, the worst scenario) by whole passes."""
    wl = workloads.c3()
    scen = workloads.c4_scenarios()
    c = capi.Context(0)
    c.set_physics(False)
    cid = c.add_child(*wl.edges())
    c.set_density(cid, c.hu_to_density(wl.hu.ravel()))
    sid = c.add_scorer(cid, capi.DOSE_W)
    N = c.set_spot_plan(wl.spots)
    d1, d2 = c.add_stat_scorers(cid)
    es = [workloads.scenario_edges(wl, sh) for sh, _ in scen]
    c.set_scenarios(cid, [e[0] for e in es], [e[1] for e in es], [e[2] for e in es], [k for _, k in scen])
    # tuned on the scenario workload itself (500 000 histories x 21 scenarios per candidate): with 21
    # instances per history the launch mode that wins differs from the single-scenario plan's
    t_tune, tune = _cuda_time(torch, lambda: c.autotune(0, min(N, 500_000), 11, plan=True))
    best = tune[np.argmax(tune["histories_per_s"])]
    c.transport_plan(0, min(N, 50_000), 1)
    c.reset()
    t, (passes, achieved) = _cuda_time(
        torch, lambda: c.run_plan_until_stat(d1, d2, 0.01, 0.5, args.max_passes, 0xC4))
    st = c.stats()
    c.close()
    return {"workload": "c4: the c3 CT and 2000-spot plan x 21 scenarios", "scenarios": len(scen),
            "spots": len(wl.spots), "histories_per_pass": N, "passes": passes, "seconds": t,
            "worst_scenario_estimate": achieved,
            "instance_primaries_per_s": passes * N * len(scen) / t,
            "criterion": "reference estimator <= 1% over voxels > 50% of max dose, worst scenario",
            "tuning": {"seconds": t_tune, "candidates": int(len(tune)),
                       "chosen": {"block": int(best["block"]), "blocks_per_sm": int(best["blocks_per_sm"]),
                                  "streamed": int(best["streamed"]), "primary_chunk": int(best["primary_chunk"])}},
            "waves": st["waves"]}


# ------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------

def nvtx_range(torch, name):
    """Open (name) or close (None) the NVTX range around the timed steps, so that a profiler's
    launch list can be restricted to them (ncu --nvtx --nvtx-include "timed_steps/")."""
    try:
        if name is None:
            torch.cuda.nvtx.range_pop()
        else:
            torch.cuda.nvtx.range_push(name)
    except Exception:  # noqa: BLE001  (no NVTX in this torch build: nothing to mark)
        pass


def run_gpu(args, wl):
    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from moquimc_gb300 import capi

    N = args.histories or wl.histories
    ctx = capi.Context(local)
    stream = torch.cuda.Stream(device=local)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_physics(wl.physics_debug)
    xe, ye, ze = wl.edges()
    cid = ctx.add_child(xe, ye, ze)
    ctx.set_hu(cid, wl.hu)
    sid = ctx.add_scorer(cid, capi.DOSE_W)
    ctx.set_post_step_mode(args.post_step_mode)
    if args.queue_sort >= 0:
        ctx.set_queue_sort(args.queue_sort)
    from moquimc_gb300 import replicas

    vseed, seed_base = replicas.replica_seeds(rank)
    verts = wl.vertices(N, vseed)
    d_verts = torch.from_numpy(verts.view(np.uint8)).to(f"cuda:{local}")
    torch.cuda.synchronize()
    ctx.set_vertices_ptr(d_verts.data_ptr(), N, on_device=True)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    # the tuner picks the launch shape, queue size and launch mode on a sample of the workload
    # (into scratch tallies); results do not depend on the choice
    n_tune = N if args.tune_histories == 0 else args.tune_histories
    tune = ctx.autotune(0, min(N, n_tune), seed_base + 7) if args.tune_histories >= 0 else None
    for w in range(args.warmup):
        ctx.transport(0, N, seed_base + w)
    ctx.reset()
    s0 = ctx.stats()

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.4)
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    t_wall0 = time.perf_counter()
    nvtx_range(torch, "timed_steps")
    for k in range(args.steps):
        ctx.transport(0, N, seed_base + 100 + k)
    nvtx_range(torch, None)
    ev1.record(stream)
    torch.cuda.synchronize()
    t_wall1 = time.perf_counter()
    barrier()
    clk = clocks.stop(t_wall0, t_wall1)
    ms = ev0.elapsed_time(ev1)
    s1 = ctx.stats()
    ms_max = replicas.max_over_ranks(ms, device=f"cuda:{local}")
    value = N * args.steps * ws / (ms_max / 1e3)

    steps = s1["steps"] - s0["steps"]
    launches = s1["wave_launches"] - s0["wave_launches"]
    wave_ms = s1["wave_ms"] - s0["wave_ms"]
    gpu_launches = s1["kernel_launches"] - s0["kernel_launches"]
    peaks = measured_peaks()
    bytes_per_launch = BYTES_PER_STEP_DOSE * steps / max(launches, 1)
    achieved = bytes_per_launch / (wave_ms / max(launches, 1) / 1e3) / 1e9 if wave_ms > 0 else 0.0
    tps = wave_traffic_per_step()
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
        "frac": achieved / peaks["hbm_gbs"], "peak_source": f"{peaks['source']} hbm_gbs",
        "traffic": (tps * steps / max(launches, 1)) if tps else None,
        "kernel": "k_wave (timed with its post-step kernel k_post, which finishes the ~0.2% of steps that end "
                  "in a nuclear interaction)",
        "algorithmic_bytes_per_launch": bytes_per_launch,
        "avg_launch_ms": wave_ms / max(launches, 1), "transport_steps_per_s": steps / (wave_ms / 1e3) if wave_ms else 0,
        "wave_share_of_step": wave_ms / ms if ms > 0 else None,
    }
    # the tally updates: one FP64 atomic add per transport step (the dose scorer)
    steps_per_s = steps / (wave_ms / 1e3) if wave_ms else 0.0
    try:
        apeak = fp64_atomic_peak(torch, f"cuda:{local}")
        roofline["atomics"] = {"per_step": 1, "achieved_per_s": steps_per_s, "peak_per_s": apeak,
                               "frac": steps_per_s / apeak if apeak else None,
                               "peak_source": "measured here: torch index_add_ of FP64 into a 16 MB array, random indices"}
    except Exception as exc:  # noqa: BLE001  (the atomic peak is supplementary)
        roofline["atomics"] = {"error": f"{type(exc).__name__}: {exc}"}

    # ---- end to end through the C ABI with host buffers (pinned), H2D + D2H inside the region
    nvox = int(np.prod(wl.nxyz))
    h_verts = torch.from_numpy(verts.view(np.uint8).copy()).pin_memory()
    h_dose = torch.empty(nvox, dtype=torch.float64).pin_memory()
    ctx.set_vertices_ptr(h_verts.data_ptr(), N, on_device=False)
    ctx.transport(0, N, seed_base + 50)
    ctx.tally_to_ptr(sid, h_dose.data_ptr(), on_device=False)
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(args.steps):
        ctx.set_vertices_ptr(h_verts.data_ptr(), N, on_device=False)
        ctx.transport(0, N, seed_base + 500 + k)
        ctx.tally_to_ptr(sid, h_dose.data_ptr(), on_device=False)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = e0.elapsed_time(e1)
    e2e_value = N * args.steps * ws / (replicas.max_over_ranks(e2e_ms, device=f"cuda:{local}") / 1e3)

    # ---- the replicas' dose volumes are summed once at the end (the path's only exchange step)
    if ws > 1:
        replicas.sum_tallies(ctx.tally(sid), device=f"cuda:{local}")

    line = None
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            try:
                n_proc = os.cpu_count() or 1
                r = reference_cpu_sample(wl, args.ref_histories, n_proc, 4242)
                cpu = {"value": r["value"], "unit": "primaries/s", "cores": n_proc, "kind": "reference",
                       "sample": f"{args.ref_histories} histories per process x {n_proc} processes (transport phase, "
                                 f"slowest process)"}
            except Exception as exc:  # noqa: BLE001
                cpu = {"value": None, "unit": "primaries/s", "cores": 0, "kind": "reference",
                       "sample": f"unavailable: {exc}"}
        line = {
            "metric": METRIC, "value": value, "unit": "primaries/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(wl, N),
            "e2e": {"value": e2e_value, "unit": "primaries/s", "h2d_bytes_per_step": int(verts.nbytes),
                    "d2h_bytes_per_step": int(nvox * 8)},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": gpu_launches,
            "transport": {"steps_per_primary": steps / (N * args.steps), "tracks": s1["tracks"] - s0["tracks"],
                          "waves": s1["waves"] - s0["waves"], "host_wall_s": t_wall1 - t_wall0},
        }
        if tune is not None:
            best = tune[np.argmax(tune["histories_per_s"])]
            line["tuning"] = {"sample_histories": min(N, n_tune), "candidates": len(tune),
                              "chosen": {"block": int(best["block"]), "blocks_per_sm": int(best["blocks_per_sm"]),
                                         "streamed": int(best["streamed"]), "primary_chunk": int(best["primary_chunk"])},
                              "best_over_worst": float(tune["histories_per_s"].max() / tune["histories_per_s"].min())}
        if not args.no_plan:
            from moquimc_gb300 import optimize, workloads

            for key, fn in (("plan", lambda: plan_section(torch, capi, workloads, args)),
                            ("robust", lambda: robust_section(torch, capi, workloads, args)),
                            ("robust_full", lambda: robust_full_section(torch, capi, workloads, args)),
                            ("dij", lambda: dij_section(torch, capi, workloads, optimize, args.dij_stride))):
                if key not in args.sections.split(","):
                    continue
                try:
                    line[key] = fn()
                except Exception as exc:  # noqa: BLE001  (a failed section is reported, not hidden)
                    line[key] = {"error": f"{type(exc).__name__}: {exc}"}
        print(json.dumps(line), flush=True)
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("mqi", "reference"), default="mqi")
    ap.add_argument("--workload", choices=("c1", "c2"), default="c2")
    ap.add_argument("--histories", type=int, default=0)
    ap.add_argument("--ref-histories", type=int, default=3000, help="histories per CPU process per sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plan", action="store_true", help="skip the plan, robust and Dij sections")
    ap.add_argument("--sections", default="plan,robust,dij",
                    help="plan-level sections to run (comma-separated; robust_full -- the whole c4 configuration to 1%% "
                         "sigma, several minutes -- only when named)")
    ap.add_argument("--dij-stride", type=int, default=1, help="Dij section on every n-th spot of the plan")
    ap.add_argument("--plain-stride", type=int, default=10, help="time every n-th spot for the plain per-spot rate")
    ap.add_argument("--robust-stride", type=int, default=20, help="spots of the plan in the robust sample")
    ap.add_argument("--max-passes", type=int, default=30, help="plan passes allowed for the 1%% criterion")
    ap.add_argument("--post-step-mode", type=int, default=-1, choices=(-1, 0, 1),
                    help="nuclear post-steps: -1 by run size, 0 inside the wave, 1 in the post-step kernel")
    ap.add_argument("--queue-sort", type=int, default=-1,
                    help="sort the queue by energy bin before waves of at least this many entries (0: never; "
                         "-1: the library default)")
    ap.add_argument("--tune-histories", type=int, default=0,
                    help="tuner sample (0: the step's histories; -1: no tuning)")
    args = ap.parse_args()
    from moquimc_gb300 import workloads

    wl = workloads.WORKLOADS[args.workload]()
    if args.impl == "reference":
        return run_reference(args, wl)
    return run_gpu(args, wl)


if __name__ == "__main__":
    sys.exit(main())
