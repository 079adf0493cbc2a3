#!/usr/bin/env python3
"""Benchmark: primary protons per second of the GB300 proton transport (one JSON line).

Default workload (the configuration the headline metric is quoted on): a 256^3 phantom of 1 mm
voxels -- water with a 30 mm lung slab and a 15 mm bone slab -- and one 150 MeV Gaussian spot
(sigma 4 mm), 1e6 histories per step, FP32 stepping, FP64 dose tally.  A step transports the
1e6 histories; the tally accumulates over steps.  Inputs (density 67 MB, vertices 28 MB, dose
tally 134 MB) exceed the 129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mqi|reference] [--workload c2|c1]

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
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


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
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
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
        for ln in self.lines:
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
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def wave_traffic_per_step() -> float | None:
    """DRAM bytes per transport step of the wave kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "k_wave_traffic.json")
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
# GPU arm
# ------------------------------------------------------------------------------------------

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
    verts = wl.vertices(N, 3 + 1000 * rank)
    d_verts = torch.from_numpy(verts.view(np.uint8)).to(f"cuda:{local}")
    torch.cuda.synchronize()
    ctx.set_vertices_ptr(d_verts.data_ptr(), N, on_device=True)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    seed_base = 0x5EED0000 + 7919 * rank
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
    for k in range(args.steps):
        ctx.transport(0, N, seed_base + 100 + k)
    ev1.record(stream)
    torch.cuda.synchronize()
    t_wall1 = time.perf_counter()
    barrier()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    s1 = ctx.stats()
    ms_t = torch.tensor([ms], device=f"cuda:{local}")
    if ws > 1:
        torch.distributed.all_reduce(ms_t, op=torch.distributed.ReduceOp.MAX)
    ms_max = float(ms_t.item())
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
        "kernel": "k_wave", "algorithmic_bytes_per_launch": bytes_per_launch,
        "avg_launch_ms": wave_ms / max(launches, 1), "transport_steps_per_s": steps / (wave_ms / 1e3) if wave_ms else 0,
        "wave_share_of_step": wave_ms / ms if ms > 0 else None,
    }

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
    e_t = torch.tensor([e2e_ms], device=f"cuda:{local}")
    if ws > 1:
        torch.distributed.all_reduce(e_t, op=torch.distributed.ReduceOp.MAX)
    e2e_value = N * args.steps * ws / (float(e_t.item()) / 1e3)

    # ---- the replicas' dose volumes are summed once at the end (the path's only exchange step)
    if ws > 1:
        dose = torch.from_numpy(ctx.tally(sid)).to(f"cuda:{local}")
        torch.distributed.all_reduce(dose)

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
    args = ap.parse_args()
    from moquimc_gb300 import workloads

    wl = workloads.WORKLOADS[args.workload]()
    if args.impl == "reference":
        return run_reference(args, wl)
    return run_gpu(args, wl)


if __name__ == "__main__":
    sys.exit(main())
