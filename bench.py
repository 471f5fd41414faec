#!/usr/bin/env python
"""Benchmark of the GB300 SBR path: rays x bounces/s (executed ray segments
per second) on the synthetic urban canyon (1 km^2, 400 boxes, 4,802 tris,
level-9 icosahedron = 2,621,442 rays, 6 reflections + 1 transmission, 10,000
receivers, isotropic Tx at 28 GHz).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line on rank 0.  `value` = segments / device time with the scene
and receivers resident (CUDA events on the engine's stream, from the first
kernel to the last, results left on the device).  `e2e` = the same metric
through the C ABI with host buffers: receivers copied in and fields + all
surviving paths copied out inside the timed region (wall clock).
Several GPUs (torchrun) run independent replicas, one per GPU; value sums
their segments over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NODE_BYTES = 96      # NodeRec
RAY_BYTES = 96       # RayRec
SEGMENT_BYTES = 84   # algorithmic bytes per executed segment (trace)
EVENT_BYTES = 16     # per capture event (group-table rank + count update)


def _env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.f = None

    def __enter__(self):
        try:
            self.f = tempfile.TemporaryFile("w+")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.f:
            return None
        self.f.seek(0)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = max(mx, float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_baseline(wl, level: int = 5, threads: int = 0):
    """The oracle (CPU restatement of the reference algorithm) on a bounded
    sample of the same workload: same scene, receivers and depth, level-5
    icosahedron (10,242 rays) instead of level 9."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build as oracle_build  # oracle/build.py
    oracle_build.build_oracle()
    import oracle as orc
    from copy import deepcopy
    req = deepcopy(wl.request)
    req.tessellation = level
    sc = orc.OracleScene.from_scene(wl.scene)
    nthreads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    out = orc.solve(sc, req, wl.scene.materials, threads=nthreads)
    dt = time.perf_counter() - t0
    seg = out["counts"]["segments"]
    return {"value": seg / dt, "unit": "segments/s", "cores": nthreads, "kind": "port",
            "sample": f"{wl.name} at icosahedron level {level} ({10 * 4 ** level + 2} rays, "
                      f"{len(req.rx)} receivers): {seg} segments in {dt:.2f} s"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    from sbrsolver_gb300 import scenes
    wl = scenes.urban_scene()
    level = 5
    vals = []
    for i in range(args.warmup + args.steps):
        b = cpu_baseline(wl, level)
        if i >= args.warmup:
            vals.append(b["value"])
    v = statistics.mean(vals)
    line = {"metric": "rays x bounces/s", "value": v, "unit": "segments/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl.name, "sample_level": level},
            "cpu_baseline": {"value": v, "unit": "segments/s", "cores": b["cores"],
                             "kind": "port", "sample": b["sample"]},
            "e2e": {"value": v, "unit": "segments/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--level", type=int, default=9,
                    help="icosahedron level (9 = the benchmark; lower for profiling runs)")
    args = ap.parse_args()
    rank, world, local = _env_int("RANK", 0), _env_int("WORLD_SIZE", 1), _env_int("LOCAL_RANK", 0)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    import numpy as np
    import torch

    torch.cuda.set_device(local)
    from sbrsolver_gb300 import api, scenes
    from sbrsolver_gb300.build import build_library
    build_library()

    wl = scenes.urban_scene(level=args.level)
    scene = api.DeviceScene.from_scene(wl.scene)
    rx_dev = torch.tensor(wl.request.rx, dtype=torch.float64, device=f"cuda:{local}")
    torch.cuda.synchronize()
    q_dev, _keep = api.request_from_workload(wl.request, args.precision)
    q_dev.rx = C.cast(C.c_void_p(rx_dev.data_ptr()), C.POINTER(C.c_double))
    q_dev.rx_on_device = 1
    req_dev = (q_dev, _keep)
    req_host = api.request_from_workload(wl.request, args.precision)

    for _ in range(args.warmup):
        api.solve(scene, req_dev, with_paths=False)
    # ---- device-resident timing
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    dev_ms, seg, stage = [], [], {"trace_ms": 0.0, "capture_ms": 0.0, "correct_ms": 0.0,
                                 "field_ms": 0.0}
    counts = None
    with Clocks(local) as ck:
        for _ in range(args.steps):
            r = api.solve(scene, req_dev, with_paths=False)
            dev_ms.append(r.timing["device_ms"])
            seg.append(r.counts["segments"])
            for k in stage:
                stage[k] += r.timing[k]
            counts = r.counts
    torch.cuda.synchronize()
    clocks = ck.summary()
    t_dev = sum(dev_ms) / 1e3
    # ---- end to end through the C ABI with host buffers
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_seg = 0
    d2h = 0
    for _ in range(args.steps):
        r = api.solve(scene, req_host, with_paths=True)
        e2e_seg += r.counts["segments"]
        d2h = 6 * 8 * len(wl.request.rx) + r.counts["paths"] * 64 + r.counts["rays"] * (12 + 48)
    torch.cuda.synchronize()
    t_e2e = time.perf_counter() - t0
    h2d = 8 * 3 * len(wl.request.rx) + 160
    # ---- aggregate over ranks (replicas)
    tot_seg, max_t, max_e2e, tot_e2e = sum(seg), t_dev, t_e2e, e2e_seg
    if dist:
        t = torch.tensor([float(sum(seg)), t_dev, t_e2e, float(e2e_seg)], dtype=torch.float64)
        g = [torch.zeros_like(t) for _ in range(world)]
        dist.all_gather(g, t)
        tot_seg = sum(x[0].item() for x in g)
        max_t = max(x[1].item() for x in g)
        max_e2e = max(x[2].item() for x in g)
        tot_e2e = sum(x[3].item() for x in g)
    if rank == 0:
        peak, peak_kind = peaks()
        steps = args.steps
        n_nodes = counts["segments"]
        depth = wl.request.max_reflection + wl.request.max_transmission
        cap_ms = stage["capture_ms"] / steps
        tr_ms = stage["trace_ms"] / steps
        if cap_ms >= tr_ms:
            kern, ms = "k_capture", cap_ms
            alg = n_nodes * NODE_BYTES + counts["captured"] * EVENT_BYTES
        else:
            kern, ms = "k_trace", tr_ms / (depth + 1)
            alg = n_nodes * SEGMENT_BYTES / (depth + 1)
        achieved = alg / (ms / 1e3) / 1e9
        launches_per_step = 6 + 7 + (depth + 1) + 1 + 2 + 1 + 4
        line = {
            "metric": "rays x bounces/s", "value": tot_seg / max_t, "unit": "segments/s",
            "n_gpus": world, "steps": steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * max_t / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic",
            "config": {"workload": wl.name, "triangles": wl.scene.n_tri,
                       "rays": counts["launches"], "receivers": len(wl.request.rx),
                       "max_reflection": wl.request.max_reflection,
                       "max_transmission": wl.request.max_transmission,
                       "field_precision": args.precision,
                       "parallelism": f"replicas{world}",
                       "l2": "working set (node pool) larger than L2 each step"},
            "counts": counts,
            "stages_ms": {k: v / steps for k, v in stage.items()},
            "e2e": {"value": tot_e2e / max_e2e, "unit": "segments/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": 1e3 * max_e2e / steps},
            "roofline": {"bound": "hbm", "kernel": kern, "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "algorithmic_bytes_per_launch": alg,
                         "launch_ms": ms},
            "gpu_launches": launches_per_step * steps,
            "clocks": clocks,
        }
        if not args.no_cpu_baseline and world == 1:
            try:
                line["cpu_baseline"] = cpu_baseline(wl)
            except Exception as e:  # reported, never fatal to the GPU number
                line["cpu_baseline"] = {"error": str(e)}
        print(json.dumps(line), flush=True)
    scene.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
