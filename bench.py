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
surviving paths copied out (into flat numpy arrays, the form of
sbr_result_paths) inside the timed region (wall clock).
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
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of k_trace's
# first launch of the level-9 urban solve (its 2,621,442 launch rays), from
# one ncu capture of that launch alone: profiles/k_trace_urban_L9_first_launch.md
TRACE_FIRST_LAUNCH_DRAM_BYTES = 277407488 + 698306816


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
                                          "--format=csv,noheader,nounits", "-lms", "50"],
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


def batched_workload(seed: int = 0x5B5 + 2, n_tx: int = 256):
    """256 transmitters on the urban scene (sbrsolver_gb300.scenes.batched_workload)."""
    from sbrsolver_gb300 import scenes
    return scenes.batched_workload(seed, n_tx)


def serving_stream(scene_wls, n: int, seed: int = 0x5B5 + 4):
    """Request mix on resident scenes: scene uniform, Tx uniform over the
    scene (2-40 m above its floor), frequency log-uniform 0.9-60 GHz,
    icosahedron level U{5..10}, receivers log-uniform 100-100k (1.5 m above
    the floor), 2-8 bounces."""
    import numpy as np
    from sbrsolver_gb300 import scenes
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        si = int(rng.integers(0, len(scene_wls)))
        wl = scene_wls[si]
        v = wl.scene.tri.reshape(-1, 3)
        lo, hi = v.min(0), v.max(0)
        floor = float(wl.request.rx[:, 2].min() - 1.5)
        nrx = int(round(np.exp(rng.uniform(np.log(100), np.log(100000)))))
        rx = np.column_stack([rng.uniform(lo[0], hi[0], nrx), rng.uniform(lo[1], hi[1], nrx),
                              np.full(nrx, floor + 1.5)])
        tx = (float(rng.uniform(lo[0], hi[0])), float(rng.uniform(lo[1], hi[1])),
              floor + float(rng.uniform(2, 40)))
        out.append((si, scenes.Request(
            tx=tx, rx=rx, max_reflection=int(rng.integers(2, 9)), max_transmission=0,
            frequency=float(np.exp(rng.uniform(np.log(0.9e9), np.log(60e9)))),
            tessellation=int(rng.integers(5, 11)), antenna=int(rng.integers(0, 3)))))
    return out


def run_batched(precision: str, best_rate: float = 0.0):
    """256 transmitters as one batched call against 256 plain calls, overall
    and per icosahedron level (each level's requests batched on their own).

    The batch's launch shapes come from the library's autotuner (run first,
    untimed).  Both paths are reported in wall-clock time through the C ABI
    and in device time (sbr_timing.device_ms).  The Amdahl ceiling is the
    speed-up the batch would show if every one of its segments ran at the
    best segment rate measured on this scene in this run (`best_rate`, the
    fastest of the batched solves and the single level-9 benchmark solve):
    plain time / (segments / best rate)."""
    from sbrsolver_gb300 import api
    wl, reqs = batched_workload()
    sc = api.DeviceScene.from_scene(wl.scene)
    qs = [api.request_from_workload(r, precision) for r in reqs]
    api.solve(sc, qs, with_paths=False)  # warm-up: sizes the buffers for the batch
    t0 = time.perf_counter()
    tuned = sc.autotune(qs, rounds=1)
    tune_s = time.perf_counter() - t0
    t_req, d_req, seg_req = [], [], []
    t0 = time.perf_counter()
    for q in qs:
        t1 = time.perf_counter()
        r = api.solve(sc, q, with_paths=False)
        t_req.append(time.perf_counter() - t1)
        d_req.append(r.timing["device_ms"] / 1e3)
        seg_req.append(r.counts["segments"])
    t_plain = time.perf_counter() - t0
    seg_plain = sum(seg_req)
    t0 = time.perf_counter()
    rb = api.solve(sc, qs, with_paths=False)
    t_batch = time.perf_counter() - t0
    d_batch = rb.timing["device_ms"] / 1e3
    by_level = {}
    rates = [rb.counts["segments"] / d_batch, best_rate]
    for lvl in sorted({r.tessellation for r in reqs}):
        idx = [i for i, r in enumerate(reqs) if r.tessellation == lvl]
        sub = [qs[i] for i in idx]
        api.solve(sc, sub, with_paths=False)  # sizes the workspace for this sub-batch
        t0 = time.perf_counter()
        rs = api.solve(sc, sub, with_paths=False)
        tb = time.perf_counter() - t0
        db = rs.timing["device_ms"] / 1e3
        rates.append(rs.counts["segments"] / db)
        tp = sum(t_req[i] for i in idx)
        dp = sum(d_req[i] for i in idx)
        seg = sum(seg_req[i] for i in idx)
        by_level[str(lvl)] = {"requests": len(idx), "segments": rs.counts["segments"],
                              "segment_share": seg / seg_plain,
                              "plain_time_share": tp / t_plain,
                              "plain": seg / tp, "batched": rs.counts["segments"] / tb,
                              "speedup": (rs.counts["segments"] / tb) / (seg / tp),
                              "plain_device": seg / dp, "batched_device": rs.counts["segments"] / db,
                              "speedup_device": (rs.counts["segments"] / db) / (seg / dp)}
    err = None
    if precision != "fp64":  # untimed: the batch's field error against FP64
        qc = [api.request_from_workload(r, precision, field_check=True) for r in reqs]
        rc = api.solve(sc, qc, with_paths=False)
        err = api.field_error_stats(rc.field, rc.field_fp64)
    sc.close()
    best = max(rates)
    d_plain = sum(d_req)
    return {"workload": "urban 256 Tx, levels 6-9, R5, 4096 shared receivers",
            "requests": len(qs), "segments": rb.counts["segments"],
            "batched": rb.counts["segments"] / t_batch, "plain": seg_plain / t_plain,
            "unit": "segments/s", "batched_s": t_batch, "plain_s": t_plain,
            "speedup": (rb.counts["segments"] / t_batch) / (seg_plain / t_plain),
            "batched_device_s": d_batch, "plain_device_s": d_plain,
            "speedup_device": (rb.counts["segments"] / d_batch) / (seg_plain / d_plain),
            "ceiling": {"best_rate": best,
                        "speedup": t_plain / (seg_plain / best),
                        "speedup_device": d_plain / (seg_plain / best),
                        "rule": "plain time / (segments / best segment rate measured on "
                                "this scene in this run)"},
            "autotuned": dict(tuned, tuning_s=tune_s),
            "by_level": by_level, "field_precision": precision,
            "field_error_vs_fp64": err}


def run_serving(precision: str, n_req: int = 96, rates=(10.0, 50.0, 500.0), slots: int = 2,
                policy=None, graphs: bool = True, arrival_seed: int = 99):
    """The config-4 mix through the server at Poisson arrival rates `rates`
    (req/s), against the same requests solved one at a time.  At the highest
    rate the queue saturates, so its throughput is the sustained capacity.
    Two slots: on this mix four concurrent solves gave 6 % more throughput at
    saturation but 2.4x the p99 latency at 50 req/s (large requests slowed by
    the ones sharing the GPU with them)."""
    import numpy as np
    from sbrsolver_gb300 import api, scenes
    wls = [scenes.small_scene(), scenes.urban_scene(), scenes.large_scene()]
    scs = [api.DeviceScene.from_scene(w.scene) for w in wls]
    if not graphs:
        for sc in scs:
            sc.set_tuning(pipeline_graph=-1)
    stream = serving_stream(wls, n_req)
    qs = [(si, api.request_from_workload(r, precision)) for si, r in stream]
    for si, q in qs:
        api.solve(scs[si], q, with_paths=False)  # warm-up: sizes every workspace
    # plain: one request at a time (service time of each, wall clock)
    t0 = time.perf_counter()
    seg, service = 0, []
    for si, q in qs:
        t1 = time.perf_counter()
        seg += api.solve(scs[si], q, with_paths=False).counts["segments"]
        service.append(time.perf_counter() - t1)
    plain = seg / (time.perf_counter() - t0)
    sweep = []
    for rate in rates:
        rng = np.random.default_rng(arrival_seed)
        arrivals = np.cumsum(rng.exponential(1.0 / rate, len(qs)))
        # the plain path under the same arrivals: one request at a time in
        # arrival order, each taking its measured service time
        free, plain_lat = 0.0, []
        for a, sv in zip(arrivals, service):
            free = max(free, a) + sv
            plain_lat.append(1e3 * (free - a))
        srv = api.Server(scs, slots=slots)
        if policy is not None:
            srv.set_policy(*policy)
        lat, seg_s, done = [], 0, 0
        t0 = time.perf_counter()
        nxt = 0
        while done < len(qs):
            now = time.perf_counter() - t0
            while nxt < len(qs) and arrivals[nxt] <= now:
                srv.submit(qs[nxt][0], qs[nxt][1], nxt)
                nxt += 1
            for c in srv.poll(timeout_ms=2 if nxt < len(qs) else 100):
                if c["status"] == 0:
                    lat.append(c["latency_ms"])
                    seg_s += c["counts"]["segments"]
                done += 1
        makespan = time.perf_counter() - t0
        srv.close()
        sweep.append({"rate_req_s": rate, "p50_ms": float(np.percentile(lat, 50)),
                      "p99_ms": float(np.percentile(lat, 99)), "served": seg_s / makespan,
                      "completed": len(lat), "makespan_s": makespan,
                      "plain_p50_ms": float(np.percentile(plain_lat, 50)),
                      "plain_p99_ms": float(np.percentile(plain_lat, 99)),
                      "plain_served": seg / max(free, 1e-9)})
    for sc in scs:
        sc.close()
    top = sweep[-1]
    levels = [r.tessellation for _, r in stream]
    return {"workload": "config-4 mix on 3 resident scenes (small, urban, large)",
            "requests": len(qs), "slots": slots, "unit": "segments/s", "plain": plain,
            "request_levels": {str(l): levels.count(l) for l in sorted(set(levels))},
            "service_ms": {"p50": float(np.percentile(service, 50)) * 1e3,
                           "max": float(max(service)) * 1e3},
            "field_precision": precision,
            "sweep": sweep, "served": top["served"], "p50_ms": top["p50_ms"],
            "p99_ms": top["p99_ms"], "speedup": top["served"] / plain}


def run_precision(level: int = 10, n_rx: int = 50000):
    """Precision study on the large terrain scene: the same solve with the
    field in FP64, in FP32 (Fresnel and rotations FP32, path length and phase
    FP64, compensated FP32 receiver sums) and in FP32 with an FP32 phase.
    Reports throughput per mode, whether the path sets are identical, and
    each FP32 mode's field error against the FP64 field (which the parity
    tests pin to the CPU oracle)."""
    import numpy as np
    from sbrsolver_gb300 import api, scenes
    t0 = time.perf_counter()
    wl = scenes.large_scene(level=level, n_rx=n_rx)
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    sc = api.DeviceScene.from_scene(wl.scene)
    create_s = time.perf_counter() - t0
    res = {}
    modes = {}
    for mode in ("fp64", "fp32", "fp32_phase"):
        q = api.request_from_workload(wl.request, mode, field_check=(mode != "fp64"))
        api.solve(sc, q, with_paths=False)  # warm-up (sizes the workspace)
        r = api.solve(sc, q, with_paths="arrays")
        res[mode] = r
        modes[mode] = {"device_ms": r.timing["device_ms"], "field_ms": r.timing["field_ms"],
                       "segments_per_s": r.counts["segments"] / (r.timing["device_ms"] / 1e3)}
    sc.close()
    ref = res["fp64"]
    for mode in ("fp32", "fp32_phase"):
        r = res[mode]
        modes[mode]["same_path_set"] = api.same_path_set(r.paths, ref.paths)
        modes[mode]["shadow_fp64_equals_fp64_run"] = bool(np.array_equal(r.field_fp64, ref.field))
        modes[mode]["error_vs_fp64"] = api.field_error_stats(r.field, ref.field)
        modes[mode]["device_reported"] = r.field_error
    c = ref.counts
    return {"workload": f"large terrain: {wl.scene.n_tri} tris, icosahedron level {level} "
                        f"({c['launches']} rays), R8 T0, {n_rx} receivers, half-wave 3.5 GHz",
            "segments": c["segments"], "paths": c["paths"], "rays": c["rays"],
            "scene_generation_s": gen_s, "scene_create_s": create_s, "modes": modes,
            "tolerance": {"rel_mag": 1e-4, "phase_rad": 1e-3}}


def replica_totals(dist, world: int, segments: float, seconds: float, e2e_segments: float,
                   e2e_seconds: float):
    """Whole-job totals of independent replicas: segments summed over ranks,
    time = the slowest rank's (device and end to end).  dist is
    torch.distributed (any backend) or None for one process."""
    if not dist:
        return segments, seconds, e2e_segments, e2e_seconds
    import torch
    t = torch.tensor([segments, seconds, e2e_segments, e2e_seconds], dtype=torch.float64)
    g = [torch.zeros_like(t) for _ in range(world)]
    dist.all_gather(g, t)
    return (sum(x[0].item() for x in g), max(x[1].item() for x in g),
            sum(x[2].item() for x in g), max(x[3].item() for x in g))


def run_reference(args, rank, world):
    if rank != 0:
        return
    from sbrsolver_gb300 import scenes
    wl = scenes.urban_scene()
    level = 5
    vals, secs = [], []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        b = cpu_baseline(wl, level)
        if i >= args.warmup:
            vals.append(b["value"])
            secs.append(time.perf_counter() - t0)
    v = statistics.mean(vals)
    line = {"metric": "rays x bounces/s", "value": v, "unit": "segments/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * statistics.mean(secs), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl.name, "triangles": wl.scene.n_tri,
                       "rays": 10 * 4 ** 9 + 2, "receivers": len(wl.request.rx),
                       "max_reflection": wl.request.max_reflection,
                       "max_transmission": wl.request.max_transmission,
                       "field_precision": "fp64", "parallelism": "host cores",
                       "sample": f"icosahedron level {level} of the same workload"},
            "cpu_baseline": {"value": v, "unit": "segments/s", "cores": b["cores"],
                             "kind": "port", "sample": b["sample"]},
            "e2e": {"value": v, "unit": "segments/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_scene_prep(api, scenes, reps: int = 3) -> dict:
    """Scene preparation of the large terrain: the library's own phase times
    (sbr_scene_info.prep_*) for the device build, best of `reps` after one
    untimed creation (CUDA context and module start-up), and the host build
    (SBR_SCENE_HOST_PREP) once."""
    wl = scenes.large_scene(level=5)
    api.DeviceScene.from_scene(wl.scene).close()
    fields = ("prep_total_ms", "prep_host_ms", "prep_device_tables_ms", "prep_search_bvh_ms",
              "prep_reference_bvh_ms", "prep_upload_ms")
    runs = []
    for _ in range(reps):
        t = time.perf_counter()
        sc = api.DeviceScene.from_scene(wl.scene)
        wall = 1e3 * (time.perf_counter() - t)
        inf = sc.info()
        runs.append(dict({f: getattr(inf, f) for f in fields}, wall_ms=wall))
        sc.close()
    t = time.perf_counter()
    sc = api.DeviceScene.from_scene(wl.scene, host_prep=True)
    host_ms = 1e3 * (time.perf_counter() - t)
    inf = sc.info()
    sc.close()
    best = min(runs, key=lambda r: r["wall_ms"])
    return {"metric": "scene preparation", "workload": "large terrain", "triangles": wl.scene.n_tri,
            "bvh_nodes": inf.n_bvh_nodes, "bvh_depth": inf.bvh_depth, "unit": "ms",
            "device_build": best, "device_runs_wall_ms": [r["wall_ms"] for r in runs],
            "host_build_wall_ms": host_ms}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32", "fp32_phase"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--level", type=int, default=9,
                    help="icosahedron level (9 = the benchmark; lower for profiling runs)")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-precision", action="store_true")
    ap.add_argument("--tuning", default="",
                    help="launch shapes of the benchmark scene, e.g. trace_kernel=2,find_steps=16 "
                         "(sbr_tuning field names; default: the library's)")
    ap.add_argument("--scene-prep", action="store_true",
                    help="only time the scene preparation of the large terrain (580,484 "
                         "triangles), device-built and host-built, and print that JSON line")
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
    if args.scene_prep:
        if rank == 0:
            print(json.dumps(run_scene_prep(api, scenes)))
        return

    wl = scenes.urban_scene(level=args.level)
    t_scene = time.perf_counter()
    scene = api.DeviceScene.from_scene(wl.scene)
    scene_ms = 1e3 * (time.perf_counter() - t_scene)
    if args.tuning:
        scene.set_tuning(**{k: int(v) for k, v in (kv.split("=") for kv in args.tuning.split(","))})
    rx_dev = torch.tensor(wl.request.rx, dtype=torch.float64, device=f"cuda:{local}")
    torch.cuda.synchronize()
    q_dev, _keep = api.request_from_workload(wl.request, args.precision)
    q_dev.rx = C.cast(C.c_void_p(rx_dev.data_ptr()), C.POINTER(C.c_double))
    q_dev.rx_on_device = 1
    req_dev = (q_dev, _keep)
    req_host = api.request_from_workload(wl.request, args.precision)

    for _ in range(args.warmup):
        api.solve(scene, req_dev, with_paths=False)
    # stage counts, and the FP32 field modes' error on this workload (untimed)
    q_chk = api.request_from_workload(wl.request, args.precision, stage_counts=True)
    captured = api.solve(scene, q_chk, with_paths=False).counts["captured"]
    fp32_error = {}
    for mode in ("fp32", "fp32_phase"):
        r_chk = api.solve(scene, api.request_from_workload(wl.request, mode, field_check=True),
                          with_paths=False)
        fp32_error[mode] = api.field_error_stats(r_chk.field, r_chk.field_fp64)
    # ---- device-resident timing
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    dev_ms, seg, stage = [], [], {"trace_ms": 0.0, "capture_ms": 0.0, "correct_ms": 0.0,
                                 "field_ms": 0.0, "capture_kernel_ms": 0.0,
                                 "trace_kernel_ms": 0.0, "trace_kernel_launches": 0.0,
                                 "trace_kernel_first_ms": 0.0}
    counts = None
    with Clocks(local) as ck:
        # NVTX range "timed": lets a profiler select exactly these solves
        torch.cuda.nvtx.range_push("timed")
        for _ in range(args.steps):
            r = api.solve(scene, req_dev, with_paths=False)
            dev_ms.append(r.timing["device_ms"])
            seg.append(r.counts["segments"])
            for k in stage:
                stage[k] += r.timing[k]
            counts = r.counts
        torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    clocks = ck.summary()
    t_dev = sum(dev_ms) / 1e3
    # ---- end to end through the C ABI with host buffers
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_seg = 0
    d2h = 0
    for _ in range(args.steps):
        r = api.solve(scene, req_host, with_paths="arrays")
        e2e_seg += r.counts["segments"]
        d2h = 6 * 8 * len(wl.request.rx) + r.counts["paths"] * 64 + r.counts["rays"] * (12 + 48)
    torch.cuda.synchronize()
    t_e2e = time.perf_counter() - t0
    h2d = 8 * 3 * len(wl.request.rx) + 160
    # ---- aggregate over ranks (replicas)
    tot_seg, max_t, tot_e2e, max_e2e = replica_totals(dist, world, float(sum(seg)), t_dev,
                                                      float(e2e_seg), t_e2e)
    if rank == 0:
        peak, peak_kind = peaks()
        steps = args.steps
        n_nodes = counts["segments"]
        cap_ms = stage["capture_kernel_ms"] / steps  # the capture kernel alone
        tr_ms = stage["trace_kernel_ms"] / steps      # k_trace alone, all its launches
        if cap_ms >= tr_ms:  # the kernel with the larger total time
            kern, ms, launch = "k_capture_fast", cap_ms, "the one launch per solve"
            alg = n_nodes * NODE_BYTES + captured * EVENT_BYTES
            traffic = None
        else:
            # k_trace's first launch: the launch rays, one segment each
            kern, ms = "k_trace", stage["trace_kernel_first_ms"] / steps
            launch = f"first launch ({counts['launches']} launch rays)"
            alg = counts["launches"] * SEGMENT_BYTES
            traffic = TRACE_FIRST_LAUNCH_DRAM_BYTES if wl.name == "urban_L9_R6T1" else None
        achieved = alg / (ms / 1e3) / 1e9
        launches_per_step = counts["gpu_kernels"]  # counted by the library
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
                       "launch_shapes": scene.tuning(req_host),
                       "l2": "working set (node pool) larger than L2 each step"},
            "counts": dict(counts, captured=captured),
            "scene_create_ms": scene_ms,
            "field_error": ("FP64 field: the reference's arithmetic; parity tests hold it "
                            "within 1e-9 of the oracle" if args.precision == "fp64" else
                            fp32_error[args.precision]),
            "stages_ms": {k: v / steps for k, v in stage.items()},
            "e2e": {"value": tot_e2e / max_e2e, "unit": "segments/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": 1e3 * max_e2e / steps,
                    "call": "api.solve(scene, request with host receivers, "
                            "with_paths='arrays'): fields and every path array read back"},
            "roofline": {"bound": "hbm", "kernel": kern, "launch": launch,
                         "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "algorithmic_bytes_per_launch": alg,
                         "traffic_frac": (traffic / (ms / 1e3) / 1e9 / peak) if traffic else None,
                         "launch_ms": ms,
                         "kernel_ms_per_step": {"k_trace": tr_ms, "k_capture_fast": cap_ms}},
            "gpu_launches": launches_per_step * steps,
            "clocks": clocks,
        }
        if not args.no_batched and args.level == 9:
            line["batched"] = run_batched(args.precision, best_rate=tot_seg / max_t)
        if not args.no_serving and args.level == 9:
            line["serving"] = run_serving(args.precision)
        if not args.no_precision and args.level == 9:
            line["precision"] = run_precision()
            line["precision"]["urban_L9"] = fp32_error
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
