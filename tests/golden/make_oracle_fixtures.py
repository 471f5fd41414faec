"""Generates the full-size oracle fixtures in tests/golden/ (TEST INFRASTRUCTURE).

The reference itself cannot run these sizes (it allocates
Paths[launches][receivers], RTSolver.cpp:461-468), so they come from the
FP64 CPU restatement (oracle/sbr_oracle.cpp), which reproduces every
reference-made fixture bit for bit (tests/test_oracle_golden.py).  Each case
is a workload of the benchmark or the precision study at full size:

  urban_L9_R6T1_rx10000  the benchmark solve: urban canyon, level 9
                         (2,621,442 rays), 6 reflections + 1 transmission,
                         all 10,000 receivers
  large_L9_R8_rx5000     the large terrain (580,484 triangles) at level 9,
                         8 reflections, every 10th of its 50,000 receivers
  batch_L6L7L9_rx4096    a subset of the 256-transmitter batch: every
                         level-6 and level-7 request plus the first two
                         level-9 requests (129 requests, 4,096 receivers)

Each fixture stores the surviving paths (receiver, launch, BFS position,
facet ids, coplanar ids, interaction kinds, corrected points), the received
fields, the stage counts and a sha256 of the inputs, so the GPU tests
regenerate the workload from its seed and check that it is the same one.

  python tests/golden/make_oracle_fixtures.py [case ...]   (all cores; about
  an hour on 8 cores for all three)
"""
from __future__ import annotations

import hashlib
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from sbrsolver_gb300 import scenes  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def urban_L9():
    wl = scenes.urban_scene()
    return wl.scene, [wl.request]


def large_L9():
    wl = scenes.large_scene(level=9)
    wl.request.rx = np.ascontiguousarray(wl.request.rx[::10])
    return wl.scene, [wl.request]


def batch_subset():
    wl, reqs = scenes.batched_workload()
    nine = [i for i, q in enumerate(reqs) if q.tessellation == 9][:2]
    keep = [i for i, q in enumerate(reqs) if q.tessellation in (6, 7) or i in nine]
    return wl.scene, [reqs[i] for i in keep]


CASES = {"urban_L9_R6T1_rx10000": urban_L9, "large_L9_R8_rx5000": large_L9,
         "batch_L6L7L9_rx4096": batch_subset}


def inputs_sha256(scene, requests) -> str:
    """Hash of everything a solve reads: triangles, normals, materials and,
    per request, every parameter and receiver coordinate."""
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(scene.tri, np.float32).tobytes())
    h.update(np.ascontiguousarray(scene.normal, np.float32).tobytes())
    h.update(np.ascontiguousarray(scene.material_id, np.int32).tobytes())
    h.update(repr([tuple(float(x) for x in m) for m in scene.materials]).encode())
    for q in requests:
        h.update(repr((tuple(float(x) for x in q.tx), q.max_reflection, q.max_transmission,
                       float(q.frequency), q.tessellation,
                       tuple(float(x) for x in q.tx_coord_sys), float(q.pt),
                       bool(q.use_fresnel), q.antenna)).encode())
        h.update(np.ascontiguousarray(q.rx, np.float64).tobytes())
    return h.hexdigest()


def solve_all(scene, requests):
    import oracle as orc
    osc = orc.OracleScene.from_scene(scene)
    out = []
    for i, q in enumerate(requests):
        t0 = time.time()
        r = orc.solve(osc, q, scene.materials)
        out.append(r)
        print(f"  request {i}: level {q.tessellation}, {r['counts']['segments']} segments, "
              f"{r['counts']['paths']} paths, {time.time() - t0:.1f} s", flush=True)
    return out


def to_npz(path: str, results, sha: str) -> None:
    P, req, field, counts = [], [], [], []
    for k, r in enumerate(results):
        P += r["paths"]
        req += [k] * len(r["paths"])
        field.append(np.stack([r["field"].real, r["field"].imag], -1).reshape(-1, 6))
        c = r["counts"]
        counts.append([c["segments"], c["captured"], c["corrected"], c["paths"], c["rays"]])
    off = np.cumsum([0] + [p["n_rays"] for p in P]).astype(np.int64)
    cat = lambda k: np.array([v for p in P for v in p[k]], np.int32)  # noqa: E731
    np.savez_compressed(
        path,
        counts=np.array(counts, np.int64),  # per request: segments, captured, corrected, paths, rays
        rx_per_request=np.array([len(f) for f in field], np.int64),
        field=np.concatenate(field, 0),
        path_request=np.array(req, np.int32),
        path_receiver=np.array([p["receiver"] for p in P], np.int32),
        path_launch=np.array([p["launch"] for p in P], np.int64),
        path_field=np.array([p["field"] for p in P], np.float64).reshape(-1, 6),
        path_offset=off, tri=cat("tri"), cop=cat("cop"), kind=cat("kind"),
        points=np.concatenate([p["points"] for p in P], 0) if P else np.zeros((0, 6)),
        inputs_sha256=sha)


def main(names) -> None:
    import build as oracle_build  # oracle/build.py
    oracle_build.build_oracle()
    for name in names:
        scene, reqs = CASES[name]()
        print(f"{name}: {scene.n_tri} triangles, {len(reqs)} request(s)", flush=True)
        t0 = time.time()
        res = solve_all(scene, reqs)
        to_npz(os.path.join(OUT, name + ".npz"), res, inputs_sha256(scene, reqs))
        seg = sum(r["counts"]["segments"] for r in res)
        print(f"{name}: {seg} segments, {sum(r['counts']['paths'] for r in res)} paths, "
              f"{time.time() - t0:.0f} s", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:] or list(CASES))
