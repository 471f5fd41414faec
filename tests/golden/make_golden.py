"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run where the reference checkout exists:
    SBR_REFERENCE_DIR=<checkout> python tests/golden/make_golden.py [--variants | --bvh | --ico]
It compiles the reference's own sources (oracle/build_ref.sh -> oracle/_ref/
ref_harness), runs each case through RTSolver::ExecuteRayTracing, and stores
the surviving paths and fields per receiver as .npz.  For the reference's
own main() scene it first checks the run against the outputs the reference
ships (data/output/ElectricField.csv at printed precision, and the
(launch, receiver) pairs of data/output/RayPath.vtk) and records that check
in the fixture.  The scenes are regenerated from their seeds by
sbrsolver_gb300.scenes, so fixtures hold outputs plus a hash of the inputs.
"""
from __future__ import annotations

import hashlib
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from sbrsolver_gb300 import scenes  # noqa: E402
import build as oracle_build  # noqa: E402  (oracle/build.py)

OUT = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("SBR_REFERENCE_DIR", "")  # the reference checkout (required)


def parse_report(path: str) -> dict:
    counts, fields, paths = {}, {}, []
    cur = None
    for line in open(path):
        t = line.split()
        if t[0] in ("segments", "launches", "receivers", "triangles", "loop_mismatch"):
            counts[t[0]] = int(t[1])
        elif t[0] == "path":
            cur = {"receiver": int(t[1]), "launch": int(t[2]), "n_rays": int(t[3]),
                   "field": [float(x) for x in t[4:10]], "tri": [], "cop": [], "refl": [],
                   "trans": [], "points": []}
            paths.append(cur)
        elif t[0] == "ray":
            cur["tri"].append(int(t[1]))
            cur["cop"].append(int(t[2]))
            cur["refl"].append(int(t[3]))
            cur["trans"].append(int(t[4]))
            cur["points"].append([float(x) for x in t[5:11]])
        elif t[0] == "field":
            fields[int(t[1])] = [float(x) for x in t[2:8]]
    n_rx = counts["receivers"]
    field = np.array([fields[k] for k in range(n_rx)], np.float64).reshape(n_rx, 6)
    return {"counts": counts, "field": field, "paths": paths}


def to_npz(rep: dict, stages: dict, inputs_sha: str, extra: dict, path: str) -> None:
    P = rep["paths"]
    off = np.cumsum([0] + [p["n_rays"] for p in P]).astype(np.int64)
    cat = lambda k: np.array([v for p in P for v in p[k]], np.int32)  # noqa: E731
    kind = np.array([0 if (r < 0 and t < 0) else (1 if r >= 0 else 2)
                     for p in P for r, t in zip(p["refl"], p["trans"])], np.int32)
    np.savez_compressed(
        path,
        segments=rep["counts"]["segments"], launches=rep["counts"]["launches"],
        captured=stages.get("captured", -1), corrected=stages.get("corrected", -1),
        field=rep["field"],
        path_receiver=np.array([p["receiver"] for p in P], np.int32),
        path_launch=np.array([p["launch"] for p in P], np.int64),
        path_field=np.array([p["field"] for p in P], np.float64).reshape(-1, 6),
        path_offset=off, tri=cat("tri"), cop=cat("cop"), kind=kind,
        points=np.array([q for p in P for q in p["points"]], np.float64).reshape(-1, 6),
        inputs_sha256=inputs_sha, **extra)


def run_case(wl, name: str, extra: dict | None = None) -> dict:
    with tempfile.TemporaryDirectory() as d:
        case = scenes.write_oracle_case(wl, d)
        subprocess.run([oracle_build.REF_HARNESS, "case", case], check=True)
        rep = parse_report(os.path.join(d, "out.txt"))
        st = os.path.join(d, "stages.txt")
        subprocess.run([oracle_build.REF_HARNESS, "stages", case, st], check=True)
        stages = {l.split()[0]: int(l.split()[1]) for l in open(st)}
        h = hashlib.sha256()
        for f in ("scene.stl", "trimat.txt", "rx.txt"):
            h.update(open(os.path.join(d, f), "rb").read())
        sha = h.hexdigest()
    assert rep["counts"]["loop_mismatch"] == 0
    assert stages["segments"] == rep["counts"]["segments"]
    to_npz(rep, stages, sha, extra or {}, os.path.join(OUT, name + ".npz"))
    print(f"{name}: {rep['counts']['segments']} segments, {stages['captured']} captured, "
          f"{stages['corrected']} corrected, {len(rep['paths'])} paths")
    return rep


def pin_reference_main(rep: dict) -> dict:
    """Checks the main() run against the reference's shipped outputs."""
    num = r"[+-]?(?:\d+\.?\d*|\.\d+)(?:e[+-]?\d+)?"
    gold = []
    for ln in open(os.path.join(REF, "SBRSolver_rev2/data/output/ElectricField.csv")).read().splitlines()[1:]:
        vals = []
        for c in ln.split(",")[3:]:
            m = re.fullmatch(f"({num})({num})i", c)
            vals += [float(m.group(1)), float(m.group(2))]
        gold.append(vals)
    gold = np.array(gold)
    ours = np.array([[float("%.6g" % x) for x in row] for row in rep["field"]])
    field_ok = bool(np.array_equal(gold, ours))
    L = open(os.path.join(REF, "SBRSolver_rev2/data/output/RayPath.vtk")).read().splitlines()
    n = int([l for l in L if l.startswith("CELL_DATA")][0].split()[1])
    i = L.index(f"LaunchID 1 {n} int")
    lid = [int(x) for x in L[i + 1:i + 1 + n]]
    i = L.index(f"ReceiverID 1 {n} int")
    rid = [int(x) for x in L[i + 1:i + 1 + n]]
    pairs_ok = sorted(zip(lid, rid)) == sorted((p["launch"], p["receiver"]) for p in rep["paths"])
    print("reference main(): ElectricField.csv match at printed precision:", field_ok,
          "| RayPath.vtk (launch, receiver) pairs match:", pairs_ok, f"({n} paths)")
    assert field_ok and pairs_ok
    return {"shipped_field_csv_match": field_ok, "shipped_raypath_pairs_match": pairs_ok,
            "shipped_field_csv": gold}


def shipped_output_hashes() -> None:
    """sha256 and size of the output files the reference ships for its main()
    run (field CSV, ray-path / receiver VTK) and of its level-3 launch-ray VTK
    from (0, 0, 5); the writers in the library must reproduce them byte for
    byte from the reference_main fixture."""
    import json
    out = {}
    for f in ("ElectricField.csv", "RayPath.vtk", "RxLocations.vtk", "Icosahedron.vtk"):
        b = open(os.path.join(REF, "SBRSolver_rev2/data/output", f), "rb").read()
        out[f] = {"sha256": hashlib.sha256(b).hexdigest(), "bytes": len(b)}
    with open(os.path.join(OUT, "shipped_outputs.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
    print("shipped output hashes written")


def coefficient_sweep() -> None:
    """RefCoeffTest vs the shipped coeff_test.csv (1000 angles, eps2 = 1-10j):
    magnitudes are compared exactly at printed precision; the shipped phases
    sit exactly pi away from the current sign convention (FieldCompute.cpp:249,
    277), so only phase modulo pi is pinned."""
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "coeff.csv")
        subprocess.run([oracle_build.REF_HARNESS, "coeff", "1000", "1.8e9", "1", "0", "1", "-10",
                        out], check=True)
        ours = np.loadtxt(out, delimiter=",", skiprows=1)
    shipped = np.loadtxt(os.path.join(REF, "SBRSolver_rev2/data/output/coeff_test.csv"),
                         delimiter=",", skiprows=1)
    assert np.array_equal(ours[:, [0, 1, 3]], shipped[:, [0, 1, 3]])
    dphi = np.angle(np.exp(1j * (ours[:, [2, 4]] - shipped[:, [2, 4]]))) % np.pi
    assert np.all(np.minimum(dphi, np.pi - dphi) < 2e-5)
    np.savez_compressed(os.path.join(OUT, "fresnel_sweep.npz"), reference=ours, shipped=shipped)
    print("coeff_test.csv: magnitudes identical, phases equal modulo pi")


def parse_scene_dump(path: str) -> dict:
    """The harness's `scene` dump (the reference's mesh after
    StlToGeometry + BVH::ConstructBVH) as arrays in a numbering-free form:
    mesh_order (triangle id at each position of the sorted triangle vector),
    coplanar ids and frame rows by triangle id, and the tree in depth-first
    order from the root (children[0] before children[1], BVH.h:276-328):
    node boxes, leaf sizes (-1 for an inner node) and the leaves' triangle
    ids in visit order."""
    with open(path) as fh:
        n = int(fh.readline().split()[1])
        mesh_order = np.zeros(n, np.int32)
        cop = np.zeros(n, np.int32)
        frames = np.zeros((n, 9), np.float64)
        for k in range(n):
            t = fh.readline().split()
            i = int(t[1])
            mesh_order[k] = i
            cop[i] = int(t[2])
            frames[i] = [float(x) for x in t[3:12]]
        m = int(fh.readline().split()[1])
        children = np.zeros((m, 2), np.int64)
        boxes = np.zeros((m, 6), np.float64)
        objs = []
        for k in range(m):
            t = fh.readline().split()
            children[k] = (int(t[1]), int(t[2]))
            # the boxes hold float values (bounds of float vertices), printed
            # with 9 significant digits: read back as float, then widened
            boxes[k] = np.array(t[3:9], np.float32)
            objs.append([int(x) for x in t[10:10 + int(t[9])]])
    pre_boxes, leaf_n, leaf_ids, stack = [], [], [], [0]
    while stack:
        k = stack.pop()
        pre_boxes.append(boxes[k])
        if children[k][0] < 0:
            leaf_n.append(len(objs[k]))
            leaf_ids += objs[k]
        else:
            leaf_n.append(-1)
            stack += [int(children[k][1]), int(children[k][0])]
    return {"mesh_order": mesh_order, "coplanar": cop, "frames": frames,
            "boxes": np.array(pre_boxes, np.float64).reshape(-1, 6),
            "leaf_n": np.array(leaf_n, np.int32), "leaf_ids": np.array(leaf_ids, np.int32)}


BVH_ARRAYS = ("mesh_order", "coplanar", "frames", "boxes", "leaf_n", "leaf_ids")


def reference_bvh_fixtures() -> None:
    """The reference's own scene preparation (StlToGeometry, ConstructBVH)
    on the seeded small, urban and terrain scenes and on three meshes with
    many equal sort keys (stored in the fixture, so the test needs no
    generator): a lattice of colliding box centres, centres ordered to drive
    std::sort into its heap sort, and a flat grid.  The terrain (580,484
    triangles) keeps sha256 digests of its arrays."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from test_gpu_scene_prep import _tie_heavy_scene  # noqa: E402
    meshes = {"small": scenes.small_scene().scene, "urban": scenes.urban_scene(level=2).scene,
              "large": scenes.large_scene().scene}
    tri, nrm = _tie_heavy_scene(1, 3000)
    meshes["ties"] = scenes.Scene("ties", tri, nrm, np.zeros(len(tri), np.int32), [])
    keys = np.loadtxt(os.path.join(OUT, "introsort_killer_3000.txt"), dtype=np.int64)
    n = len(keys)
    tri = np.zeros((n, 3, 3), np.float32)
    tri[:, :, 0] = (keys.astype(np.float32) * np.float32(0.25))[:, None]
    tri[:, :, 1] = (np.arange(n, dtype=np.float32) * np.float32(0.5))[:, None]
    tri[:, 1, 1] += np.float32(1.0)
    tri[:, 2, 2] = np.float32(1.0)
    nrm = np.tile(np.array([[1.0, 0.0, 0.0]], np.float32), (n, 1))
    meshes["heap_sort"] = scenes.Scene("heap_sort", tri, nrm, np.zeros(n, np.int32), [])
    k = 40
    xs, ys = np.meshgrid(np.arange(k, dtype=np.float32), np.arange(k, dtype=np.float32))
    x0, y0 = xs.ravel(), ys.ravel()
    z = np.zeros_like(x0)
    a = np.stack([np.stack([x0, y0, z], 1), np.stack([x0 + 1, y0, z], 1),
                  np.stack([x0 + 1, y0 + 1, z], 1)], 1)
    b = np.stack([np.stack([x0, y0, z], 1), np.stack([x0 + 1, y0 + 1, z], 1),
                  np.stack([x0, y0 + 1, z], 1)], 1)
    tri = np.concatenate([a, b]).astype(np.float32)
    nrm = np.tile(np.array([[0.0, 0.0, 1.0]], np.float32), (len(tri), 1))
    meshes["flat"] = scenes.Scene("flat", tri, nrm, np.zeros(len(tri), np.int32), [])
    for name, sc in meshes.items():
        with tempfile.TemporaryDirectory() as d:
            stl = os.path.join(d, "scene.stl")
            scenes.write_stl(sc, stl)
            out = os.path.join(d, "dump.txt")
            subprocess.run([oracle_build.REF_HARNESS, "scene", stl, out], check=True)
            rep = parse_scene_dump(out)
        h = hashlib.sha256(np.ascontiguousarray(sc.tri, "<f4").tobytes() +
                           np.ascontiguousarray(sc.normal, "<f4").tobytes()).hexdigest()
        extra = {"inputs_sha256": h, "n_nodes": len(rep["leaf_n"])}
        if name == "large":
            for key in BVH_ARRAYS:
                extra[key + "_sha256"] = hashlib.sha256(np.ascontiguousarray(rep[key]).tobytes()).hexdigest()
        else:
            extra.update(rep)
            if name in ("ties", "heap_sort", "flat"):
                extra.update(tri=sc.tri, normal=sc.normal)
        np.savez_compressed(os.path.join(OUT, f"refbvh_{name}.npz"), **extra)
        print(f"refbvh_{name}: {sc.n_tri} triangles, {extra['n_nodes']} nodes, "
              f"{int((rep['leaf_n'] >= 0).sum())} leaves")


def icosphere_digests() -> None:
    """sha256 of the reference's launch directions (GenerateRaysOnIcosahedron,
    Icosahedron.cpp:80-109; little-endian float64, x y z per ray) at levels
    6-10, the levels of the benchmark workloads, whose arrays are too large to
    commit."""
    import json
    out = {}
    for lvl in range(6, 11):
        with tempfile.TemporaryDirectory() as d:
            f = os.path.join(d, "ico.bin")
            subprocess.run([oracle_build.REF_HARNESS, "ico", str(lvl), f], check=True)
            b = open(f, "rb").read()
        out[str(lvl)] = {"rays": len(b) // 24, "sha256": hashlib.sha256(b).hexdigest()}
    with open(os.path.join(OUT, "icosphere_digests.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
    print("icosahedron digests of levels 6-10 written")


VARIANTS = ("small_L5_R4T1_halfwave_rotated", "urban_L5_R3T1_rx1600_halfwave_rotated",
            "urban_L5_R3T1_rx1600_isotropic_nofresnel")


def request_variants() -> None:
    """Request options main() never sets (patterns, frame, power, Fresnel
    switch; sbrsolver_gb300.scenes.request_variant), through the reference."""
    for name in VARIANTS:
        run_case(scenes.request_variant(name), name)


def main() -> None:
    if oracle_build.build_reference(REF) is None:
        raise SystemExit("reference checkout not found: set SBR_REFERENCE_DIR to it")
    main_wl = scenes.reference_main_scene()
    rep = run_case(main_wl, "reference_main")
    pins = pin_reference_main(rep)
    d = dict(np.load(os.path.join(OUT, "reference_main.npz")))
    d.update(pins)
    np.savez_compressed(os.path.join(OUT, "reference_main.npz"), **d)
    shipped_output_hashes()
    coefficient_sweep()
    run_case(scenes.small_scene(), "small_L6_R3")
    wl = scenes.small_scene()
    wl.request.antenna = 1
    wl.request.tessellation = 4
    wl.request.max_transmission = 1
    run_case(wl, "small_L4_R3T1_hertzian")
    run_case(scenes.urban_scene(level=5, rx_pitch=100.0), "urban_L5_R6T1_rx100")
    run_case(scenes.urban_scene(level=4, rx_pitch=50.0, max_reflection=3, max_transmission=2),
             "urban_L4_R3T2_rx400")
    # finite-thickness walls: the reference's own ComputeRefcField /
    # ComputeTransField with a non-zero width (its main() always passes 0)
    run_case(scenes.slab_walls(scenes.urban_scene(level=5, rx_pitch=25.0, max_reflection=3,
                                                  max_transmission=2), (0.5, 0.2, 0.01)),
             "urban_L5_R3T2_rx1600_slab")
    request_variants()
    reference_bvh_fixtures()
    # icosahedron launch directions, bit-exact
    for lvl in (0, 1, 2, 5):
        with tempfile.TemporaryDirectory() as d:
            f = os.path.join(d, "ico.bin")
            subprocess.run([oracle_build.REF_HARNESS, "ico", str(lvl), f], check=True)
            v = np.fromfile(f, np.float64).reshape(-1, 3)
        np.save(os.path.join(OUT, f"icosphere_L{lvl}.npy"), v)
    print("icosahedron levels 0,1,2,5 written")
    icosphere_digests()


if __name__ == "__main__":
    if "--outputs-only" in sys.argv:  # refresh only shipped_outputs.json
        shipped_output_hashes()
    elif "--ico" in sys.argv:  # (re)write only the launch-direction digests
        if oracle_build.build_reference(REF) is None:
            raise SystemExit("reference checkout not found: set SBR_REFERENCE_DIR to it")
        icosphere_digests()
    elif "--bvh" in sys.argv:  # (re)write only the reference-BVH fixtures
        if oracle_build.build_reference(REF) is None:
            raise SystemExit("reference checkout not found: set SBR_REFERENCE_DIR to it")
        reference_bvh_fixtures()
    elif "--variants" in sys.argv:  # (re)write only the request-variant fixtures
        if oracle_build.build_reference(REF) is None:
            raise SystemExit("reference checkout not found: set SBR_REFERENCE_DIR to it")
        request_variants()
    else:
        main()
