"""GPU path against the reference: identical path sets (receiver, launch,
facet ids, coplanar ids, interaction kinds, ray counts) and received fields
within 1e-4 relative magnitude / 1e-3 rad phase, through the C ABI."""
import os
import warnings

import numpy as np
import pytest

import oracle as orc
from helpers import field_close, golden_field, golden_paths, max_rel_err, path_keys
from sbrsolver_gb300 import api, scenes
from test_oracle_golden import CASES, GOLD, _case

pytestmark = pytest.mark.gpu


def _gpu(wl, precision="fp64", scene=None):
    sc = scene or api.DeviceScene.from_scene(wl.scene)
    return api.solve(sc, api.request_from_workload(wl.request, precision, stage_counts=True)), sc


def _check_against(res, ref_paths, ref_field, counts=None, tight=True):
    assert path_keys(res.paths) == path_keys(ref_paths)
    for p, q in zip(res.paths, ref_paths):
        # corrected points come from FP64 arithmetic in the reference order
        np.testing.assert_array_equal(p["points"], q["points"])
    bad = field_close(res.field, ref_field)
    assert not bad, bad[:5]
    if tight:
        assert max_rel_err(res.field, ref_field) < 1e-9
    if counts:
        for k, v in counts.items():
            assert res.counts[k] == v, (k, res.counts[k], v)


@pytest.mark.parametrize("name", CASES)
def test_golden_cases(built, name):
    g = np.load(os.path.join(GOLD, name + ".npz"))
    wl = _case(name)
    res, _ = _gpu(wl)
    _check_against(res, golden_paths(g), golden_field(g),
                   {"segments": int(g["segments"]), "captured": int(g["captured"]),
                    "corrected": int(g["corrected"])})


@pytest.mark.parametrize("name", CASES)
def test_fp32_field_mode_within_tolerance(built, name):
    g = np.load(os.path.join(GOLD, name + ".npz"))
    res, _ = _gpu(_case(name), precision="fp32")
    assert path_keys(res.paths) == path_keys(golden_paths(g))
    bad = field_close(res.field, golden_field(g))
    assert not bad, bad[:5]


def test_scene_tables_match_oracle(built):
    for wl in (scenes.small_scene(), scenes.urban_scene(level=3)):
        sc = api.DeviceScene.from_scene(wl.scene)
        o = orc.OracleScene.from_scene(wl.scene)
        np.testing.assert_array_equal(sc.mesh_order(), o.mesh_order())
        np.testing.assert_array_equal(sc.coplanar_ids(), o.coplanar_ids())


def _oracle(wl):
    return orc.solve(orc.OracleScene.from_scene(wl.scene), wl.request, wl.scene.materials)


@pytest.mark.parametrize("level,R,T,antenna", [(6, 6, 1, 0), (5, 3, 2, 2), (6, 8, 0, 1),
                                               (4, 0, 3, 0), (0, 2, 1, 1)])
def test_urban_variants(built, level, R, T, antenna):
    wl = scenes.urban_scene(level=level, rx_pitch=125.0, max_reflection=R, max_transmission=T)
    wl.request.antenna = antenna
    ref = _oracle(wl)
    res, _ = _gpu(wl)
    _check_against(res, ref["paths"], ref["field"],
                   {k: ref["counts"][k] for k in ("segments", "captured", "corrected")})


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_slab_walls_against_oracle(built, precision):
    """Finite-thickness walls (slab coefficients with width > 0): same path
    set as the oracle, fields within tolerance; FP64 fields tight."""
    wl = scenes.urban_scene(level=6, rx_pitch=25.0, max_reflection=4, max_transmission=2)
    wl = scenes.slab_walls(wl, (0.3, 0.15, 0.006))
    ref = _oracle(wl)
    assert any(k == 2 for p in ref["paths"] for k in p["kind"])
    res, _ = _gpu(wl, precision=precision)
    _check_against(res, ref["paths"], ref["field"],
                   {k: ref["counts"][k] for k in ("segments", "captured", "corrected")},
                   tight=precision == "fp64")


def test_identity_mesh_order(built):
    """A caller whose triangle vector stays in file order: image correction
    and frames then use the hit triangle itself."""
    wl = scenes.small_scene()
    sc = api.DeviceScene.from_scene(wl.scene)
    sc.set_mesh_order(np.arange(wl.scene.n_tri, dtype=np.int32))
    res, _ = _gpu(wl, scene=sc)
    assert res.counts["corrected"] > 253  # more reflections survive correction
    ref_sc = orc.OracleScene.from_scene(wl.scene)
    assert res.counts["segments"] == 96720


def test_batch_equals_single(built):
    wl = scenes.small_scene()
    a = scenes.small_scene()
    a.request.tx = (30.0, -60.0, 12.0)
    a.request.tessellation = 5
    a.request.antenna = 0
    sc = api.DeviceScene.from_scene(wl.scene)
    r1 = api.solve(sc, api.request_from_workload(wl.request))
    r2 = api.solve(sc, api.request_from_workload(a.request))
    rb = api.solve(sc, [api.request_from_workload(wl.request), api.request_from_workload(a.request)])
    np.testing.assert_array_equal(rb.field, np.concatenate([r1.field, r2.field]))
    assert rb.counts["segments"] == r1.counts["segments"] + r2.counts["segments"]
    pb = [p for p in rb.paths if p["request"] == 0]
    assert path_keys(pb) == path_keys(r1.paths)
    pb = [p for p in rb.paths if p["request"] == 1]
    assert path_keys(pb) == path_keys(r2.paths)


def test_edge_cases(built):
    wl = scenes.small_scene()
    sc = api.DeviceScene.from_scene(wl.scene)
    # no receivers
    wl0 = scenes.small_scene()
    wl0.request.rx = np.zeros((0, 3))
    r = api.solve(sc, api.request_from_workload(wl0.request))
    assert r.counts["paths"] == 0 and r.counts["segments"] == 96720
    # receiver exactly at the transmitter, receivers on a facet, no bounces
    wl1 = scenes.small_scene()
    wl1.request.rx = np.array([wl1.request.tx, (5.0, 5.0, 0.0), (50.0, -10.0, 1.5)])
    wl1.request.max_reflection = 0
    ref = _oracle(wl1)
    res = api.solve(sc, api.request_from_workload(wl1.request))
    assert path_keys(res.paths) == path_keys(ref["paths"])
    # the receiver at the transmitter has a zero-length direct path: its field
    # is not finite on either side, and must be non-finite in the same places
    assert not np.all(np.isfinite(ref["field"][0]))
    with warnings.catch_warnings():
        warnings.simplefilter("error", RuntimeWarning)
        assert not field_close(res.field, ref["field"])
    # bad requests
    bad = scenes.small_scene()
    bad.request.tessellation = 13
    with pytest.raises(Exception):
        api.solve(sc, api.request_from_workload(bad.request))


@pytest.mark.parametrize("which", ["urban", "large"])
def test_fast_capture_equals_plain_capture_at_scale(built, which):
    """At sizes the oracle cannot reach, the capture stage's fast path (image-
    correction prefilter, correction-cone cell culling, deferred FP64 pass)
    must give exactly what its plain path gives (reception test first, every
    decision inline; used when stage counts are requested)."""
    wl = (scenes.urban_scene(level=8) if which == "urban"
          else scenes.large_scene(level=8, n_rx=20000))
    sc = api.DeviceScene.from_scene(wl.scene)
    fast = api.solve(sc, api.request_from_workload(wl.request, "fp64"), with_paths="arrays")
    plain = api.solve(sc, api.request_from_workload(wl.request, "fp64", stage_counts=True),
                      with_paths="arrays")
    assert fast.counts["corrected"] == plain.counts["corrected"] > 0
    assert fast.counts["paths"] == plain.counts["paths"] > 0
    assert api.same_path_set(fast.paths, plain.paths)
    np.testing.assert_array_equal(fast.field, plain.field)
    sc.close()


def _bary_edge_distance(tri, p):
    """min(u, v, 1-u-v) of point p on triangle tri (3x3), the barycentric
    distance from the triangle's nearest edge (as sbr_path.near_edge uses)."""
    v1 = tri[0].astype(np.float64)
    e1, e2 = tri[1].astype(np.float64) - v1, tri[2].astype(np.float64) - v1
    w = np.asarray(p, np.float64) - v1
    d00, d01, d11 = e1 @ e1, e1 @ e2, e2 @ e2
    d20, d21 = w @ e1, w @ e2
    den = d00 * d11 - d01 * d01
    u = (d11 * d20 - d01 * d21) / den
    v = (d00 * d21 - d01 * d20) / den
    return min(u, v, 1.0 - u - v)


def test_near_edge_paths_listed(built):
    """Paths with an interaction point within 1e-6 (barycentric) of a
    triangle edge are listed separately (sbr_path.near_edge).  The ground's
    two triangles share the diagonal y = x; the transmitter stands over it
    and each receiver is placed so that its ground reflection lands 0, 1e-4,
    1e-3 and 1 m off the diagonal (barycentric 0, 5e-7, 5e-6, 5e-3).  The
    path set equals the oracle's, and each flag equals the one computed on
    the CPU from the oracle's corrected points."""
    mb = scenes._MeshBuilder()
    scenes._ground(mb, 100.0, 0)
    scene = mb.build("diagonal", [(2.4e9, 0.0, 0.0, 15.0, 0.0, 0.005)])
    ht, hr = 10.0, 1.5
    frac = ht / (ht + hr)  # where the specular point splits the Tx -> Rx projection
    offsets = [0.0, 1e-4, 1e-3, 1.0]
    rx = np.array([(30.0 + 7 * k, 30.0 + 7 * k + off / frac, hr) for k, off in enumerate(offsets)])
    req = scenes.Request(tx=(-20.0, -20.0, ht), rx=rx, max_reflection=1, max_transmission=0,
                         frequency=2.4e9, tessellation=6, antenna=2)
    wl = scenes.Workload("diagonal", scene, req)
    ref = _oracle(wl)
    sc = api.DeviceScene.from_scene(scene)
    res = api.solve(sc, api.request_from_workload(req))
    order = sc.mesh_order()
    sc.close()
    assert path_keys(res.paths) == path_keys(ref["paths"])
    expect, seen = [], {}
    for p in ref["paths"]:
        flag = 0
        for r in range(p["n_rays"] - 1):
            d = _bary_edge_distance(scene.tri[order[p["tri"][r]]], p["points"][r][3:6])
            flag |= int(d < 1e-6)
            seen[p["receiver"]] = d
        expect.append(flag)
    got = [int(p["near_edge"]) for p in res.paths]
    assert got == expect
    # every receiver has its ground reflection, at the planned distances
    assert sorted(seen) == [0, 1, 2, 3]
    assert seen[0] < 1e-12 and 4e-7 < seen[1] < 6e-7 and 4e-6 < seen[2] < 6e-6 and seen[3] > 1e-3
    assert got.count(1) == 2 and res.counts["near_edge_paths"] == 2


def test_launch_shapes_do_not_change_results(built):
    """Launch shapes (sbr_tuning) change only speed: extreme shapes (65,536-ray
    chunks, so the level-7 request's launch rays span three launch pairs; one
    FP64 resolution block per SM; refills at 4 idle lanes every 8 steps) give
    bit-identical paths and fields, and the autotuner's choice too."""
    wl = scenes.urban_scene(level=6, rx_pitch=50.0, max_reflection=4, max_transmission=1)
    b = scenes.urban_scene(level=7, rx_pitch=100.0, max_reflection=3, max_transmission=0)
    b.request.tx = (120.0, -80.0, 15.0)
    sc = api.DeviceScene.from_scene(wl.scene)
    qs = [api.request_from_workload(wl.request), api.request_from_workload(b.request)]
    ref = api.solve(sc, qs, with_paths="arrays")
    assert sc.tuning(qs) == sc.tuning()  # no mix tuned yet: the scene default
    sc.set_tuning(find_steps=8, find_refill=4, find_blocks_per_sm=2, trace_blocks_per_sm=1,
                  capture_blocks_per_sm=1, trace_chunk_log2=16)
    t = sc.tuning(qs)
    assert t["trace_chunk_log2"] == 16 and t["trace_blocks_per_sm"] == 1
    odd = api.solve(sc, qs, with_paths="arrays")
    assert api.same_path_set(odd.paths, ref.paths)
    np.testing.assert_array_equal(odd.field, ref.field)
    assert odd.counts["gpu_kernels"] > ref.counts["gpu_kernels"]  # more launch pairs
    # both FP64 resolution kernels (a ray per lane; 64 rays per warp in shared
    # memory), with the default shapes and the extreme ones
    for shapes in ({}, dict(find_steps=8, find_refill=4, trace_chunk_log2=16)):
        for kernel in (1, 2):
            sc.set_tuning(trace_kernel=kernel, **shapes)
            assert sc.tuning(qs)["trace_kernel"] == kernel
            r = api.solve(sc, qs, with_paths="arrays")
            assert api.same_path_set(r.paths, ref.paths), (kernel, shapes)
            np.testing.assert_array_equal(r.field, ref.field)
            assert r.counts["fp64_triangle_tests"] == ref.counts["fp64_triangle_tests"]
    sc.set_tuning()  # back to the defaults
    chosen = sc.autotune(qs, rounds=1)
    assert chosen["device_ms"] > 0
    assert {k: v for k, v in chosen.items() if k != "device_ms"} == sc.tuning(qs)
    tuned = api.solve(sc, qs, with_paths="arrays")
    assert api.same_path_set(tuned.paths, ref.paths)
    np.testing.assert_array_equal(tuned.field, ref.field)
    with pytest.raises(Exception):
        sc.set_tuning(find_refill=33)
    with pytest.raises(Exception):
        sc.set_tuning(trace_kernel=3)
    sc.close()
