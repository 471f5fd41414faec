"""Scene preparation on the GPU (sbr_prep.cuh) against the host build.

By default a scene's coplanar groups (Preprocessor.cpp:116-246), triangle
frames and boxes (Triangle.cpp:37-70), search BVH and reference BVH
(BVH/BVH.h:135-230, with std::sort's order of equal keys restated on the
device) are built on the GPU; SBR_SCENE_HOST_PREP builds them all on the
host.  The two must give identical tables, bit for bit, and the same
solve."""
import os
import time

import numpy as np
import pytest

from sbrsolver_gb300 import api, scenes

pytestmark = pytest.mark.gpu


def _scene(name):
    if name == "small":
        return scenes.small_scene()
    if name == "urban":
        return scenes.urban_scene(level=5, rx_pitch=100.0)
    wl = scenes.large_scene(level=5)
    wl.request.rx = wl.request.rx[::100].copy()
    return wl


@pytest.mark.parametrize("name", ["small", "urban", "large"])
def test_device_tables_equal_host_tables(built, name):
    wl = _scene(name)
    t0 = time.perf_counter()
    host = api.DeviceScene.from_scene(wl.scene, host_prep=True)
    t1 = time.perf_counter()
    dev = api.DeviceScene.from_scene(wl.scene)
    t2 = time.perf_counter()
    inf = dev.info()
    print(f"{name}: {wl.scene.n_tri} triangles, host preparation {1e3 * (t1 - t0):.0f} ms, "
          f"device {1e3 * (t2 - t1):.0f} ms (in the library {inf.prep_total_ms:.1f}: host "
          f"records {inf.prep_host_ms:.1f}, merge/coplanar/frames {inf.prep_device_tables_ms:.1f}, "
          f"search BVH {inf.prep_search_bvh_ms:.1f}, reference BVH "
          f"{inf.prep_reference_bvh_ms:.1f}, upload {inf.prep_upload_ms:.1f})")
    np.testing.assert_array_equal(dev.coplanar_ids(), host.coplanar_ids())
    np.testing.assert_array_equal(dev.mesh_order(), host.mesh_order())
    for a, b in zip(dev.triangle_frames(), host.triangle_frames()):
        np.testing.assert_array_equal(a.view(np.int64), b.view(np.int64))  # bit for bit
    ra_, rb_ = dev.reference_bvh(), host.reference_bvh()
    assert ra_["max_depth"] == rb_["max_depth"] and len(ra_["links"]) == len(rb_["links"])
    np.testing.assert_array_equal(ra_["links"], rb_["links"])
    np.testing.assert_array_equal(ra_["order"], rb_["order"])
    np.testing.assert_array_equal(ra_["boxes"].view(np.int64), rb_["boxes"].view(np.int64))
    sa, sb = dev.search_bvh(), host.search_bvh()
    assert sa["max_depth"] == sb["max_depth"]
    np.testing.assert_array_equal(sa["order"], sb["order"])
    np.testing.assert_array_equal(sa["nodes"], sb["nodes"])
    assert len(sa["nodes"]) > 1
    q = api.request_from_workload(wl.request)
    ra = api.solve(dev, q, with_paths="arrays")
    rb = api.solve(host, q, with_paths="arrays")
    assert api.same_path_set(ra.paths, rb.paths) and ra.counts["paths"] > 0
    np.testing.assert_array_equal(ra.field, rb.field)
    dev.close()
    host.close()


def test_device_prep_edge_cases(built):
    """One triangle, two triangles (the search BVH is a leaf), and a scene
    with a degenerate triangle (refused, as the host refuses it)."""
    wl = scenes.small_scene()
    for n in (1, 2, 9):
        mesh = api.Mesh(wl.scene.tri[:n], wl.scene.normal[:n], wl.scene.material_id[:n])
        mats = [api.MaterialProperties(*m) for m in wl.scene.materials]
        a = api.DeviceScene(mesh, mats)
        b = api.DeviceScene(mesh, mats, host_prep=True)
        np.testing.assert_array_equal(a.search_bvh()["nodes"], b.search_bvh()["nodes"])
        for k in ("links", "order", "boxes"):
            np.testing.assert_array_equal(a.reference_bvh()[k], b.reference_bvh()[k])
        np.testing.assert_array_equal(a.mesh_order(), b.mesh_order())
        np.testing.assert_array_equal(a.coplanar_ids(), b.coplanar_ids())
        a.close()
        b.close()
    # 5,000 copies of one triangle stacked along z: every x and y key equal,
    # so the device sort's partition rounds and warp sorts see nothing but
    # ties, as std::sort does on the host
    base = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]], np.float32)
    k = np.arange(5000, dtype=np.float32)[:, None, None]
    stack_tri = base[None] + np.concatenate([0 * k, 0 * k, 0.01 * k], axis=2)
    stack_nrm = np.tile(np.array([[0.0, 0.0, 1.0]], np.float32), (5000, 1))
    mesh = api.Mesh(stack_tri.astype(np.float32), stack_nrm, np.zeros(5000, np.int32))
    mats = [api.MaterialProperties(*m) for m in wl.scene.materials]
    a = api.DeviceScene(mesh, mats)
    b = api.DeviceScene(mesh, mats, host_prep=True)
    for key in ("links", "order", "boxes"):
        np.testing.assert_array_equal(a.reference_bvh()[key], b.reference_bvh()[key])
    np.testing.assert_array_equal(a.mesh_order(), b.mesh_order())
    a.close()
    b.close()
    tri = wl.scene.tri.copy()
    tri[3, 2] = tri[3, 1]  # two vertices of triangle 3 coincide
    mesh = api.Mesh(tri, wl.scene.normal, wl.scene.material_id)
    for host_prep in (False, True):
        with pytest.raises(Exception) as e:
            api.DeviceScene(mesh, [api.MaterialProperties(*m) for m in wl.scene.materials],
                            host_prep=host_prep)
        assert "degenerate" in str(e.value)


def _tie_heavy_scene(seed: int, n: int):
    """Random triangles whose box centres collide a lot: vertex coordinates on a
    coarse lattice (a few distinct values per axis), some triangles repeated
    at another height, so every sort of the reference BVH build sees long runs
    of equal keys."""
    rng = np.random.default_rng(seed)
    q = rng.integers(2, 12)  # lattice points per axis
    base = rng.integers(0, q, size=(n, 3, 3)).astype(np.float32) * np.float32(2.5)
    base[:, 1, 0] += np.float32(1.0)  # keep the three vertices apart
    base[:, 2, 1] += np.float32(1.0)
    base[:, :, 2] += (np.arange(n, dtype=np.float32) * np.float32(1e-3))[:, None]  # no merges
    e1 = base[:, 1] - base[:, 0]
    e2 = base[:, 2] - base[:, 0]
    nrm = np.cross(e1, e2)
    ln = np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm = np.where(ln > 0, nrm / np.where(ln > 0, ln, 1), np.float32([0, 0, 1]))  # collinear: any
    return base, nrm.astype(np.float32)


@pytest.mark.parametrize("seed,n", [(1, 3000), (2, 20000), (3, 70000)])
def test_reference_bvh_random_ties(built, seed, n):
    tri, nrm = _tie_heavy_scene(seed, n)
    wl = scenes.small_scene()
    mats = [api.MaterialProperties(*m) for m in wl.scene.materials]
    mesh = api.Mesh(tri, nrm, np.zeros(n, np.int32))
    a = api.DeviceScene(mesh, mats)
    b = api.DeviceScene(mesh, mats, host_prep=True)
    ra, rb = a.reference_bvh(), b.reference_bvh()
    assert ra["max_depth"] == rb["max_depth"]
    for key in ("links", "order"):
        np.testing.assert_array_equal(ra[key], rb[key])
    np.testing.assert_array_equal(ra["boxes"].view(np.int64), rb["boxes"].view(np.int64))
    np.testing.assert_array_equal(a.mesh_order(), b.mesh_order())
    a.close()
    b.close()


def test_reference_bvh_flat_scene(built):
    """A ground grid of 3,200 triangles, all at z = 0: every box is flat, every
    surface area 0 and every split cost 0/0, so the host's tree is one leaf;
    the device's must be the same."""
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
    wl = scenes.small_scene()
    mats = [api.MaterialProperties(*m) for m in wl.scene.materials]
    mesh = api.Mesh(tri, nrm, np.zeros(len(tri), np.int32))
    d = api.DeviceScene(mesh, mats)
    h = api.DeviceScene(mesh, mats, host_prep=True)
    rd, rh = d.reference_bvh(), h.reference_bvh()
    assert len(rh["links"]) == 1  # one leaf
    for key in ("links", "order"):
        np.testing.assert_array_equal(rd[key], rh[key])
    np.testing.assert_array_equal(rd["boxes"].view(np.int64), rh["boxes"].view(np.int64))
    np.testing.assert_array_equal(d.mesh_order(), h.mesh_order())
    np.testing.assert_array_equal(d.coplanar_ids(), h.coplanar_ids())
    d.close()
    h.close()


@pytest.mark.parametrize("n", [1000, 3000])
def test_reference_bvh_heap_sort(built, n):
    """Box centres along x that drive std::sort past its depth budget into its
    heap sort at the root (tests/golden/make_introsort_killer.cpp): 1,000 keys
    (a warp's sort in shared memory) and 3,000 (partition rounds, then the heap
    sort of a long segment in global memory).  The device tree must equal the
    host one."""
    keys = np.loadtxt(os.path.join(os.path.dirname(__file__), "golden",
                                   f"introsort_killer_{n}.txt"), dtype=np.int64)
    assert len(keys) == n and len(np.unique(keys)) == n
    x = keys.astype(np.float32) * np.float32(0.25)
    y = np.arange(n, dtype=np.float32) * np.float32(0.5)
    tri = np.zeros((n, 3, 3), np.float32)  # triangles in the planes x = const
    tri[:, :, 0] = x[:, None]
    tri[:, :, 1] = y[:, None]
    tri[:, 1, 1] += np.float32(1.0)
    tri[:, 2, 2] = np.float32(1.0)
    nrm = np.tile(np.array([[1.0, 0.0, 0.0]], np.float32), (n, 1))
    wl = scenes.small_scene()
    mats = [api.MaterialProperties(*m) for m in wl.scene.materials]
    mesh = api.Mesh(tri, nrm, np.zeros(n, np.int32))
    a = api.DeviceScene(mesh, mats)
    b = api.DeviceScene(mesh, mats, host_prep=True)
    ra, rb = a.reference_bvh(), b.reference_bvh()
    for key in ("links", "order"):
        np.testing.assert_array_equal(ra[key], rb[key])
    np.testing.assert_array_equal(ra["boxes"].view(np.int64), rb["boxes"].view(np.int64))
    np.testing.assert_array_equal(a.mesh_order(), b.mesh_order())
    a.close()
    b.close()
