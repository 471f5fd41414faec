"""Scene preparation against the reference's own: StlToGeometry and
BVH::ConstructBVH (Preprocessor.cpp:69-246, BVH/BVH.h:135-230) run on the
same STL by the reference harness (tests/golden/make_golden.py --bvh).  Each
fixture holds the triangle id at each position of the sorted triangle vector,
the coplanar ids and frame rows by triangle id, and the tree in depth-first
order from the root (node boxes, leaf sizes with -1 for inner nodes, the
leaves' triangle ids in visit order); the 580,484-triangle terrain holds
sha256 digests of those arrays."""
import hashlib
import os

import numpy as np
import pytest

import oracle as orc
from sbrsolver_gb300 import api, scenes

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SCENES = ["small", "urban", "large", "ties", "heap_sort", "flat"]


def _fixture(name):
    return np.load(os.path.join(GOLD, f"refbvh_{name}.npz"))


def _mesh(name, g):
    """Triangles and facet normals the fixture was made from."""
    if "tri" in g:
        return g["tri"], g["normal"]
    sc = {"small": scenes.small_scene, "urban": lambda: scenes.urban_scene(level=2),
          "large": scenes.large_scene}[name]().scene
    return sc.tri, sc.normal


def _check(g, key, got):
    got = np.ascontiguousarray(got)
    if key + "_sha256" in g:
        assert hashlib.sha256(got.tobytes()).hexdigest() == str(g[key + "_sha256"]), key
    else:
        want = g[key]
        assert got.shape == want.shape, (key, got.shape, want.shape)
        if got.dtype.kind == "f":  # bit for bit, signed zeros included
            np.testing.assert_array_equal(got.view(np.int64), want.view(np.int64), err_msg=key)
        else:
            np.testing.assert_array_equal(got, want, err_msg=key)


def _depth_first(bvh):
    """Boxes, leaf sizes (-1 inner) and leaf triangle ids from the library's
    reference BVH, walked from the root with child 0 first."""
    links, boxes, order = bvh["links"], bvh["boxes"], bvh["order"]
    pre_boxes, leaf_n, leaf_ids, stack = [], [], [], [0]
    while stack:
        k = stack.pop()
        pre_boxes.append(boxes[k])
        c0, c1, first, count = (int(x) for x in links[k, :4])
        if c0 < 0:
            leaf_n.append(count)
            leaf_ids.append(order[first:first + count])
        else:
            leaf_n.append(-1)
            stack += [c1, c0]
    return (np.array(pre_boxes, np.float64).reshape(-1, 6), np.array(leaf_n, np.int32),
            np.concatenate(leaf_ids).astype(np.int32))


@pytest.mark.parametrize("name", SCENES)
def test_fixture_inputs_are_reproducible(name):
    g = _fixture(name)
    tri, nrm = _mesh(name, g)
    h = hashlib.sha256(np.ascontiguousarray(tri, "<f4").tobytes() +
                       np.ascontiguousarray(nrm, "<f4").tobytes()).hexdigest()
    assert h == str(g["inputs_sha256"])


@pytest.mark.parametrize("name", [s for s in SCENES if s != "large"])
def test_fixture_boxes_bound_the_fixture_tree(name):
    """The fixture's boxes are exact: a leaf's box is the bounds of its
    triangles' (float) vertices and an inner node's the union of its two
    children's (in depth-first order node k's children are k + 1 and
    k + 1 + size(k + 1)); every triangle sits in exactly one leaf."""
    g = _fixture(name)
    tri, _ = _mesh(name, g)
    boxes, leaf_n, leaf_ids = g["boxes"], g["leaf_n"], g["leaf_ids"]
    m = len(leaf_n)
    size = np.ones(m, np.int64)
    for k in range(m - 1, -1, -1):
        if leaf_n[k] < 0:
            size[k] = 1 + size[k + 1] + size[k + 1 + size[k + 1]]
    assert size[0] == m
    assert np.array_equal(np.sort(leaf_ids), np.arange(len(tri)))
    v = tri.astype(np.float64)
    lo, hi = v.min(axis=1), v.max(axis=1)
    at = 0
    for k in range(m):
        if leaf_n[k] >= 0:
            ids = leaf_ids[at:at + leaf_n[k]]
            at += leaf_n[k]
            want = np.concatenate([lo[ids].min(axis=0), hi[ids].max(axis=0)])
        else:
            a, b = boxes[k + 1], boxes[k + 1 + size[k + 1]]
            want = np.concatenate([np.minimum(a[:3], b[:3]), np.maximum(a[3:], b[3:])])
        np.testing.assert_array_equal(boxes[k], want, err_msg=f"node {k}")


@pytest.mark.parametrize("name", SCENES)
def test_oracle_mesh_order_and_coplanar_ids(built, name):
    g = _fixture(name)
    tri, nrm = _mesh(name, g)
    sc = orc.OracleScene(tri, nrm, np.zeros(len(tri), np.int32))
    _check(g, "mesh_order", sc.mesh_order())
    _check(g, "coplanar", sc.coplanar_ids())


@pytest.mark.gpu
@pytest.mark.parametrize("host_prep", [False, True], ids=["device", "host"])
@pytest.mark.parametrize("name", SCENES)
def test_scene_tables_match_reference(built, name, host_prep):
    g = _fixture(name)
    tri, nrm = _mesh(name, g)
    mats = [api.MaterialProperties(*m) for m in scenes.small_scene().scene.materials]
    sc = api.DeviceScene(api.Mesh(tri, nrm, np.zeros(len(tri), np.int32)), mats,
                         host_prep=host_prep)
    try:
        boxes, leaf_n, leaf_ids = _depth_first(sc.reference_bvh())
        assert len(leaf_n) == int(g["n_nodes"])
        _check(g, "boxes", boxes)
        _check(g, "leaf_n", leaf_n)
        _check(g, "leaf_ids", leaf_ids)
        _check(g, "mesh_order", sc.mesh_order())
        _check(g, "coplanar", sc.coplanar_ids())
        frames = sc.triangle_frames()[0].reshape(len(tri), 9)
        _check(g, "frames", frames)
    finally:
        sc.close()
