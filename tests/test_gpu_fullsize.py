"""GPU path against the oracle at full benchmark sizes.

The fixtures (tests/golden/make_oracle_fixtures.py) hold the FP64 CPU
oracle's complete output for:

  urban_L9_R6T1_rx10000  the benchmark solve itself: urban canyon, level 9
                         (2,621,442 rays), 6 reflections + 1 transmission,
                         all 10,000 receivers
  large_L9_R8_rx5000     the large terrain (580,484 triangles) at level 9,
                         8 reflections, 5,000 of its 50,000 receivers
  batch_L6L7L9_rx4096    a subset of the 256-transmitter batch (every level-6
                         and level-7 request plus two level-9 requests), run
                         as ONE batched call

Each test regenerates the workload from its seed, checks the input hash the
fixture recorded, solves it on the GPU through the C ABI on the fast capture
path (the one the benchmark times) and asserts: the identical path set
(request, receiver, launch, ray count, facet ids, coplanar ids, interaction
kinds, in the reference's order), bit-equal corrected points, the segment,
corrected-capture and path counts, and every field component within 1e-4
relative magnitude / 1e-3 rad (FP64 field: within 1e-9)."""
import os

import numpy as np
import pytest

from helpers import field_close, max_rel_err
from sbrsolver_gb300 import api

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _fixtures():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_oracle_fixtures", os.path.join(GOLD, "make_oracle_fixtures.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


FX = _fixtures()


def _fixture_paths(g):
    off = g["path_offset"]
    return {"request": g["path_request"].astype(np.int64),
            "receiver": g["path_receiver"].astype(np.int64),
            "launch": g["path_launch"].astype(np.int64),
            "n_rays": np.diff(off).astype(np.int64), "tri": g["tri"], "cop": g["cop"],
            "kind": g["kind"], "points": g["points"]}


def _gpu_paths(p):
    return {"request": p["request"].astype(np.int64), "receiver": p["receiver"].astype(np.int64),
            "launch": p["launch"].astype(np.int64), "n_rays": p["n_rays"].astype(np.int64),
            "tri": p["tri"], "cop": p["cop"], "kind": p["kind"], "points": p["points"]}


@pytest.mark.parametrize("name", list(FX.CASES))
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_fullsize_against_oracle(built, name, precision):
    path = os.path.join(GOLD, name + ".npz")
    if not os.path.exists(path):
        pytest.skip(f"{name}.npz not generated (tests/golden/make_oracle_fixtures.py {name})")
    g = np.load(path)
    scene, reqs = FX.CASES[name]()
    assert FX.inputs_sha256(scene, reqs) == str(g["inputs_sha256"]), \
        "the workload generator no longer makes the fixture's inputs"
    sc = api.DeviceScene.from_scene(scene)
    try:
        qs = [api.request_from_workload(r, precision) for r in reqs]
        res = api.solve(sc, qs if len(qs) > 1 else qs[0], with_paths="arrays")
    finally:
        sc.close()
    counts = g["counts"]  # per request: segments, captured, corrected, paths, rays
    assert res.counts["segments"] == int(counts[:, 0].sum())
    assert res.counts["corrected"] == int(counts[:, 2].sum())
    assert res.counts["paths"] == int(counts[:, 3].sum())
    assert res.counts["rays"] == int(counts[:, 4].sum())
    a, b = _gpu_paths(res.paths), _fixture_paths(g)
    # the batched result lists paths request by request
    for k in ("request", "receiver", "launch", "n_rays", "tri", "cop", "kind"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    # corrected points: FP64 image method in the reference's operation order
    np.testing.assert_array_equal(a["points"], b["points"])
    ref_field = np.ascontiguousarray(g["field"], np.float64).view(np.complex128).reshape(-1, 3)
    assert res.field.shape == ref_field.shape
    bad = field_close(res.field, ref_field)
    assert not bad, (len(bad), bad[:5])
    if precision == "fp64":
        assert max_rel_err(res.field, ref_field) < 1e-9
