"""Server (continuous admission, overlapping solves): every result equals the
same request solved alone, and batches equal separate solves."""
import time

import numpy as np
import pytest

from helpers import path_keys
from sbrsolver_gb300 import api, scenes

pytestmark = pytest.mark.gpu


def _requests():
    small = scenes.small_scene()
    urban = scenes.urban_scene(level=5, rx_pitch=100.0)
    reqs = []
    rng = np.random.default_rng(7)
    for i in range(8):
        wl = small if i % 2 == 0 else urban
        r = wl.request
        half = 90.0 if i % 2 == 0 else 450.0
        tx = (float(rng.uniform(-half, half)), float(rng.uniform(-half, half)), float(rng.uniform(5, 30)))
        nrx = int(rng.integers(8, 200))
        rx = np.column_stack([rng.uniform(-half, half, (nrx, 2)), np.full(nrx, 1.5)])
        req = scenes.Request(tx=tx, rx=rx, max_reflection=int(rng.integers(1, 5)),
                             max_transmission=int(rng.integers(0, 2)),
                             frequency=float(np.exp(rng.uniform(np.log(0.9e9), np.log(60e9)))),
                             tessellation=int(rng.integers(3, 7)), antenna=int(rng.integers(0, 3)))
        reqs.append((i % 2, req))
    return small, urban, reqs


@pytest.mark.parametrize("policy", [None, (0, 1, 0.0), (64 << 30, 64, 1e15),
                                    (2 << 30, 64, 16e9, 1), (0, 1, 16e9, 2)],
                         ids=["default", "never_batched", "batch_everything_fifo",
                              "one_large_at_once", "unbatched_two_at_once"])
def test_results_identical_alone_and_in_the_mix(built, policy):
    small, urban, reqs = _requests()
    sc = [api.DeviceScene.from_scene(small.scene), api.DeviceScene.from_scene(urban.scene)]
    alone = [api.solve(sc[s], api.request_from_workload(r), with_paths=True) for s, r in reqs]
    srv = api.Server(sc, slots=4)
    if policy is not None:
        srv.set_policy(*policy)
    with pytest.raises(Exception):
        srv.set_policy(1 << 30, 0, 1e9)  # at least one request per pass
    with pytest.raises(Exception):
        srv.set_policy(1 << 30, 8, 1e9, -1)  # a limit on large solves is >= 0
    keep = []
    for tag, (s, r) in enumerate(reqs):
        q = api.request_from_workload(r)
        keep.append(q)
        srv.submit(s, q, tag)
    got = {}
    t0 = time.time()
    while len(got) < len(reqs) and time.time() - t0 < 300:
        for c in srv.poll(timeout_ms=200, with_paths=True):
            assert c["status"] == 0
            got[c["tag"]] = c
    srv.close()
    assert len(got) == len(reqs)
    for tag, ref in enumerate(alone):
        res = got[tag]["result"]
        np.testing.assert_array_equal(res.field, ref.field)
        assert path_keys(res.paths) == path_keys(ref.paths)
        assert res.counts["segments"] == ref.counts["segments"]
        assert got[tag]["latency_ms"] >= got[tag]["queue_ms"] >= 0


def test_batch_of_many_equals_separate(built):
    small, urban, reqs = _requests()
    sc = api.DeviceScene.from_scene(urban.scene)
    ur = [r for s, r in reqs if s == 1]
    sep = [api.solve(sc, api.request_from_workload(r)) for r in ur]
    bat = api.solve(sc, [api.request_from_workload(r) for r in ur])
    np.testing.assert_array_equal(bat.field, np.concatenate([x.field for x in sep]))
    for i, x in enumerate(sep):
        assert path_keys([p for p in bat.paths if p["request"] == i]) == path_keys(x.paths)
