"""The device pipeline as a CUDA graph.

A solve whose pipeline (request structure, capacities, buffers, launch
shapes) ran before on the scene is captured as a graph the second time and,
from then on, replayed by one graph launch (a few graphs are kept per scene); the uploads read pinned staging buffers, so a
replay with other transmitter positions, powers or receiver coordinates of the
same counts computes the new inputs.  These tests check that replays happen
(counts["pipeline_graph"]) and that a replayed solve gives bit-identical
results to an eager solve of the same requests on a fresh scene."""
import ctypes as C
import dataclasses

import numpy as np
import pytest

from sbrsolver_gb300 import api, scenes

pytestmark = pytest.mark.gpu


def _solve(sc, reqs, precision="fp64"):
    qs = [api.request_from_workload(r, precision) for r in reqs]
    return api.solve(sc, qs if len(qs) > 1 else qs[0], with_paths="arrays")


def _same(a, b):
    np.testing.assert_array_equal(a.field, b.field)
    for k in ("request", "receiver", "launch", "n_rays", "tri", "cop", "kind", "points"):
        np.testing.assert_array_equal(a.paths[k], b.paths[k], err_msg=k)
    for k in ("segments", "captured", "corrected", "paths", "rays", "fp64_field_paths",
              "fp64_field_receivers"):
        assert a.counts[k] == b.counts[k], k


def _eager(wl_scene, reqs, precision="fp64"):
    sc = api.DeviceScene.from_scene(wl_scene)
    # workspaces are pooled per device: without this a fresh scene whose
    # pipeline matches one that ran before would replay its graph
    sc.set_tuning(pipeline_graph=-1)
    try:
        r = _solve(sc, reqs, precision)
        assert r.counts["pipeline_graph"] == 0
        return r
    finally:
        sc.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_repeat_is_captured_then_replayed(built, precision):
    wl = scenes.urban_scene(level=6)
    sc = api.DeviceScene.from_scene(wl.scene)
    try:
        runs = [_solve(sc, [wl.request], precision) for _ in range(7)]
        # eager while the pipeline is new (the first solves of a fresh
        # workspace grow its tables from the occupancy they see, which changes
        # the pipeline), captured the second time it repeats, then replayed
        flags = [r.counts["pipeline_graph"] for r in runs]
        assert flags[-3:] == [1, 1, 1], flags
        for r in runs[1:]:
            _same(r, runs[0])
        # the replay counts the kernels of the captured pipeline
        assert runs[6].counts["gpu_kernels"] == runs[5].counts["gpu_kernels"]
        # new transmitter position and power, receivers moved, same counts:
        # the graph replays and reads the new staged inputs
        moved = dataclasses.replace(
            wl.request, tx=tuple(np.add(wl.request.tx, (3.25, -2.5, 0.75))), pt=2.0,
            rx=wl.request.rx + np.array([0.5, -0.25, 0.0]))
        r = _solve(sc, [moved], precision)
        assert r.counts["pipeline_graph"] == 1
        _same(r, _eager(wl.scene, [moved], precision))
        assert not np.array_equal(r.field, runs[0].field)
        # another receiver count: a new pipeline, run eagerly
        fewer = dataclasses.replace(wl.request, rx=wl.request.rx[:-7])
        r = _solve(sc, [fewer], precision)
        assert r.counts["pipeline_graph"] == 0
        _same(r, _eager(wl.scene, [fewer], precision))
        # the first pipeline's graph is kept: it replays between the others
        r = _solve(sc, [wl.request], precision)
        assert r.counts["pipeline_graph"] == 1
        _same(r, runs[0])
        r = _solve(sc, [fewer], precision)  # seen once before: captured now
        assert r.counts["pipeline_graph"] == 1
        _same(r, _eager(wl.scene, [fewer], precision))
    finally:
        sc.close()


def test_batch_replay_and_device_receivers(built):
    import torch
    wl = scenes.urban_scene(level=5)
    reqs = [wl.request,
            dataclasses.replace(wl.request, tx=tuple(np.add(wl.request.tx, (-10.0, 4.0, 1.0))),
                                tessellation=4, max_reflection=3)]
    sc = api.DeviceScene.from_scene(wl.scene)
    try:
        first = [_solve(sc, reqs) for _ in range(6)]
        flags = [r.counts["pipeline_graph"] for r in first]
        assert flags[0] == 0 and flags[-2:] == [1, 1], flags
        _same(first[5], first[0])
        _same(first[0], _eager(wl.scene, reqs))
        # receivers resident on the device: the pointer is part of the
        # pipeline, the coordinates are read at replay time
        rx = torch.tensor(wl.request.rx, dtype=torch.float64, device="cuda")
        q = api.request_from_workload(wl.request)
        d, keep = api.request_from_workload(wl.request)
        d.rx = C.cast(C.c_void_p(rx.data_ptr()), C.POINTER(C.c_double))
        d.rx_on_device = 1
        dev = (d, keep)
        torch.cuda.synchronize()
        outs = [api.solve(sc, dev, with_paths="arrays") for _ in range(5)]
        flags = [o.counts["pipeline_graph"] for o in outs]
        assert flags[0] == 0 and flags[-2:] == [1, 1], flags  # the pointer is a new pipeline
        ref = api.solve(sc, q, with_paths="arrays")
        _same(outs[4], ref)
        rx += torch.tensor([1.0, 0.5, 0.0], dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        moved = api.solve(sc, dev, with_paths="arrays")
        assert moved.counts["pipeline_graph"] == 1
        host_moved = dataclasses.replace(wl.request, rx=rx.cpu().numpy())
        _same(moved, _eager(wl.scene, [host_moved]))
    finally:
        sc.close()


def test_concurrent_threads_capture_and_replay(built):
    """Four threads solve the same two requests over and over on one scene:
    each solve checks a workspace out of the pool, so graphs are captured and
    replayed in several workspaces while other threads launch and allocate
    (thread-local capture); every result equals the eager one."""
    import threading
    wl = scenes.urban_scene(level=5)
    other = dataclasses.replace(wl.request, tx=tuple(np.add(wl.request.tx, (7.0, -3.0, 2.0))),
                                max_reflection=3)
    refs = [_eager(wl.scene, [wl.request]), _eager(wl.scene, [other])]
    sc = api.DeviceScene.from_scene(wl.scene)
    errors, flags = [], []

    def work(t):
        try:
            for k in range(6):
                which = (t + k) % 2
                r = _solve(sc, [wl.request if which == 0 else other])
                flags.append(r.counts["pipeline_graph"])
                _same(r, refs[which])
        except Exception as e:  # reported below
            errors.append(repr(e))

    threads = [threading.Thread(target=work, args=(t,)) for t in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    sc.close()
    assert not errors, errors[:3]
    assert len(flags) == 24 and sum(flags) > 0  # some solves ran as graph replays
