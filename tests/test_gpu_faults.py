"""Failure handling on the GPU path, with every failure made on the host.

No test here faults or hangs the GPU.  A device allocation failure is
injected by the library's own hook (sbr_fault_inject_alloc: the allocation
fails as on a full device, without calling cudaMalloc); admission pressure is
a server budget of one byte; bad inputs are NaN / inf coordinates.  Each case
must come back as a status, and the library must work normally afterwards.
The reference reports no errors from its solve at all (RTSolver.cpp:52-126),
so these behaviours are this library's own contract (include/sbr.h)."""
import ctypes as C
import time

import numpy as np
import pytest

from sbrsolver_gb300 import _lib, api, scenes

pytestmark = pytest.mark.gpu


def _many_receivers(n, seed=11):
    """n receivers over the small scene at 1.5 m: more than any other test of
    the suite uploads, so the solve must grow its receiver buffers."""
    rng = np.random.default_rng(seed)
    return np.column_stack([rng.uniform(-90, 90, n), rng.uniform(-90, 90, n), np.full(n, 1.5)])


@pytest.fixture
def disarm():
    yield
    _lib.load().sbr_fault_inject_alloc(-1)


def _small_request(rx, level=0):
    wl = scenes.small_scene()
    wl.request.rx = rx
    wl.request.tessellation = level
    wl.request.max_reflection = 0
    return wl


def test_injected_oom_in_scene_create(built, disarm):
    lib = _lib.load()
    wl = scenes.small_scene()
    lib.sbr_fault_inject_alloc(0)
    with pytest.raises(_lib.SbrError) as e:
        api.DeviceScene.from_scene(wl.scene)
    assert e.value.status == _lib.ERR_OOM
    lib.sbr_fault_inject_alloc(-1)
    sc = api.DeviceScene.from_scene(wl.scene)  # works again
    assert sc.info().n_triangles == wl.scene.n_tri
    sc.close()


def test_injected_oom_in_solve_then_recovery(built, disarm):
    lib = _lib.load()
    wl = _small_request(_many_receivers(1_500_000))
    sc = api.DeviceScene.from_scene(wl.scene)
    q = api.request_from_workload(wl.request)
    lib.sbr_fault_inject_alloc(0)  # the receiver upload must grow a buffer
    with pytest.raises(_lib.SbrError) as e:
        api.solve(sc, q, with_paths=False)
    assert e.value.status == _lib.ERR_OOM
    assert "cudaMalloc" in str(e.value)
    lib.sbr_fault_inject_alloc(-1)
    r1 = api.solve(sc, q, with_paths=False)
    r2 = api.solve(sc, q, with_paths=False)
    assert r1.counts["paths"] > 0
    np.testing.assert_array_equal(r1.field, r2.field)
    sc.close()


def test_server_reports_injected_oom_and_keeps_serving(built, disarm):
    lib = _lib.load()
    wl = _small_request(_many_receivers(3_000_000, seed=12))
    sc = api.DeviceScene.from_scene(wl.scene)
    ok = scenes.small_scene()
    ok.request.tessellation = 3
    expect = api.solve(sc, api.request_from_workload(ok.request), with_paths=False)
    srv = api.Server([sc], slots=1)
    big = api.request_from_workload(wl.request)
    lib.sbr_fault_inject_alloc(0)
    srv.submit(0, big, 1)
    got = []
    t0 = time.time()
    while not got and time.time() - t0 < 120:
        got += srv.poll(timeout_ms=200)
    assert got and got[0]["tag"] == 1 and got[0]["status"] == _lib.ERR_OOM
    assert got[0]["result"] is None
    lib.sbr_fault_inject_alloc(-1)
    small = api.request_from_workload(ok.request)
    srv.submit(0, small, 2)
    got = []
    t0 = time.time()
    while not got and time.time() - t0 < 120:
        got += srv.poll(timeout_ms=200)
    assert got[0]["tag"] == 2 and got[0]["status"] == _lib.OK
    srv.close()
    sc.close()
    assert got[0]["counts"]["paths"] == expect.counts["paths"]


def test_server_budget_of_one_byte_runs_one_at_a_time(built):
    """With an HBM budget smaller than any request, the server admits a
    request only when nothing else is on the GPU: every request completes,
    and no two run at the same time."""
    wl = scenes.small_scene()
    sc = api.DeviceScene.from_scene(wl.scene)
    srv = api.Server([sc], slots=3, hbm_budget=1)
    qs, t_sub = [], {}
    for k in range(6):
        w = scenes.small_scene()
        w.request.tessellation = 4 + k % 2
        w.request.tx = (-30.0 + 10 * k, 5.0, 10.0)
        qs.append(api.request_from_workload(w.request))
    for k, q in enumerate(qs):
        t_sub[k] = time.perf_counter()
        srv.submit(0, q, k)
    done = []
    t0 = time.time()
    while len(done) < len(qs) and time.time() - t0 < 120:
        done += srv.poll(timeout_ms=200)
    srv.close()
    sc.close()
    assert sorted(c["tag"] for c in done) == list(range(len(qs)))
    assert all(c["status"] == _lib.OK for c in done)
    spans = sorted((t_sub[c["tag"]] * 1e3 + c["queue_ms"], t_sub[c["tag"]] * 1e3 + c["latency_ms"])
                   for c in done)
    for (a0, a1), (b0, b1) in zip(spans, spans[1:]):
        assert b0 >= a1 - 0.5, (spans, "two requests overlapped under a 1-byte budget")


@pytest.mark.parametrize("what", ["tx_nan", "txcs_inf", "rx_inf", "pt_nan"])
def test_non_finite_request_rejected(built, what):
    wl = scenes.small_scene()
    sc = api.DeviceScene.from_scene(wl.scene)
    r = wl.request
    if what == "tx_nan":
        r.tx = (0.0, float("nan"), 10.0)
    elif what == "txcs_inf":
        r.tx_coord_sys = (1, 0, 0, 0, float("inf"), 0, 0, 0, 1)
    elif what == "rx_inf":
        r.rx = r.rx.copy()
        r.rx[3, 0] = -np.inf
    else:
        r.pt = float("nan")
    with pytest.raises(_lib.SbrError) as e:
        api.solve(sc, api.request_from_workload(r))
    assert e.value.status == _lib.ERR_INVALID_ARG
    assert "finite" in str(e.value)
    sc.close()


def test_non_finite_device_receivers_rejected(built):
    """Receivers the caller placed on the device are checked on the device:
    the solve returns an argument error and the next solve is unaffected."""
    torch = pytest.importorskip("torch")
    wl = scenes.small_scene()
    sc = api.DeviceScene.from_scene(wl.scene)
    good = api.solve(sc, api.request_from_workload(wl.request), with_paths=False)
    rx = torch.tensor(wl.request.rx, dtype=torch.float64, device="cuda")
    rx[7, 2] = float("nan")
    q, keep = api.request_from_workload(wl.request)
    q.rx = C.cast(C.c_void_p(rx.data_ptr()), C.POINTER(C.c_double))
    q.rx_on_device = 1
    torch.cuda.synchronize()
    with pytest.raises(_lib.SbrError) as e:
        api.solve(sc, (q, keep), with_paths=False)
    assert e.value.status == _lib.ERR_INVALID_ARG
    assert "receiver coordinates must be finite" in str(e.value)
    again = api.solve(sc, api.request_from_workload(wl.request), with_paths=False)
    np.testing.assert_array_equal(again.field, good.field)
    sc.close()
