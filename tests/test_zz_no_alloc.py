"""The allocation-free per-receiver field sum, through the C ABI.

It serves callers that cannot allocate device memory (their device memory is
held by another framework's caching allocator, or their footprint must stay
fixed after start-up), so these tests hand it device buffers it did not
allocate itself (torch tensors) and call it twice in a row: the second call
must not see the first call's leftovers in the shared scratch array.  Its
output is checked against the fields sbr_solve returns for the same paths,
and, on a skewed synthetic path list (receivers with many paths, which take
the block-wide sort), against the same ordered sum formed on the CPU.
Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from helpers import field_close
from sbrsolver_gb300 import _lib, api, scenes

pytestmark = pytest.mark.gpu

PRECISION = {"fp64": 0, "fp32": 1, "fp32_phase": 2}


def _call(lib, torch, recv, rank, pf, n_paths, n_rx, prec):
    out = torch.full((n_rx * 6,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    st = lib.sbr_receiver_field_sum_noalloc(
        C.c_void_p(recv.data_ptr()), C.c_void_p(rank.data_ptr()), C.c_void_p(pf.data_ptr()),
        n_paths, n_rx, prec, C.c_void_p(out.data_ptr()),
        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return st, out


@pytest.mark.parametrize("precision", ["fp64", "fp32", "fp32_phase"])
def test_noalloc_field_sum_matches_solve(built, precision):
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    wl = scenes.reference_main_scene()   # 3000 receivers, 3133 paths, up to 2 per receiver
    sc = api.DeviceScene.from_scene(wl.scene)
    res = api.solve(sc, api.request_from_workload(wl.request, precision))
    n_rx = len(wl.request.rx)
    recv = torch.tensor([p["receiver"] for p in res.paths], dtype=torch.int32, device="cuda")
    rank = torch.tensor([(p["launch"] << 17) | p["heap"] for p in res.paths], dtype=torch.int64,
                        device="cuda")
    pf = torch.tensor(np.array([p["field"] for p in res.paths]).reshape(-1), dtype=torch.float64,
                      device="cuda")
    ref = np.stack([res.field.real, res.field.imag], -1).reshape(n_rx, 6)
    # the solve's FP32 mode sums in FP64 the receivers its error bound could
    # not certify (field_bound 0); this entry point always sums an FP32
    # precision in compensated FP32, so those receivers agree within the
    # field tolerance, every other receiver to the last bits
    same = np.ones(n_rx, bool) if precision != "fp32" else res.field_bound != 0
    for _ in range(2):
        st, out = _call(lib, torch, recv, rank, pf, len(res.paths), n_rx, PRECISION[precision])
        _lib.check(st)
        got = out.cpu().numpy().reshape(n_rx, 6)
        np.testing.assert_allclose(got[same], ref[same], rtol=1e-12, atol=0)
        c = np.ascontiguousarray(got).view(np.complex128).reshape(-1, 3)
        assert not field_close(c, res.field)
    sc.close()


def _ordered_sum(recv, rank, pf, n_rx, precision):
    """The sum the entry point defines, on the CPU: each receiver's paths in
    (rank, path index) order, added one after the other in FP64, or in FP32
    with Neumaier compensation for the FP32 precisions."""
    out = np.zeros((n_rx, 6))
    order = np.lexsort((np.arange(len(rank)), rank))
    for r in range(n_rx):
        idx = [i for i in order if recv[i] == r]
        if precision == 0:
            acc = [0.0] * 6
            for i in idx:
                for k in range(6):
                    acc[k] = acc[k] + float(pf[i, k])
            out[r] = acc
        else:
            f = np.float32
            s, c = [f(0)] * 6, [f(0)] * 6
            for i in idx:
                for k in range(6):
                    x = f(pf[i, k])
                    t = f(s[k] + x)
                    c[k] = f(c[k] + (f(f(s[k] - t) + x) if abs(s[k]) >= abs(x) else f(f(x - t) + s[k])))
                    s[k] = t
            out[r] = [float(a) + float(b) for a, b in zip(s, c)]
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_skewed_receivers(built, precision):
    """One receiver with 1,500 paths and one with 40 (block-wide sorts), the
    rest with 0-3 (one thread each), ranks shuffled and some repeated."""
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    rng = np.random.default_rng(7)
    n_rx = 64
    recv = np.concatenate([np.zeros(1500, np.int32), np.ones(40, np.int32),
                           rng.integers(2, n_rx, 120).astype(np.int32)])
    rng.shuffle(recv)
    n = len(recv)
    rank = rng.integers(0, 1 << 30, n).astype(np.int64)
    rank[::50] = rank[1::50][: len(rank[::50])]  # repeated ranks: ties go by path index
    pf = rng.normal(size=(n, 6)) * np.exp(rng.uniform(-20, 5, (n, 1)))
    ref = _ordered_sum(recv, rank, pf, n_rx, precision)
    t = lambda a, dt: torch.tensor(a, dtype=dt, device="cuda")  # noqa: E731
    args = (t(recv, torch.int32), t(rank, torch.int64), t(pf.reshape(-1), torch.float64))
    for _ in range(2):
        st, out = _call(lib, torch, *args, n, n_rx, precision)
        _lib.check(st)
        np.testing.assert_array_equal(out.cpu().numpy().reshape(n_rx, 6), ref)


def test_noalloc_rejects_bad_input(built):
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    st = lib.sbr_receiver_field_sum_noalloc(None, None, None, 0, 1 << 20, 0, C.c_void_p(1), None)
    assert st == _lib.ERR_INVALID_ARG
    assert b"n_rx" in lib.sbr_last_error()
    st = lib.sbr_receiver_field_sum_noalloc(None, None, None, 0, 4, 7, C.c_void_p(1), None)
    assert st == _lib.ERR_INVALID_ARG
    assert b"field_precision" in lib.sbr_last_error()
    # more paths on one receiver than the per-receiver limit (2,048)
    n = 2049
    recv = torch.zeros(n, dtype=torch.int32, device="cuda")
    rank = torch.arange(n, dtype=torch.int64, device="cuda")
    pf = torch.zeros(6 * n, dtype=torch.float64, device="cuda")
    st, _ = _call(lib, torch, recv, rank, pf, n, 2, 0)
    assert st == _lib.ERR_INVALID_ARG
    assert b"more than 2048" in lib.sbr_last_error()
    # a receiver index outside [0, n_rx)
    recv = torch.tensor([0, 5], dtype=torch.int32, device="cuda")
    st, _ = _call(lib, torch, recv, rank[:2], pf[:12], 2, 2, 0)
    assert st == _lib.ERR_INVALID_ARG
    # the next valid call is not affected by the failed ones
    recv = torch.tensor([1, 0, 1], dtype=torch.int32, device="cuda")
    pf = torch.arange(18, dtype=torch.float64, device="cuda")
    st, out = _call(lib, torch, recv, torch.tensor([5, 1, 2], dtype=torch.int64, device="cuda"),
                    pf, 3, 2, 0)
    _lib.check(st)
    got = out.cpu().numpy().reshape(2, 6)
    np.testing.assert_array_equal(got[0], np.arange(6, 12))
    np.testing.assert_array_equal(got[1], np.arange(12, 18) + np.arange(0, 6))


def test_noalloc_inside_cuda_graph(built):
    """Captured into a CUDA graph (torch.cuda.graph), the call only enqueues
    its kernels; replays sum whatever the path buffers hold at replay time."""
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    rng = np.random.default_rng(11)
    n_rx, n = 48, 400
    recv = rng.integers(0, n_rx, n).astype(np.int32)
    recv[:60] = 3  # one receiver with a block-wide sort
    rank = rng.integers(0, 1 << 30, n).astype(np.int64)
    pf = rng.normal(size=(n, 6))
    t = lambda a, dt: torch.tensor(a, dtype=dt, device="cuda")  # noqa: E731
    d_recv, d_rank, d_pf = t(recv, torch.int32), t(rank, torch.int64), t(pf.reshape(-1),
                                                                        torch.float64)
    st, _ = _call(lib, torch, d_recv, d_rank, d_pf, n, n_rx, 0)  # set-up outside the capture
    _lib.check(st)
    out = torch.zeros(n_rx * 6, dtype=torch.float64, device="cuda")
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g):
        st = lib.sbr_receiver_field_sum_noalloc(
            C.c_void_p(d_recv.data_ptr()), C.c_void_p(d_rank.data_ptr()),
            C.c_void_p(d_pf.data_ptr()), n, n_rx, 0, C.c_void_p(out.data_ptr()),
            C.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(st)
    for scale in (1.0, -0.5):
        d_pf.copy_(t(scale * pf.reshape(-1), torch.float64))
        out.zero_()
        g.replay()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy().reshape(n_rx, 6),
                                      _ordered_sum(recv, rank, scale * pf, n_rx, 0))
