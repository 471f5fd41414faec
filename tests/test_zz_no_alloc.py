"""The allocation-free per-receiver field sum, through the C ABI, against the
fields sbr_solve returns.

It is meant for callers that cannot allocate device memory (inside CUDA
graph capture, or with device memory owned by another framework's pool), so
this test hands it device buffers it did not allocate itself (torch tensors)
and calls it twice in a row: the second call must not see the first call's
leftovers in the shared scratch array.  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from sbrsolver_gb300 import _lib, api, scenes

pytestmark = pytest.mark.gpu


def _inputs(res, torch):
    recv = torch.tensor([p["receiver"] for p in res.paths], dtype=torch.int32, device="cuda")
    rank = torch.tensor([(p["launch"] << 17) | p["heap"] for p in res.paths], dtype=torch.int64,
                        device="cuda")
    pf = torch.tensor(np.array([p["field"] for p in res.paths]).reshape(-1), dtype=torch.float64,
                      device="cuda")
    return recv, rank, pf


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_noalloc_field_sum_matches_solve(built, precision):
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    wl = scenes.reference_main_scene()   # 3000 receivers, 3133 paths, up to 2 per receiver
    sc = api.DeviceScene.from_scene(wl.scene)
    res = api.solve(sc, api.request_from_workload(wl.request, precision))
    n_rx = len(wl.request.rx)
    recv, rank, pf = _inputs(res, torch)
    ref = np.stack([res.field.real, res.field.imag], -1).reshape(n_rx, 6)
    prec = 1 if precision == "fp32" else 0
    for _ in range(2):
        out = torch.full((n_rx * 6,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        st = lib.sbr_receiver_field_sum_noalloc(
            C.c_void_p(recv.data_ptr()), C.c_void_p(rank.data_ptr()), C.c_void_p(pf.data_ptr()),
            len(res.paths), n_rx, prec, C.c_void_p(out.data_ptr()),
            C.c_void_p(torch.cuda.current_stream().cuda_stream))
        _lib.check(st)
        got = out.cpu().numpy().reshape(n_rx, 6)
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0)
    sc.close()


def test_noalloc_rejects_oversize(built):
    lib = _lib.load()
    st = lib.sbr_receiver_field_sum_noalloc(None, None, None, 0, 1 << 20, 0, C.c_void_p(1), None)
    assert st == _lib.ERR_INVALID_ARG
    assert b"n_rx" in lib.sbr_last_error()
