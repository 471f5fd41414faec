"""Tabulated antenna patterns (the TXPattern.dat grid): parsing without a
GPU, and on a GPU a table built from the Hertzian dipole reproducing the
analytic Hertzian pattern's paths exactly and its fields to the bilinear
interpolation error."""
import ctypes as C

import numpy as np
import pytest

from sbrsolver_gb300 import _lib, api, scenes


def hertzian_table(d=1.0):
    th = np.arange(0, 180 + d / 2, d)
    nt, npp = len(th), int(round(360 / d))
    t = np.zeros((nt, npp, 4), np.float64)
    s = np.abs(np.sin(np.radians(th)))
    with np.errstate(divide="ignore"):
        g = np.where(s > 0, 20 * np.log10(np.sqrt(1.5) * np.maximum(s, 1e-300)), -400.0)
    t[:, :, 0] = g[:, None]
    t[:, :, 1] = 90.0          # j
    t[:, :, 2] = -400.0        # no E_phi
    return t


def test_read_pattern_file_like_reference(tmp_path):
    t = hertzian_table(30.0)
    f = str(tmp_path / "TXPattern.dat")
    api.write_pattern_file(f, t, 30.0, 30.0)
    out = {}
    assert api.Preprocessor.ReadPatternFile(f, out)
    assert len(out) == t.shape[0] * t.shape[1]          # the title and grid lines are skipped
    assert out[(90.0, 0.0)][1] == pytest.approx(90.0)
    assert not api.Preprocessor.ReadPatternFile(str(tmp_path / "missing.dat"), {})


def test_pattern_file_errors_without_gpu(built, tmp_path):
    lib = _lib.load()
    h = C.c_void_p()
    assert lib.sbr_pattern_read(str(tmp_path / "none.dat").encode(), C.byref(h)) == _lib.ERR_IO
    f = tmp_path / "holes.dat"
    f.write_text("0 0 0 0 0 0\n0 180 0 0 0 0\n10 0 0 0 0 0\n")  # (10, 180) missing
    assert lib.sbr_pattern_read(str(f).encode(), C.byref(h)) == _lib.ERR_INVALID_ARG
    assert b"missing grid point" in lib.sbr_last_error()
    bad = np.zeros(4, np.float32)
    assert lib.sbr_pattern_create(1, 3, 1.0, 1.0, bad.ctypes.data_as(C.POINTER(C.c_float)),
                                  C.byref(h)) == _lib.ERR_INVALID_ARG


@pytest.mark.gpu
def test_tabulated_hertzian_matches_analytic(built, tmp_path):
    f = str(tmp_path / "TXPattern.dat")
    api.write_pattern_file(f, hertzian_table(1.0), 1.0, 1.0)
    pat = api.AntennaPattern.read(f)
    assert pat.info() == (181, 360, 1.0, 1.0)
    wl = scenes.small_scene()
    wl.request.antenna = 1
    sc = api.DeviceScene.from_scene(wl.scene)
    ana = api.solve(sc, api.request_from_workload(wl.request), with_paths="arrays")
    q = api.make_request(wl.request.tx, wl.request.tx_coord_sys, wl.request.max_reflection,
                         wl.request.max_transmission, wl.request.frequency, wl.request.pt,
                         wl.request.use_fresnel, wl.request.rx, wl.request.tessellation,
                         antenna=3, pattern=pat)
    tab = api.solve(sc, q, with_paths="arrays")
    assert api.same_path_set(tab.paths, ana.paths) and tab.counts["paths"] > 0
    a, b = ana.paths["field"], tab.paths["field"]          # per path: (Ex re, im, Ey, Ez)
    ea = np.linalg.norm(a, axis=1)
    assert np.max(np.linalg.norm(a - b, axis=1) / ea) < 1e-4  # bilinear error ~ (1 deg)^2 / 8
    # a request without its pattern is refused
    q2 = api.make_request(wl.request.tx, wl.request.tx_coord_sys, 1, 0, wl.request.frequency, 1.0,
                          True, wl.request.rx, 2, antenna=3)
    with pytest.raises(_lib.SbrError):
        api.solve(sc, q2)
    pat.close()
    sc.close()
