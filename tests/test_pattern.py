"""Tabulated antenna patterns (the TXPattern.dat grid).

The reference reads TXPattern.dat (Preprocessor::ReadPatternFile,
Preprocessor.cpp:3-35) but never applies it, so antenna type 3's rule is
this project's: E_theta, E_phi = sqrt(60 Pt) 10^(g/20) e^(j arg), bilinear on
the grid.  The oracle states that rule on its own (oracle/sbr_oracle.cpp,
Pattern) and is pinned where the reference does define a value: a table
sampled from the Hertzian dipole must reproduce the reference's own Hertzian
run (the shipped main() scene, 3,133 paths) to the interpolation error.  The
GPU is then checked against the oracle with a two-polarisation table whose
gains and phases vary over the whole sphere."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle as orc
from helpers import field_close, golden_paths, path_keys
from sbrsolver_gb300 import _lib, api, scenes

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


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


def rippled_table(d=2.0, seed=3):
    """Both polarisations, gains and phases varying smoothly over the sphere
    (a few lobes), so every grid cell interpolates something different."""
    th = np.radians(np.arange(0, 180 + d / 2, d))[:, None]
    ph = np.radians(np.arange(0, 360, d))[None, :]
    rng = np.random.default_rng(seed)
    a = rng.uniform(0.5, 2.0, 6)
    t = np.zeros((th.shape[0], ph.shape[1], 4))
    t[:, :, 0] = -3 + 6 * np.sin(a[0] * th) * np.cos(2 * ph + a[1])
    t[:, :, 1] = 40 * np.cos(a[2] * th) + 25 * np.sin(ph)
    t[:, :, 2] = -8 + 4 * np.cos(3 * th) * np.sin(ph + a[3])
    t[:, :, 3] = -70 + 30 * np.sin(a[4] * th + ph)
    return t


def test_oracle_tabulated_hertzian_matches_reference(built):
    """The oracle's type 3 with a 1-degree Hertzian table against the
    reference's own Hertzian run: identical paths, every path's field within
    the bilinear interpolation error (~(1 deg)^2/8 = 4e-5 of its magnitude)."""
    g = np.load(os.path.join(GOLD, "reference_main.npz"))
    wl = scenes.reference_main_scene()
    wl.request.antenna = 3
    out = orc.solve(orc.OracleScene.from_scene(wl.scene), wl.request, wl.scene.materials,
                    pattern=(hertzian_table(1.0), 1.0, 1.0))
    ref = golden_paths(g)
    assert path_keys(out["paths"]) == path_keys(ref) and len(ref) == 3133
    a = np.array([p["field"] for p in out["paths"]])
    b = np.asarray(g["path_field"], np.float64).reshape(-1, 6)
    rel = np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)
    assert rel.max() < 1e-4, rel.max()
    assert rel.max() > 1e-9  # the table really is interpolated, not the analytic form


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


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_tabulated_pattern_against_oracle(built, tmp_path, precision):
    """Antenna type 3 with a two-polarisation table: the GPU's paths equal the
    oracle's and its received fields are within 1e-4 / 1e-3 rad (FP64 field:
    the table's single-precision amplitudes differ from the oracle's double
    ones by ~1e-7)."""
    t = rippled_table(2.0)
    f = str(tmp_path / "TXPattern.dat")
    api.write_pattern_file(f, t, 2.0, 2.0)
    pat = api.AntennaPattern.read(f)
    # the table as the file holds it: 6 significant digits, parsed as float32
    tab = np.vectorize(lambda v: float(np.float32(f"{v:.6g}")))(t)
    for wl in (scenes.small_scene(),
               scenes.urban_scene(level=5, rx_pitch=50.0, max_reflection=3, max_transmission=1)):
        wl.request.antenna = 3
        ref = orc.solve(orc.OracleScene.from_scene(wl.scene), wl.request, wl.scene.materials,
                        pattern=(tab, 2.0, 2.0))
        sc = api.DeviceScene.from_scene(wl.scene)
        q = api.make_request(wl.request.tx, wl.request.tx_coord_sys, wl.request.max_reflection,
                             wl.request.max_transmission, wl.request.frequency, wl.request.pt,
                             wl.request.use_fresnel, wl.request.rx, wl.request.tessellation,
                             antenna=3, precision=precision, pattern=pat)
        res = api.solve(sc, q)
        sc.close()
        assert path_keys(res.paths) == path_keys(ref["paths"]) and ref["paths"]
        assert np.abs(ref["field"][:, 2]).max() > 0  # E_phi reaches the receivers
        bad = field_close(res.field, ref["field"])
        assert not bad, bad[:5]
    pat.close()
