"""The oracle (CPU restatement) against golden fixtures produced by the
reference's own sources (tests/golden/make_golden.py)."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle as orc
from helpers import golden_field, golden_paths, path_keys
from sbrsolver_gb300 import scenes

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _case(name):
    if name == "reference_main":
        return scenes.reference_main_scene()
    if name == "small_L6_R3":
        return scenes.small_scene()
    if name == "small_L4_R3T1_hertzian":
        wl = scenes.small_scene()
        wl.request.antenna = 1
        wl.request.tessellation = 4
        wl.request.max_transmission = 1
        return wl
    if name == "urban_L5_R3T2_rx1600_slab":
        return scenes.slab_walls(scenes.urban_scene(level=5, rx_pitch=25.0, max_reflection=3,
                                                    max_transmission=2), SLAB_WIDTHS)
    if name == "urban_L5_R6T1_rx100":
        return scenes.urban_scene(level=5, rx_pitch=100.0)
    if name == "urban_L4_R3T2_rx400":
        return scenes.urban_scene(level=4, rx_pitch=50.0, max_reflection=3, max_transmission=2)
    return scenes.request_variant(name)


CASES = ["reference_main", "small_L6_R3", "small_L4_R3T1_hertzian", "urban_L5_R6T1_rx100",
         "urban_L4_R3T2_rx400", "urban_L5_R3T2_rx1600_slab",
         # pattern, transmitter frame, power and Fresnel-switch variants
         "small_L5_R4T1_halfwave_rotated", "urban_L5_R3T1_rx1600_halfwave_rotated",
         "urban_L5_R3T1_rx1600_isotropic_nofresnel"]
# slab coefficients instead of infinite walls: ground 0.5 m, concrete walls
# 0.2 m, glass 0.01 m thick
SLAB_WIDTHS = (0.5, 0.2, 0.01)


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(built, name):
    g = np.load(os.path.join(GOLD, name + ".npz"))
    wl = _case(name)
    sc = orc.OracleScene.from_scene(wl.scene)
    out = orc.solve(sc, wl.request, wl.scene.materials)
    assert out["counts"]["segments"] == int(g["segments"])
    assert out["counts"]["captured"] == int(g["captured"])
    assert out["counts"]["corrected"] == int(g["corrected"])
    ref_paths = golden_paths(g)
    assert path_keys(out["paths"]) == path_keys(ref_paths)
    for p, q in zip(out["paths"], ref_paths):
        np.testing.assert_array_equal(p["points"], q["points"])
    # same host arithmetic; libm may differ in the last bit across machines
    np.testing.assert_allclose(out["field"], golden_field(g), rtol=1e-12, atol=1e-300)


def test_reference_main_pins_shipped_outputs():
    """The fixture generator checked the reference run against the outputs the
    reference ships (ElectricField.csv, RayPath.vtk); the oracle reproduces
    the CSV at its printed precision."""
    g = np.load(os.path.join(GOLD, "reference_main.npz"))
    assert bool(g["shipped_field_csv_match"]) and bool(g["shipped_raypath_pairs_match"])
    wl = scenes.reference_main_scene()
    out = orc.solve(orc.OracleScene.from_scene(wl.scene), wl.request, wl.scene.materials)
    f = out["field"]
    ours = np.stack([f.real, f.imag], -1).reshape(-1, 6)
    printed = np.vectorize(lambda x: float("%.6g" % x))(ours)
    np.testing.assert_array_equal(printed, g["shipped_field_csv"])
    assert len(out["paths"]) == 3133


@pytest.mark.parametrize("level", [0, 1, 2, 5])
def test_icosphere_bit_exact(built, level):
    ref = np.load(os.path.join(GOLD, f"icosphere_L{level}.npy"))
    np.testing.assert_array_equal(orc.icosphere(level), ref)
    assert len(ref) == 10 * 4 ** level + 2


@pytest.mark.parametrize("level", [6, 7, 8, 9, 10])
def test_icosphere_digests(built, level):
    """The launch directions of the benchmark levels, from the oracle and from
    the library (host code, no GPU), hash like the reference's
    (tests/golden/icosphere_digests.json)."""
    import hashlib
    import json

    from sbrsolver_gb300 import api
    ref = json.load(open(os.path.join(GOLD, "icosphere_digests.json")))[str(level)]
    for v in (orc.icosphere(level), api.GenerateRaysOnIcosahedron(level)):
        v = np.ascontiguousarray(v, "<f8")
        assert len(v) == ref["rays"] == 10 * 4 ** level + 2
        assert hashlib.sha256(v.tobytes()).hexdigest() == ref["sha256"]


def test_launch_directions_arguments(built):
    from sbrsolver_gb300 import _lib, api
    lib = _lib.load()
    n = C.c_longlong(0)
    assert lib.sbr_launch_directions(13, None, 0, C.byref(n)) == _lib.ERR_INVALID_ARG
    assert lib.sbr_launch_directions(2, None, 0, None) == _lib.ERR_INVALID_ARG
    assert lib.sbr_launch_directions(2, None, 0, C.byref(n)) == _lib.OK and n.value == 162
    small = np.zeros((161, 3))
    assert lib.sbr_launch_directions(2, small.ctypes.data_as(C.POINTER(C.c_double)), 161,
                                     C.byref(n)) == _lib.ERR_CAPACITY
    for lvl in (0, 1, 2, 5):
        np.testing.assert_array_equal(api.GenerateRaysOnIcosahedron(lvl),
                                      np.load(os.path.join(GOLD, f"icosphere_L{lvl}.npy")))


def test_scene_inputs_are_reproducible(tmp_path):
    """Fixture inputs are regenerated from seeds: the STL/material/receiver
    bytes must hash to what the fixture was made from."""
    import hashlib
    for name in CASES[1:]:
        g = np.load(os.path.join(GOLD, name + ".npz"))
        d = tmp_path / name
        scenes.write_oracle_case(_case(name), str(d))
        h = hashlib.sha256()
        for f in ("scene.stl", "trimat.txt", "rx.txt"):
            h.update((d / f).read_bytes())
        assert h.hexdigest() == str(g["inputs_sha256"]), name


def test_fresnel_sweep_pins():
    """RefCoeffTest reproduces the shipped coeff_test.csv magnitudes exactly;
    the shipped phases are exactly pi away (older sign convention)."""
    g = np.load(os.path.join(GOLD, "fresnel_sweep.npz"))
    ours, shipped = g["reference"], g["shipped"]
    np.testing.assert_array_equal(ours[:, [0, 1, 3]], shipped[:, [0, 1, 3]])
    d = np.abs(np.angle(np.exp(1j * (ours[:, [2, 4]] - shipped[:, [2, 4]]))))
    assert np.all(np.abs(d - np.pi) < 2e-5)
