"""Field precision modes on the large terrain scene (580,484 triangles,
half-wave 3.5 GHz, 8 reflections) with a receiver subset, through the C ABI:
the FP64 field equals the oracle's, the FP32 field (FP64 path length and
phase, compensated FP32 receiver sums) is within 1e-4 relative magnitude and
1e-3 rad, the FP32-phase mode is measured, every mode yields the identical
path set, and the error the library reports (field_check) agrees with the
host statistics."""
import numpy as np
import pytest

import oracle as orc
from helpers import field_close, max_rel_err, path_keys
from sbrsolver_gb300 import api, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def large():
    wl = scenes.large_scene(level=6)
    wl.request.rx = wl.request.rx[::100].copy()  # 500 of the 50,000 receivers
    ref = orc.solve(orc.OracleScene.from_scene(wl.scene), wl.request, wl.scene.materials)
    sc = api.DeviceScene.from_scene(wl.scene)
    yield wl, ref, sc
    sc.close()


def _solve(sc, wl, precision, check=False):
    return api.solve(sc, api.request_from_workload(wl.request, precision, stage_counts=True,
                                                   field_check=check))


def test_fp64_matches_oracle(built, large):
    wl, ref, sc = large
    res = _solve(sc, wl, "fp64")
    assert path_keys(res.paths) == path_keys(ref["paths"])
    for k in ("segments", "captured", "corrected", "paths"):
        assert res.counts[k] == ref["counts"][k], k
    assert res.counts["paths"] > 0
    assert max_rel_err(res.field, ref["field"]) < 1e-9
    assert res.field_error is None  # nothing to compare in FP64 mode


def test_fp32_within_tolerance_with_reported_error(built, large):
    wl, ref, sc = large
    res = _solve(sc, wl, "fp32", check=True)
    assert path_keys(res.paths) == path_keys(ref["paths"])
    assert not field_close(res.field, ref["field"])
    # the FP64 shadow is the FP64 field of the same paths
    assert max_rel_err(res.field_fp64, ref["field"]) < 1e-9
    st = api.field_error_stats(res.field, res.field_fp64)
    fe = res.field_error
    assert fe["components"] == st["components"] > 0
    assert fe["over_tolerance"] == st["over_tolerance"] == 0
    for k in ("rel_mag", "phase_rad", "rel_vec"):
        assert fe[f"max_{k}"] == pytest.approx(st[f"max_{k}"], rel=1e-9, abs=1e-15)


def test_fp32_phase_mode_is_measured(built, large):
    wl, ref, sc = large
    r32 = _solve(sc, wl, "fp32", check=True)
    rph = _solve(sc, wl, "fp32_phase", check=True)
    assert path_keys(rph.paths) == path_keys(ref["paths"])
    np.testing.assert_array_equal(rph.field_fp64, r32.field_fp64)
    st = api.field_error_stats(rph.field, rph.field_fp64)
    assert rph.field_error["max_phase_rad"] == pytest.approx(st["max_phase_rad"], rel=1e-9,
                                                             abs=1e-15)
    # an FP32 phase k*L (k = 73 rad/m, L up to ~1 km) is off by up to an FP32
    # ulp of k*L; the FP64-phase mode is not worse than it
    s32 = api.field_error_stats(r32.field, r32.field_fp64)
    assert s32["max_phase_rad"] <= max(st["max_phase_rad"], 1e-6)


def test_field_check_on_urban_batch(built):
    """field_check on a batch: per-request results each carry their error."""
    wl = scenes.urban_scene(level=4, rx_pitch=50.0, max_reflection=3, max_transmission=2)
    other = scenes.urban_scene(level=5, rx_pitch=100.0)
    other.request.tx = (100.0, 150.0, 25.0)
    sc = api.DeviceScene.from_scene(wl.scene)
    qs = [api.request_from_workload(w.request, "fp32", field_check=True) for w in (wl, other)]
    rb = api.solve(sc, qs)
    r0 = api.solve(sc, qs[0])
    n0 = len(wl.request.rx)
    np.testing.assert_array_equal(rb.field_fp64[:n0], r0.field_fp64)
    np.testing.assert_array_equal(rb.field[:n0], r0.field)
    st = api.field_error_stats(rb.field, rb.field_fp64)
    assert st["components"] >= 10 and st["over_tolerance"] == 0
    sc.close()


def test_mixed_precision_batch(built):
    """Each request in a batch keeps its own field precision."""
    wl = scenes.urban_scene(level=4, rx_pitch=50.0, max_reflection=3, max_transmission=2)
    sc = api.DeviceScene.from_scene(wl.scene)
    modes = ("fp64", "fp32", "fp32_phase", "fp64")
    qs = [api.request_from_workload(wl.request, m) for m in modes]
    rb = api.solve(sc, qs)
    n = len(wl.request.rx)
    for k, m in enumerate(modes):
        alone = api.solve(sc, api.request_from_workload(wl.request, m))
        np.testing.assert_array_equal(rb.field[k * n:(k + 1) * n], alone.field)
    assert not np.array_equal(rb.field[n:2 * n], rb.field[:n])  # FP32 differs in low bits
    sc.close()


@pytest.mark.parametrize("case", ["urban_L6_R6T1", "urban_L5_slab", "large_L7"])
def test_fp32_bound_holds_and_certifies(built, case):
    """The FP32 mode's stated per-receiver bound (sbr_result_field_bound)
    really bounds every component's error against the FP64 field of the same
    paths; receivers it could not certify were recomputed in FP64 (bound 0,
    bit-equal to the FP64 field); so every component is within 1e-4 / 1e-3
    rad.  The urban canyon at 28 GHz has receivers whose paths cancel to
    1e-4 of their sum, which FP32 cannot resolve: those are the escalated
    ones."""
    if case == "urban_L6_R6T1":
        wl = scenes.urban_scene(level=6, rx_pitch=10.0)
    elif case == "urban_L5_slab":
        wl = scenes.slab_walls(scenes.urban_scene(level=5, rx_pitch=25.0, max_reflection=3,
                                                  max_transmission=2), (0.5, 0.2, 0.01))
        wl.request.use_fresnel = False
    else:
        wl = scenes.large_scene(level=7)
        wl.request.rx = wl.request.rx[::25].copy()
    sc = api.DeviceScene.from_scene(wl.scene)
    res = api.solve(sc, api.request_from_workload(wl.request, "fp32", field_check=True),
                    with_paths=False)
    sc.close()
    b = res.field_bound
    assert b is not None and np.all(b >= 0)
    err = np.abs(res.field - res.field_fp64)
    assert np.all(err <= b[:, None] * (1 + 1e-9) + 1e-300)
    zero = b == 0
    np.testing.assert_array_equal(res.field[zero], res.field_fp64[zero])
    assert not field_close(res.field, res.field_fp64)
    with_field = np.abs(res.field_fp64).max(axis=1) > 0
    assert res.counts["fp64_field_receivers"] <= int((zero & with_field).sum())
    assert int((~zero).sum()) > 0  # FP32 certified a part of the receivers itself
    if case == "urban_L6_R6T1":
        assert res.counts["fp64_field_receivers"] > 0


def test_fp64_and_phase_study_bounds(built):
    wl = scenes.urban_scene(level=4, rx_pitch=50.0)
    sc = api.DeviceScene.from_scene(wl.scene)
    r64 = api.solve(sc, api.request_from_workload(wl.request, "fp64"), with_paths=False)
    rph = api.solve(sc, api.request_from_workload(wl.request, "fp32_phase"), with_paths=False)
    sc.close()
    assert np.all(r64.field_bound == 0)
    has = np.abs(rph.field).max(axis=1) > 0
    assert np.all(rph.field_bound[has] == -1)
