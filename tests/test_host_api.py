"""Host-side mirror of the reference interface (no GPU)."""
import numpy as np
import pytest

from sbrsolver_gb300 import api, scenes


def test_generate_rx_line_matches_reference_main():
    out = []
    api.Preprocessor.GenerateRXLine((0, 0, 3), (0, 3000, 3), 1, out)
    assert len(out) == 3000
    np.testing.assert_array_equal(np.array(out), scenes.reference_main_scene().request.rx)


def test_generate_rx_plane_counts():
    out = []
    api.Preprocessor.GenerateRxPlane(-5, -5, 5, 5, 7, 1, out)
    assert len(out) == 121 and out[0] == (-5, -5, 7) and out[-1] == (5, 5, 7)


def test_stl_binary_and_ascii_read_alike(tmp_path):
    wl = scenes.small_scene()
    p = tmp_path / "s.stl"
    scenes.write_stl(wl.scene, str(p))
    m = api.Preprocessor.StlToGeometry(str(p))
    np.testing.assert_array_equal(m.vertices, wl.scene.tri)
    np.testing.assert_array_equal(m.normals, wl.scene.normal)
    a = tmp_path / "a.stl"
    with open(a, "w") as fh:
        fh.write("solid t\n")
        for v, n in zip(wl.scene.tri, wl.scene.normal):
            fh.write("facet normal %.9g %.9g %.9g\nouter loop\n" % tuple(n))
            for q in v:
                fh.write("vertex %.9g %.9g %.9g\n" % tuple(q))
            fh.write("endloop\nendfacet\n")
        fh.write("endsolid t\n")
    m2 = api.Preprocessor.StlToGeometry(str(a))
    np.testing.assert_array_equal(m2.vertices, wl.scene.tri)


def test_scene_generators_are_seeded():
    a, b = scenes.urban_scene(), scenes.urban_scene()
    np.testing.assert_array_equal(a.scene.tri, b.scene.tri)
    assert a.scene.n_tri == 4802 and scenes.small_scene().scene.n_tri == 122
    assert len(a.request.rx) == 10000 and 10 * 4 ** a.request.tessellation + 2 == 2621442


def test_pcg32_reference_values():
    # PCG32 demo stream: seed 42, sequence 54 (O'Neill's pcg32-demo output)
    g = scenes.PCG32(42, 54)
    assert [g.next_u32() for _ in range(3)] == [0xa15c02b7, 0x7b47f409, 0xba1d3330]


def test_field_error_stats_definitions():
    from sbrsolver_gb300 import api
    ref = np.array([[1 + 0j, 1e-9 + 0j, 0j], [0j, 0j, 0j], [2j, 1 + 1j, 0.5 + 0j]])
    a = ref.copy()
    a[0, 0] = 1.00005 * np.exp(2e-3j)   # 5e-5 magnitude, 2e-3 rad phase
    a[2, 1] = (1 + 1j) * 1.0002         # 2e-4 magnitude
    st = api.field_error_stats(a, ref)
    # components above 1e-6 of their receiver's largest: 1 + 3; empty receiver skipped
    assert st["components"] == 4 and st["receivers_with_field"] == 2
    assert st["max_rel_mag"] == pytest.approx(2e-4, rel=1e-6)
    assert st["max_phase_rad"] == pytest.approx(2e-3, rel=1e-6)
    assert st["over_tolerance"] == 2
    assert api.field_error_stats(ref, ref)["max_rel_vec"] == 0.0


def test_same_path_set():
    from sbrsolver_gb300 import api
    a = {k: np.arange(4) for k in ("request", "receiver", "launch", "heap", "n_rays")}
    a.update(tri=np.arange(7), cop=np.arange(7), kind=np.zeros(7))
    b = {k: v.copy() for k, v in a.items()}
    assert api.same_path_set(a, b)
    b["tri"][3] = 99
    assert not api.same_path_set(a, b)
    assert api.same_path_set([], [])
