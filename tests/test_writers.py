"""Output writers (no GPU): from the reference_main fixture (the reference's
own run of its main() scene) the library writes the field CSV, the ray-path
and receiver VTK files and the level-3 launch-ray VTK byte for byte as the
reference ships them (sha256 in tests/golden/shipped_outputs.json)."""
import ctypes as C
import hashlib
import json
import os

import numpy as np
import pytest

from helpers import golden_paths
from sbrsolver_gb300 import _lib, api, scenes

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SHIPPED = json.load(open(os.path.join(GOLD, "shipped_outputs.json")))
D = C.POINTER(C.c_double)


def _sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


@pytest.fixture(scope="module")
def main_run():
    g = np.load(os.path.join(GOLD, "reference_main.npz"))
    rx = np.ascontiguousarray(scenes.reference_main_scene().request.rx, np.float64)
    field = np.ascontiguousarray(g["field"], np.float64)
    paths = golden_paths(g)
    # the fixture lists each receiver's paths in launch then breadth-first order
    for i, p in enumerate(paths):
        p.update(request=0, heap=i)
    return rx, field, paths


def test_field_csv_byte_exact(built, main_run, tmp_path):
    rx, field, _ = main_run
    out = str(tmp_path / "ElectricField.csv")
    _lib.check(_lib.load().sbr_write_field_csv(out.encode(), rx.ctypes.data_as(D), len(rx),
                                               field.ctypes.data_as(D)))
    assert _sha(out) == SHIPPED["ElectricField.csv"]["sha256"]


def test_receivers_vtk_byte_exact(built, main_run, tmp_path):
    rx, field, _ = main_run
    out = str(tmp_path / "RxLocations.vtk")
    _lib.check(_lib.load().sbr_write_receivers_vtk(out.encode(), rx.ctypes.data_as(D), len(rx),
                                                   field.ctypes.data_as(D)))
    assert _sha(out) == SHIPPED["RxLocations.vtk"]["sha256"]


def test_paths_vtk_byte_exact(built, main_run, tmp_path):
    rx, field, paths = main_run
    P, pts = api._path_structs(paths)
    out = str(tmp_path / "RayPath.vtk")
    _lib.check(_lib.load().sbr_write_paths_vtk(out.encode(), P, len(P), pts.ctypes.data_as(D),
                                               field.ctypes.data_as(D), len(rx)))
    assert _sha(out) == SHIPPED["RayPath.vtk"]["sha256"]


def test_launch_rays_vtk_byte_exact(built, tmp_path):
    out = str(tmp_path / "Icosahedron.vtk")
    api.RTSolver().SaveIcosahedronAsVtk(out, (0.0, 0.0, 5.0), 3)
    assert _sha(out) == SHIPPED["Icosahedron.vtk"]["sha256"]


def test_writer_errors(built, main_run, tmp_path):
    lib = _lib.load()
    rx, field, paths = main_run
    assert lib.sbr_write_field_csv(b"/nonexistent/dir/f.csv", rx.ctypes.data_as(D), len(rx),
                                   field.ctypes.data_as(D)) == _lib.ERR_IO
    P, pts = api._path_structs(paths[:3])
    P[1].receiver = len(rx)  # out of range
    st = lib.sbr_write_paths_vtk(str(tmp_path / "p.vtk").encode(), P, 3, pts.ctypes.data_as(D),
                                 field.ctypes.data_as(D), len(rx))
    assert st == _lib.ERR_INVALID_ARG
    assert b"out of bounds" in lib.sbr_last_error()
    assert lib.sbr_write_launch_rays_vtk(b"x.vtk", None, 3) == _lib.ERR_INVALID_ARG
    # an empty run writes valid, empty files
    out = str(tmp_path / "empty.csv")
    _lib.check(lib.sbr_write_field_csv(out.encode(), None, 0, None))
    assert open(out).read() == "X,Y,Z,Ex,Ey,Ez\n"
