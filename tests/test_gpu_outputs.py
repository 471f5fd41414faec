"""The reference's main() run through the drop-in API on the GPU
(Preprocessor.StlToGeometry -> BVH.ConstructBVH -> RTSolver.Init ->
ExecuteRayTracing -> Save*), writing ElectricField.csv, RayPath.vtk and
RxLocations.vtk byte for byte as the reference ships them."""
import hashlib
import json
import os

import numpy as np
import pytest

from sbrsolver_gb300 import api, scenes

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SHIPPED = json.load(open(os.path.join(GOLD, "shipped_outputs.json")))


def _sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def test_reference_main_outputs_byte_exact(built, tmp_path):
    wl = scenes.reference_main_scene()
    stl = str(tmp_path / "ground.stl")
    scenes.write_stl(wl.scene, stl)
    mesh = api.Preprocessor.StlToGeometry(stl)
    bvh = api.BVH()
    bvh.ConstructBVH(mesh)
    m = wl.scene.materials[0]
    mat = api.MaterialProperties(*m)
    rx = []
    api.Preprocessor.GenerateRXLine((0, 0, 3), (0, 3000, 3), 1, rx)
    np.testing.assert_array_equal(np.asarray(rx), wl.request.rx)
    q = wl.request
    solver = api.RTSolver(api.GlobalConfig(antennaType=q.antenna))
    assert solver.Init([mat], 1, bvh) == 0
    solver.ExecuteRayTracing(q.tx, np.asarray(q.tx_coord_sys).reshape(3, 3), q.max_reflection,
                             q.max_transmission, q.frequency, q.pt, q.use_fresnel, rx, mesh,
                             q.tessellation)
    for name, save in (("ElectricField.csv", solver.SaveFieldAsCsv),
                       ("RayPath.vtk", solver.SavePathsAsVtk),
                       ("RxLocations.vtk", solver.SaveReceiversAsVtk)):
        out = str(tmp_path / name)
        assert save(out)
        assert _sha(out) == SHIPPED[name]["sha256"], name
