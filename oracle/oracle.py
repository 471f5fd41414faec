"""ctypes wrapper of the CPU restatement (TEST INFRASTRUCTURE: the oracle).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  It returns the same shapes as sbrsolver_gb300.api.solve so the
two can be compared directly.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")


class _Mat(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("frequency", "transmissionLoss", "reflectionLoss",
                                           "relPermittivityRe", "relPermittivityIm",
                                           "relConductivity", "width")]


class _Req(C.Structure):
    _fields_ = [("tx", C.c_double * 3), ("tx_coord_sys", C.c_double * 9),
                ("max_reflection", C.c_int), ("max_transmission", C.c_int),
                ("frequency", C.c_double), ("pt", C.c_double), ("use_fresnel", C.c_int),
                ("tessellation", C.c_int), ("antenna", C.c_int), ("n_rx", C.c_int),
                ("rx", C.POINTER(C.c_double)), ("n_materials", C.c_int),
                ("materials", C.POINTER(_Mat)), ("pattern", C.POINTER(C.c_float)),
                ("pat_nt", C.c_int), ("pat_np", C.c_int), ("pat_dt", C.c_double),
                ("pat_dp", C.c_double)]


class _Path(C.Structure):
    _fields_ = [("receiver", C.c_int), ("n_rays", C.c_int), ("launch", C.c_long),
                ("field", C.c_double * 6)]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} is not built; run python oracle/build.py")
        lib = C.CDLL(LIB_PATH)
        vp, I, P = C.c_void_p, C.c_int, C.POINTER
        lib.oracle_scene_from_triangles.argtypes = [I, P(C.c_float), P(C.c_float), P(vp)]
        lib.oracle_scene_set_materials.argtypes = [vp, P(I)]
        lib.oracle_scene_info.argtypes = [vp, P(I), P(I)]
        lib.oracle_scene_mesh_order.argtypes = [vp, P(I)]
        lib.oracle_scene_coplanar.argtypes = [vp, P(I)]
        lib.oracle_scene_destroy.argtypes = [vp]
        lib.oracle_scene_destroy.restype = None
        lib.oracle_icosphere.argtypes = [I, P(C.c_double), C.c_long]
        lib.oracle_solve.argtypes = [vp, P(_Req), I, P(vp)]
        lib.oracle_result_counts.argtypes = [vp] + [P(C.c_long)] * 5
        lib.oracle_result_counts.restype = None
        lib.oracle_result_copy.argtypes = [vp, P(C.c_double), P(_Path), P(C.c_long), P(I), P(I),
                                           P(I), P(C.c_double)]
        lib.oracle_result_copy.restype = None
        lib.oracle_result_destroy.argtypes = [vp]
        lib.oracle_result_destroy.restype = None
        _lib = lib
    return _lib


class OracleScene:
    def __init__(self, tri: np.ndarray, normal: np.ndarray, material_id: np.ndarray):
        lib = load()
        v = np.ascontiguousarray(tri, np.float32)
        n = np.ascontiguousarray(normal, np.float32)
        h = C.c_void_p()
        rc = lib.oracle_scene_from_triangles(len(v), v.ctypes.data_as(C.POINTER(C.c_float)),
                                             n.ctypes.data_as(C.POINTER(C.c_float)), C.byref(h))
        if rc:
            raise RuntimeError(f"oracle scene build failed ({rc})")
        ids = np.ascontiguousarray(material_id, np.int32)
        lib.oracle_scene_set_materials(h, ids.ctypes.data_as(C.POINTER(C.c_int)))
        self.h = h
        self.n = len(v)

    @classmethod
    def from_scene(cls, scene) -> "OracleScene":
        return cls(scene.tri, scene.normal, scene.material_id)

    def mesh_order(self) -> np.ndarray:
        out = np.zeros(self.n, np.int32)
        load().oracle_scene_mesh_order(self.h, out.ctypes.data_as(C.POINTER(C.c_int)))
        return out

    def coplanar_ids(self) -> np.ndarray:
        out = np.zeros(self.n, np.int32)
        load().oracle_scene_coplanar(self.h, out.ctypes.data_as(C.POINTER(C.c_int)))
        return out

    def __del__(self):
        try:
            load().oracle_scene_destroy(self.h)
        except Exception:
            pass


def icosphere(level: int) -> np.ndarray:
    n = 10 * 4 ** level + 2
    out = np.zeros(3 * n, np.float64)
    load().oracle_icosphere(level, out.ctypes.data_as(C.POINTER(C.c_double)), n)
    return out.reshape(n, 3)


def solve(scene: OracleScene, request, materials: Sequence, threads: int = 0,
          pattern=None) -> dict:
    """request: sbrsolver_gb300.scenes.Request; materials: MaterialProperties
    tuples; pattern (antenna 3 only): (table, d_theta, d_phi) with table an
    (n_theta, n_phi, 4) array of g_theta dB, arg_theta deg, g_phi dB, arg_phi
    deg.  Returns field (n_rx, 3) complex, counts and paths (receiver-major,
    then launch, then BFS order, as the reference enumerates them)."""
    lib = load()
    rx = np.ascontiguousarray(request.rx, np.float64).reshape(-1, 3)
    mats = (_Mat * len(materials))(*[_Mat(*m) for m in materials])
    q = _Req()
    for i in range(3):
        q.tx[i] = float(request.tx[i])
    for i in range(9):
        q.tx_coord_sys[i] = float(request.tx_coord_sys[i])
    q.max_reflection = request.max_reflection
    q.max_transmission = request.max_transmission
    q.frequency = request.frequency
    q.pt = request.pt
    q.use_fresnel = int(request.use_fresnel)
    q.tessellation = request.tessellation
    q.antenna = request.antenna
    q.n_rx = len(rx)
    q.rx = rx.ctypes.data_as(C.POINTER(C.c_double))
    q.n_materials = len(materials)
    q.materials = mats
    if pattern is not None:
        tab = np.ascontiguousarray(pattern[0], np.float32)
        q.pattern = tab.ctypes.data_as(C.POINTER(C.c_float))
        q.pat_nt, q.pat_np = int(tab.shape[0]), int(tab.shape[1])
        q.pat_dt, q.pat_dp = float(pattern[1]), float(pattern[2])
    h = C.c_void_p()
    rc = lib.oracle_solve(scene.h, C.byref(q), int(threads), C.byref(h))
    if rc:
        raise RuntimeError(f"oracle solve failed ({rc})")
    try:
        seg, cap, cor, npth, nray = (C.c_long(), C.c_long(), C.c_long(), C.c_long(), C.c_long())
        lib.oracle_result_counts(h, C.byref(seg), C.byref(cap), C.byref(cor), C.byref(npth),
                                 C.byref(nray))
        field = np.zeros(6 * len(rx), np.float64)
        P = (_Path * max(1, npth.value))()
        off = np.zeros(npth.value + 1, np.int64)
        nr = max(1, nray.value)
        tri = np.zeros(nr, np.int32)
        cop = np.zeros(nr, np.int32)
        kind = np.zeros(nr, np.int32)
        pts = np.zeros(6 * nr, np.float64)
        ip = C.POINTER(C.c_int)
        lib.oracle_result_copy(h, field.ctypes.data_as(C.POINTER(C.c_double)), P,
                               off.ctypes.data_as(C.POINTER(C.c_long)), tri.ctypes.data_as(ip),
                               cop.ctypes.data_as(ip), kind.ctypes.data_as(ip),
                               pts.ctypes.data_as(C.POINTER(C.c_double)))
        paths = []
        for i in range(npth.value):
            p = P[i]
            o, n = int(off[i]), int(p.n_rays)
            paths.append({"receiver": p.receiver, "launch": int(p.launch), "n_rays": n,
                          "tri": tri[o:o + n].tolist(), "cop": cop[o:o + n].tolist(),
                          "kind": kind[o:o + n].tolist(),
                          "points": pts[6 * o:6 * (o + n)].reshape(n, 6).copy(),
                          "field": np.array(p.field[:], np.float64)})
        return {"field": np.ascontiguousarray(field, np.float64).view(np.complex128).reshape(-1, 3),
                "counts": {"segments": seg.value, "captured": cap.value, "corrected": cor.value,
                           "paths": npth.value, "rays": nray.value,
                           "launches": 10 * 4 ** request.tessellation + 2},
                "paths": paths}
    finally:
        lib.oracle_result_destroy(h)
