"""Host-side mirror of the reference's interface for the SBR path.

Names, argument order and argument meaning follow the reference
(SBRSolver_rev2/): ``Preprocessor`` (Preprocessor.h:18-75), ``BVH``
(BVH/BVH.h:13-37), ``RTSolver`` (RTSolver.h:18-83), ``FieldCompute``
(FieldCompute.h:9-94), ``GlobalConfig`` (GlobalConfig.h:5-7, given the
settings the reference hard-codes) and ``MaterialProperties``
(common/DataStructures.h:20-28).  The work runs on the GPU through the C ABI
(include/sbr.h); nothing here computes propagation on the CPU.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _lib
from .scenes import Scene, Request as WorkRequest


@dataclass
class MaterialProperties:
    frequency: float = 0.0
    transmissionLoss: float = 0.0
    reflectionLoss: float = 0.0
    relPermittivityRe: float = 1.0
    relPermittivityIm: float = 0.0
    relConductivity: float = 0.0
    # Wall thickness (m) for the slab coefficients used when useFresnelCoeff
    # is false (FieldCompute.cpp:255-262,284-291).  The reference always
    # passes 0 (FieldCompute.cpp:131,138): reflection 0, transmission 1.
    width: float = 0.0

    def as_c(self) -> _lib.Material:
        return _lib.Material(self.frequency, self.transmissionLoss, self.reflectionLoss,
                             self.relPermittivityRe, self.relPermittivityIm, self.relConductivity,
                             self.width)


@dataclass
class GlobalConfig:
    """Settings the reference hard-codes.  antennaType 1 (Hertzian) is what
    FieldCompute.cpp:117 always uses; fieldPrecision 'fp64' reproduces the
    reference arithmetic, 'fp32' computes per-path rotations and Fresnel
    coefficients in FP32 (FP64 length and phase, compensated FP32 sums)."""

    antennaType: int = 1
    fieldPrecision: str = "fp64"
    pattern: Optional["AntennaPattern"] = None  # antennaType 3 (tabulated)


@dataclass
class Mesh:
    """The reference's std::vector<Triangle*>: float vertices and facet
    normals in file order, per-triangle material ids (Triangle::materialId,
    default 0)."""

    vertices: np.ndarray   # (n, 3, 3) float32
    normals: np.ndarray    # (n, 3) float32
    materialId: np.ndarray  # (n,) int32

    def __len__(self) -> int:
        return int(self.vertices.shape[0])


class Preprocessor:
    """Namespace of free functions (Preprocessor.h:18-75)."""

    @staticmethod
    def StlToGeometry(fileName: str, output: Optional[list] = None, saveEdges: bool = False,
                      saveFaces: bool = False, dataDir: str = "") -> Mesh:
        """Preprocessor::StlToGeometry (Preprocessor.cpp:69-114): the facets
        of a binary or ASCII STL in file order (read by the library's reader,
        the one sbr_scene_create_from_stl uses)."""
        lib, n = _lib.load(), C.c_int()
        _lib.check(lib.sbr_stl_read(os.fsencode(fileName), C.byref(n), None, None))
        vv = np.zeros((n.value, 3, 3), np.float32)
        nn = np.zeros((n.value, 3), np.float32)
        fp = C.POINTER(C.c_float)
        _lib.check(lib.sbr_stl_read(os.fsencode(fileName), C.byref(n), vv.ctypes.data_as(fp),
                                    nn.ctypes.data_as(fp)))
        mesh = Mesh(vv, nn, np.zeros(len(vv), np.int32))
        if output is not None:
            output.append(mesh)
        return mesh

    @staticmethod
    def GenerateRxPlane(xMin, yMin, xMax, yMax, height, resolution, output: list) -> None:
        """Preprocessor::GenerateRxPlane (Preprocessor.cpp:254-268)."""
        lib, n = _lib.load(), C.c_int()
        args = [float(a) for a in (xMin, yMin, xMax, yMax, height, resolution)]
        _lib.check(lib.sbr_generate_rx_plane(*args, None, 0, C.byref(n)))
        out = np.zeros(3 * n.value, np.float64)
        _lib.check(lib.sbr_generate_rx_plane(*args, _dp(out), n.value, C.byref(n)))
        output.extend(map(tuple, out.reshape(-1, 3).tolist()))

    @staticmethod
    def GenerateRXLine(start, end, resolution, output: list) -> None:
        """Preprocessor::GenerateRXLine (Preprocessor.cpp:270-284)."""
        lib, n = _lib.load(), C.c_int()
        s = np.ascontiguousarray(np.asarray(start, np.float64).reshape(3))
        e = np.ascontiguousarray(np.asarray(end, np.float64).reshape(3))
        _lib.check(lib.sbr_generate_rx_line(_dp(s), _dp(e), float(resolution), None, 0,
                                            C.byref(n)))
        out = np.zeros(3 * n.value, np.float64)
        _lib.check(lib.sbr_generate_rx_line(_dp(s), _dp(e), float(resolution), _dp(out), n.value,
                                            C.byref(n)))
        output.extend(map(tuple, out.reshape(-1, 3).tolist()))

    @staticmethod
    def ReadPatternFile(fileName: str, output: dict) -> bool:
        """Preprocessor::ReadPatternFile (Preprocessor.cpp:3-35): every line of
        six numbers becomes output[(theta, phi)] = (g_theta, arg_theta, g_phi,
        arg_phi) as float32 values; other lines are skipped."""
        try:
            with open(fileName) as fh:
                for line in fh:
                    t = line.split()
                    if len(t) != 6:
                        continue
                    try:
                        v = [float(np.float32(x)) for x in t]
                    except ValueError:
                        continue
                    output[(v[0], v[1])] = tuple(v[2:])
            return True
        except OSError:
            return False

    @staticmethod
    def ReadLocationFile(fileName: str, output: list) -> bool:
        try:
            with open(fileName) as fh:
                for line in fh:
                    t = line.split()
                    if len(t) == 3:
                        try:
                            output.append(tuple(float(x) for x in t))
                        except ValueError:
                            continue
            return True
        except OSError:
            return False


class BVH:
    """BVH<Triangle> (BVH/BVH.h:13-37).  The SAH build runs inside the scene
    upload (sbr_scene_create); ConstructBVH records the mesh, and, like the
    reference, the order it leaves the caller's triangle vector in is the one
    image correction and the field stage index by triangle id."""

    def __init__(self):
        self.mesh: Optional[Mesh] = None

    def ConstructBVH(self, objects: Mesh) -> None:
        self.mesh = objects


class DeviceScene:
    """Resident scene (triangles, BVH, materials) on the GPU."""

    def __init__(self, mesh: Mesh, materials: Sequence[MaterialProperties],
                 host_prep: bool = False):
        """host_prep: build every table on the host (SBR_SCENE_HOST_PREP)
        instead of the coplanar groups, frames and search BVH on the GPU."""
        lib = _lib.load()
        mats = (_lib.Material * len(materials))(*[m.as_c() for m in materials])
        v = np.ascontiguousarray(mesh.vertices, np.float32)
        n = np.ascontiguousarray(mesh.normals, np.float32)
        ids = np.ascontiguousarray(mesh.materialId, np.int32)
        h = C.c_void_p()
        _lib.check(lib.sbr_scene_create_ex(
            len(mesh), v.ctypes.data_as(C.POINTER(C.c_float)),
            n.ctypes.data_as(C.POINTER(C.c_float)), ids.ctypes.data_as(C.POINTER(C.c_int)),
            mats, len(materials), 1 if host_prep else 0, C.byref(h)))
        self.handle = h
        self.n_triangles = len(mesh)
        self._lib = lib

    @classmethod
    def from_scene(cls, scene: Scene, host_prep: bool = False) -> "DeviceScene":
        mats = [MaterialProperties(*m) for m in scene.materials]
        return cls(Mesh(scene.tri, scene.normal, scene.material_id), mats, host_prep)

    def triangle_frames(self) -> tuple:
        """(frames (n, 3, 3), boxes (n, 6), centres (n, 3)) by triangle id."""
        n = self.n_triangles
        f, b, c = np.zeros((n, 3, 3)), np.zeros((n, 6)), np.zeros((n, 3))
        dp = C.POINTER(C.c_double)
        _lib.check(self._lib.sbr_scene_triangle_frames(self.handle, f.ctypes.data_as(dp),
                                                       b.ctypes.data_as(dp), c.ctypes.data_as(dp)))
        return f, b, c

    def search_bvh(self) -> dict:
        """The search BVH: nodes (raw 56-byte records as int32 words), the
        leaf order (depth-first ranks) and the depth."""
        nn, md = C.c_int(0), C.c_int(0)
        _lib.check(self._lib.sbr_scene_search_bvh(self.handle, C.byref(nn), C.byref(md), None, None))
        words = np.zeros(14 * nn.value, np.int32)
        order = np.zeros(self.n_triangles, np.int32)
        _lib.check(self._lib.sbr_scene_search_bvh(
            self.handle, C.byref(nn), C.byref(md), words.ctypes.data_as(C.POINTER(C.c_float)),
            order.ctypes.data_as(C.POINTER(C.c_int))))
        return {"nodes": words.reshape(-1, 14), "order": order, "max_depth": md.value}

    def reference_bvh(self) -> dict:
        """The reference BVH in depth-first order: node boxes (n, 6), links
        (n, 6: child 0, child 1, first, count, parent, depth), the leaves'
        triangle ids in visit order, and the depth."""
        nn, md = C.c_int(0), C.c_int(0)
        _lib.check(self._lib.sbr_scene_reference_bvh(self.handle, C.byref(nn), C.byref(md), None,
                                                     None, None))
        boxes = np.zeros(6 * nn.value, np.float64)
        links = np.zeros(6 * nn.value, np.int32)
        order = np.zeros(self.n_triangles, np.int32)
        ip = C.POINTER(C.c_int)
        _lib.check(self._lib.sbr_scene_reference_bvh(
            self.handle, C.byref(nn), C.byref(md), boxes.ctypes.data_as(C.POINTER(C.c_double)),
            links.ctypes.data_as(ip), order.ctypes.data_as(ip)))
        return {"boxes": boxes.reshape(-1, 6), "links": links.reshape(-1, 6), "order": order,
                "max_depth": md.value}

    def info(self) -> _lib.SceneInfo:
        out = _lib.SceneInfo()
        _lib.check(self._lib.sbr_scene_info_get(self.handle, C.byref(out)))
        return out

    def mesh_order(self) -> np.ndarray:
        out = np.zeros(self.n_triangles, np.int32)
        _lib.check(self._lib.sbr_scene_mesh_order(self.handle, out.ctypes.data_as(C.POINTER(C.c_int))))
        return out

    def set_mesh_order(self, order: np.ndarray) -> None:
        o = np.ascontiguousarray(order, np.int32)
        _lib.check(self._lib.sbr_scene_set_mesh_order(self.handle, o.ctypes.data_as(C.POINTER(C.c_int))))

    def coplanar_ids(self) -> np.ndarray:
        out = np.zeros(self.n_triangles, np.int32)
        _lib.check(self._lib.sbr_scene_coplanar_ids(self.handle, out.ctypes.data_as(C.POINTER(C.c_int))))
        return out

    def set_tuning(self, **shapes) -> None:
        """The scene's default launch shapes (sbr_tuning field names; 0 or
        absent = the library default)."""
        t = _lib.Tuning(**{k: int(v) for k, v in shapes.items()})
        _lib.check(self._lib.sbr_scene_set_tuning(self.handle, C.byref(t)))

    def tuning(self, requests=None) -> dict:
        """The launch shapes a solve of `requests` (a request tuple or a list
        of them; None = the scene default) would use, defaults filled in."""
        arr, n = _request_array(requests)
        out = _lib.Tuning()
        _lib.check(self._lib.sbr_scene_get_tuning(self.handle, arr, n, C.byref(out)))
        return {k: int(getattr(out, k)) for k, _ in _lib.Tuning._fields_}

    def autotune(self, requests, rounds: int = 1) -> dict:
        """Runs the library's autotuner on this batch (sbr_autotune) and
        returns the chosen shapes plus the batch's device time with them."""
        arr, n = _request_array(requests)
        out, ms = _lib.Tuning(), C.c_double()
        _lib.check(self._lib.sbr_autotune(self.handle, arr, n, int(rounds), C.byref(out),
                                          C.byref(ms)))
        d = {k: int(getattr(out, k)) for k, _ in _lib.Tuning._fields_}
        d["device_ms"] = ms.value
        return d

    def close(self) -> None:
        if self.handle:
            self._lib.sbr_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _request_array(requests):
    """(sbr_request array, count) from None, one request tuple or a list."""
    if requests is None:
        return None, 0
    if isinstance(requests, tuple) and isinstance(requests[0], _lib.Request):
        requests = [requests]
    return (_lib.Request * len(requests))(*[r[0] for r in requests]), len(requests)


@dataclass
class Result:
    field: np.ndarray          # (n_rx, 3) complex128
    counts: dict
    timing: dict
    paths: object = field(default_factory=list)  # list of dicts, or dict of arrays
    # requests with field_check: FP64 field of the same paths and the error of `field`
    field_fp64: Optional[np.ndarray] = None
    field_error: Optional[dict] = None
    # per receiver: bound on each component's absolute error (0 = FP64 arithmetic,
    # -1 = none: the FP32-phase study mode); sbr_result_field_bound
    field_bound: Optional[np.ndarray] = None


def make_request(tx, tx_coord_sys, max_reflection, max_transmission, frequency, pt, use_fresnel,
                 rx: np.ndarray, tessellation: int, antenna: int = 1,
                 precision: str = "fp64", stage_counts: bool = False,
                 field_check: bool = False, pattern: Optional[AntennaPattern] = None) -> tuple:
    rx = np.ascontiguousarray(rx, np.float64).reshape(-1, 3)
    q = _lib.Request()
    for i in range(3):
        q.tx[i] = float(tx[i])
    cs = np.asarray(tx_coord_sys, np.float64).reshape(9)
    for i in range(9):
        q.tx_coord_sys[i] = float(cs[i])
    q.max_reflection = int(max_reflection)
    q.max_transmission = int(max_transmission)
    q.frequency = float(frequency)
    q.pt = float(pt)
    q.use_fresnel = 1 if use_fresnel else 0
    q.tessellation = int(tessellation)
    q.antenna = int(antenna)
    q.field_precision = {"fp64": 0, "fp32": 1, "fp32_phase": 2}[precision]
    q.n_rx = int(rx.shape[0])
    q.rx = rx.ctypes.data_as(C.POINTER(C.c_double))
    q.rx_on_device = 0
    q.stage_counts = 1 if stage_counts else 0
    q.field_check = 1 if field_check else 0
    q.pattern = pattern.handle.value if pattern is not None else None
    return (q, rx, pattern) if pattern is not None else (q, rx)  # keep rx alive with the request


def request_from_workload(req: WorkRequest, precision: str = "fp64",
                          stage_counts: bool = False, field_check: bool = False) -> tuple:
    return make_request(req.tx, req.tx_coord_sys, req.max_reflection, req.max_transmission,
                        req.frequency, req.pt, req.use_fresnel, req.rx, req.tessellation,
                        req.antenna, precision, stage_counts, field_check)


def solve(scene: DeviceScene, requests, with_paths=True) -> Result:
    """Runs one or more requests (a batch) and returns fields, counts and paths
    (a list of per-path dicts, or with with_paths="arrays" one dict of flat
    arrays: per-path request/receiver/launch/heap/ray_offset/n_rays and
    per-ray tri/cop/kind/points)."""
    lib = _lib.load()
    if isinstance(requests, tuple) and isinstance(requests[0], _lib.Request):
        requests = [requests]  # one (request, receiver array[, pattern]) tuple
    arr = (_lib.Request * len(requests))(*[r[0] for r in requests])
    h = C.c_void_p()
    _lib.check(lib.sbr_solve_batch(scene.handle, arr, len(requests), C.byref(h)))
    return _collect(h, sum(r[0].n_rx for r in requests), with_paths)


_PATH_DTYPE = None


def _path_dtype():
    """numpy's structured dtype of sbr_path (formed once)."""
    global _PATH_DTYPE
    if _PATH_DTYPE is None:
        _PATH_DTYPE = np.ctypeslib.as_array((_lib.Path * 1)()).dtype
    return _PATH_DTYPE


def _collect(h, n_rx: int, with_paths: bool) -> Result:
    """Reads an sbr_result into a Result and destroys it."""
    lib = _lib.load()
    try:
        cnt = _lib.Counts()
        _lib.check(lib.sbr_result_counts(h, C.byref(cnt)))
        f = np.zeros(6 * n_rx, np.float64)
        if n_rx:
            _lib.check(lib.sbr_result_field(h, f.ctypes.data_as(C.POINTER(C.c_double))))
        tm = _lib.Timing()
        _lib.check(lib.sbr_result_timing(h, C.byref(tm)))
        counts = {k: int(getattr(cnt, k)) for k, _ in _lib.Counts._fields_}
        timing = {k: float(getattr(tm, k)) for k, _ in _lib.Timing._fields_}
        paths = []
        if with_paths and cnt.paths:
            P = (_lib.Path * cnt.paths)()
            nr = max(1, cnt.rays)
            tri = np.zeros(nr, np.int32)
            cop = np.zeros(nr, np.int32)
            kind = np.zeros(nr, np.int32)
            pts = np.zeros(6 * nr, np.float64)
            ip = C.POINTER(C.c_int)
            _lib.check(lib.sbr_result_paths(h, P, tri.ctypes.data_as(ip), cop.ctypes.data_as(ip),
                                            kind.ctypes.data_as(ip),
                                            pts.ctypes.data_as(C.POINTER(C.c_double))))
            # the whole path set as flat arrays (cheap at 1e5-1e6 paths)
            A = np.frombuffer(P, dtype=_path_dtype())
            arrays = {k: np.array(A[k]) for k in ("request", "receiver", "launch", "heap",
                                                  "ray_offset", "n_rays", "field", "near_edge")}
            arrays.update(tri=tri[:cnt.rays], cop=cop[:cnt.rays], kind=kind[:cnt.rays],
                          points=pts[:6 * cnt.rays].reshape(-1, 6))
            if with_paths == "arrays":
                paths = arrays
            else:  # one dict per path, sliced from the flat arrays
                cols = {k: arrays[k].tolist() for k in ("request", "receiver", "launch", "heap",
                                                        "ray_offset", "n_rays", "near_edge")}
                tl, cl, kl = (arrays[k].tolist() for k in ("tri", "cop", "kind"))
                pts6, fld = arrays["points"], arrays["field"]
                for i in range(int(cnt.paths)):
                    o, n = cols["ray_offset"][i], cols["n_rays"][i]
                    paths.append({
                        "request": cols["request"][i], "receiver": cols["receiver"][i],
                        "launch": cols["launch"][i], "heap": cols["heap"][i], "n_rays": n,
                        "tri": tl[o:o + n], "cop": cl[o:o + n], "kind": kl[o:o + n],
                        "points": pts6[o:o + n], "field": fld[i],  # views
                        "near_edge": cols["near_edge"][i]})
        field_c = f.view(np.complex128).reshape(-1, 3)  # exact, inf stays inf
        res = Result(field_c, counts, timing, paths)
        if n_rx:
            fb = np.zeros(n_rx, np.float64)
            if lib.sbr_result_field_bound(h, fb.ctypes.data_as(C.POINTER(C.c_double))) == 0:
                res.field_bound = fb
        fe = _lib.FieldError()
        if lib.sbr_result_field_error(h, C.byref(fe)) == 0:
            res.field_error = {k: getattr(fe, k) for k, _ in _lib.FieldError._fields_}
            f64 = np.zeros(6 * n_rx, np.float64)
            if n_rx:
                _lib.check(lib.sbr_result_field_fp64(h, f64.ctypes.data_as(C.POINTER(C.c_double))))
            res.field_fp64 = f64.view(np.complex128).reshape(-1, 3)
        return res
    finally:
        lib.sbr_result_destroy(h)


def field_error_stats(field: np.ndarray, reference: np.ndarray, floor: float = 1e-6,
                      rel_tol: float = 1e-4, phase_tol: float = 1e-3) -> dict:
    """Error of a received field against a reference field (both (n_rx, 3)
    complex), over the components whose reference magnitude exceeds `floor`
    times the receiver's largest component (the ones that carry a phase):
    relative magnitude error ||E|-|E_ref||/|E_ref|, phase error |arg(E/E_ref)|
    and relative vector error |E-E_ref|/|E_ref| (max, median, 99th percentile),
    plus how many components fall outside rel_tol / phase_tol."""
    a = np.asarray(field).reshape(-1, 3)
    b = np.asarray(reference).reshape(-1, 3)
    mb = np.abs(b)
    scale = mb.max(axis=1, keepdims=True) if len(b) else np.zeros((0, 1))
    m = (mb > floor * scale) & (scale > 0)
    x, y, my = a[m], b[m], mb[m]
    out = {"components": int(m.sum()), "receivers": int(len(b)),
           "receivers_with_field": int((scale[:, 0] > 0).sum()) if len(b) else 0}
    if not len(y):
        return out
    rel_mag = np.abs(np.abs(x) - my) / my
    phase = np.abs(np.angle(x * np.conj(y)))
    rel_vec = np.abs(x - y) / my
    for name, v in (("rel_mag", rel_mag), ("phase_rad", phase), ("rel_vec", rel_vec)):
        out[f"max_{name}"] = float(v.max())
        out[f"median_{name}"] = float(np.median(v))
        out[f"p99_{name}"] = float(np.percentile(v, 99))
    out["over_tolerance"] = int(((rel_mag > rel_tol) | (phase > phase_tol)).sum())
    return out


def same_path_set(a: dict, b: dict) -> bool:
    """Two path sets (solve(..., with_paths="arrays")) are identical: same
    receivers, launches, BFS positions, ray counts and facet / coplanar /
    interaction sequences, in the same order."""
    keys = ("request", "receiver", "launch", "heap", "n_rays", "tri", "cop", "kind")
    if isinstance(a, list) or isinstance(b, list):
        return (not a) and (not b)
    return all(np.array_equal(a[k], b[k]) for k in keys)


class Server:
    """Request server over resident scenes (sbr_server_*): `slots` solves at
    a time, admitted in arrival order by an HBM budget, overlapping on the GPU."""

    def __init__(self, scenes: Sequence[DeviceScene], slots: int = 4, hbm_budget: int = 0):
        lib = _lib.load()
        arr = (C.c_void_p * len(scenes))(*[s.handle.value for s in scenes])
        h = C.c_void_p()
        _lib.check(lib.sbr_server_create(arr, len(scenes), int(slots), int(hbm_budget), C.byref(h)))
        self.handle = h
        self._lib = lib
        self._nrx = {}

    def set_policy(self, batch_bytes: int = 2 << 30, max_batch: int = 64,
                   aging_bytes_per_s: float = 16e9, max_large: int = 0) -> None:
        """Batching, priority and large-request concurrency policy
        (sbr_server_set_policy)."""
        _lib.check(self._lib.sbr_server_set_policy(self.handle, int(batch_bytes), int(max_batch),
                                                   float(aging_bytes_per_s), int(max_large)))

    def submit(self, scene: int, request: tuple, tag: int) -> None:
        self._nrx[int(tag)] = request[0].n_rx
        _lib.check(self._lib.sbr_server_submit(self.handle, int(scene), C.byref(request[0]), int(tag)))

    def poll(self, max_items: int = 64, timeout_ms: int = 50, with_paths: bool = False) -> list:
        buf = (_lib.Completion * max_items)()
        n = C.c_int()
        _lib.check(self._lib.sbr_server_poll(self.handle, buf, max_items, C.byref(n), int(timeout_ms)))
        out = []
        for c in buf[:n.value]:
            item = {"tag": int(c.tag), "status": int(c.status), "scene": int(c.scene),
                    "queue_ms": c.queue_ms, "latency_ms": c.latency_ms, "device_ms": c.device_ms,
                    "counts": {k: int(getattr(c.counts, k)) for k, _ in _lib.Counts._fields_},
                    "result": None}
            if c.result:
                item["result"] = _collect(C.c_void_p(c.result), self._nrx.get(int(c.tag), 0),
                                          with_paths)
            out.append(item)
        return out

    def close(self) -> None:
        if self.handle:
            self._lib.sbr_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class AntennaPattern:
    """Tabulated antenna pattern (sbr_pattern_*): the TXPattern.dat grid the
    reference reads with Preprocessor::ReadPatternFile, applied by antenna
    type 3 as E_theta, E_phi = sqrt(60 Pt) 10^(g/20) e^(j arg) (g in dB, arg
    in degrees, bilinear on the grid).  The table lives on the current GPU."""

    def __init__(self, handle):
        self.handle = handle

    @classmethod
    def read(cls, path: str) -> "AntennaPattern":
        h = C.c_void_p()
        _lib.check(_lib.load().sbr_pattern_read(os.fsencode(path), C.byref(h)))
        return cls(h)

    @classmethod
    def from_table(cls, gain_phase: np.ndarray, d_theta: float, d_phi: float) -> "AntennaPattern":
        """gain_phase: (n_theta, n_phi, 4) of g_theta, arg_theta, g_phi, arg_phi."""
        t = np.ascontiguousarray(gain_phase, np.float32)
        h = C.c_void_p()
        _lib.check(_lib.load().sbr_pattern_create(t.shape[0], t.shape[1], float(d_theta),
                                                  float(d_phi),
                                                  t.ctypes.data_as(C.POINTER(C.c_float)),
                                                  C.byref(h)))
        return cls(h)

    def info(self) -> tuple:
        nt, npp, dt, dp = C.c_int(), C.c_int(), C.c_double(), C.c_double()
        _lib.check(_lib.load().sbr_pattern_info(self.handle, C.byref(nt), C.byref(npp),
                                                C.byref(dt), C.byref(dp)))
        return nt.value, npp.value, dt.value, dp.value

    def close(self) -> None:
        if self.handle:
            _lib.load().sbr_pattern_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_pattern_file(path: str, gain_phase: np.ndarray, d_theta: float, d_phi: float) -> None:
    """Writes a table in the TXPattern.dat layout (data/TXPattern.dat: a title
    line, the grid line, then theta phi g_theta arg_theta g_phi arg_phi)."""
    t = np.asarray(gain_phase, np.float64)
    with open(path, "w") as fh:
        fh.write("Transmitter (theta, phi, g_theta, arg_theta, g_phi, arg_phi)\n")
        fh.write(f"{t.shape[0]} {t.shape[1]} {d_theta:g} {d_phi:g}\n")
        for i in range(t.shape[0]):
            for j in range(t.shape[1]):
                g = t[i, j]
                fh.write(f"{i * d_theta:g} {j * d_phi:g} {g[0]:.6g} {g[1]:.6g} {g[2]:.6g} {g[3]:.6g}\n")


def GenerateRaysOnIcosahedron(tessellation: int, origin=(0.0, 0.0, 0.0)) -> np.ndarray:
    """The unit launch directions of an icosahedron level, (10*4^L + 2, 3), in
    the reference's vertex order (Icosahedron.cpp:80-109; like the
    reference, the origin does not change them): sbr_launch_directions."""
    lib = _lib.load()
    n = C.c_longlong(0)
    _lib.check(lib.sbr_launch_directions(int(tessellation), None, 0, C.byref(n)))
    out = np.zeros((n.value, 3), np.float64)
    _lib.check(lib.sbr_launch_directions(int(tessellation), _dp(out), n.value, C.byref(n)))
    return out


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _path_structs(paths):
    """sbr_path array + flat ray points (6 per ray) from a path set in either
    form solve() returns."""
    if isinstance(paths, dict):
        n = len(paths["receiver"])
        P = (_lib.Path * n)()
        A = np.ctypeslib.as_array(P) if n else None
        for k in ("request", "receiver", "launch", "heap", "ray_offset", "n_rays"):
            if n:
                A[k] = paths[k]
        return P, np.ascontiguousarray(paths["points"], np.float64).reshape(-1)
    P = (_lib.Path * len(paths))()
    pts, off = [], 0
    for i, p in enumerate(paths):
        P[i].request, P[i].receiver, P[i].launch = p["request"], p["receiver"], p["launch"]
        P[i].heap, P[i].n_rays, P[i].ray_offset = p["heap"], p["n_rays"], off
        off += p["n_rays"]
        pts.append(np.asarray(p["points"], np.float64).reshape(-1))
    flat = np.concatenate(pts) if pts else np.zeros(0)
    return P, np.ascontiguousarray(flat, np.float64)


class FieldCompute:
    """FieldCompute (FieldCompute.h:9-94): the field stage is fused into the
    GPU solve; FieldAtReceiver reads the result."""

    def __init__(self, result: Result):
        self._result = result

    def FieldAtReceiver(self, receiverId: int) -> np.ndarray:
        return self._result.field[receiverId]


class RTSolver:
    """RTSolver (RTSolver.h:18-83)."""

    def __init__(self, config: Optional[GlobalConfig] = None):
        self.config = config or GlobalConfig()
        self._scene: Optional[DeviceScene] = None
        self._result: Optional[Result] = None
        self._receivers = None

    def Init(self, materialProperties: Sequence[MaterialProperties], materialPropertiesCount: int,
             triangles: BVH) -> int:
        if triangles.mesh is None:
            raise ValueError("BVH.ConstructBVH was not called")
        self._scene = DeviceScene(triangles.mesh, list(materialProperties)[:materialPropertiesCount])
        return 0

    def ExecuteRayTracing(self, sourcePoint, txCoordSys, maxReflectionCount: int,
                          maxTransmissionCount: int, frequency: float, pt: float,
                          useFresnelCoeff: bool, receivers, triangleMesh: Mesh,
                          txTesslation: int) -> int:
        if self._scene is None:
            raise RuntimeError("Init was not called")
        rx = np.asarray(receivers, np.float64).reshape(-1, 3)
        req = make_request(sourcePoint, txCoordSys, maxReflectionCount, maxTransmissionCount,
                           frequency, pt, useFresnelCoeff, rx, txTesslation,
                           self.config.antennaType, self.config.fieldPrecision,
                           pattern=self.config.pattern)
        self._result = solve(self._scene, req, with_paths="arrays")
        self._receivers = rx
        return int(self._result.counts["launches"]) * int(rx.shape[0])

    @property
    def result(self) -> Result:
        return self._result

    def field_compute(self) -> FieldCompute:
        return FieldCompute(self._result)

    def _need_result(self):
        if self._result is None:
            raise RuntimeError("ExecuteRayTracing was not called")
        rx = np.ascontiguousarray(self._receivers, np.float64)
        f = np.ascontiguousarray(np.stack([self._result.field.real, self._result.field.imag],
                                          -1).reshape(-1), np.float64)
        return rx, f

    def SaveFieldAsCsv(self, fname: str) -> bool:
        """RTSolver::SaveFieldAsCsv (RTSolver.cpp:692-717), byte for byte,
        including its sticky std::showpos after the first receiver row."""
        rx, f = self._need_result()
        _lib.check(_lib.load().sbr_write_field_csv(os.fsencode(fname), _dp(rx), len(rx), _dp(f)))
        return True

    def SaveReceiversAsVtk(self, fname: str) -> bool:
        """RTSolver::SaveReceiversAsVtk (RTSolver.cpp:612-690), byte for byte."""
        rx, f = self._need_result()
        _lib.check(_lib.load().sbr_write_receivers_vtk(os.fsencode(fname), _dp(rx), len(rx),
                                                       _dp(f)))
        return True

    def SavePathsAsVtk(self, fname: str) -> bool:
        """RTSolver::SavePathsAsVtk (RTSolver.cpp:510-610), byte for byte:
        paths by launch, receiver, then breadth-first tree position."""
        rx, f = self._need_result()
        P, pts = _path_structs(self._result.paths)
        _lib.check(_lib.load().sbr_write_paths_vtk(os.fsencode(fname), P, len(P), _dp(pts),
                                                   _dp(f), len(rx)))
        return True

    def SaveIcosahedronAsVtk(self, fname: str, rayOrg, tessellation: int) -> bool:
        """RTSolver::SaveIcosahedronAsVtk (RTSolver.cpp:719-766): the launch
        rays of `tessellation` as unit segments from rayOrg."""
        o = np.ascontiguousarray(np.asarray(rayOrg, np.float64).reshape(3))
        _lib.check(_lib.load().sbr_write_launch_rays_vtk(os.fsencode(fname), _dp(o),
                                                         int(tessellation)))
        return True
