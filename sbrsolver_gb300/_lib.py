"""ctypes binding of the C ABI (include/sbr.h).  Loads the in-tree
``libsbr.so``; there is no fallback: if the library or a GPU is missing the
calls fail with the library's error message."""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsbr.so")

OK, ERR_INVALID_ARG, ERR_OOM, ERR_CAPACITY, ERR_TIMEOUT, ERR_CUDA, ERR_IO, ERR_NOT_READY = range(8)
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CAPACITY", 4: "TIMEOUT", 5: "CUDA",
                6: "IO", 7: "NOT_READY"}

# Every symbol include/sbr.h declares.
EXPORTS = (
    "sbr_scene_create", "sbr_scene_create_from_stl", "sbr_scene_info_get", "sbr_scene_mesh_order",
    "sbr_scene_set_mesh_order", "sbr_scene_coplanar_ids", "sbr_scene_destroy", "sbr_solve",
    "sbr_solve_batch", "sbr_result_counts", "sbr_result_field", "sbr_result_paths",
    "sbr_result_timing", "sbr_result_destroy", "sbr_last_error", "sbr_version",
    "sbr_receiver_field_sum_noalloc", "sbr_server_create", "sbr_server_submit", "sbr_server_poll",
    "sbr_server_pending", "sbr_server_destroy", "sbr_server_set_policy",
    "sbr_result_field_error", "sbr_result_field_fp64",
    "sbr_write_field_csv", "sbr_write_receivers_vtk", "sbr_write_paths_vtk",
    "sbr_write_launch_rays_vtk", "sbr_scene_set_materials", "sbr_stl_read",
    "sbr_generate_rx_line", "sbr_generate_rx_plane", "sbr_pattern_create", "sbr_pattern_read",
    "sbr_pattern_info", "sbr_pattern_destroy", "sbr_fault_inject_alloc",
    "sbr_scene_set_tuning", "sbr_scene_get_tuning", "sbr_autotune", "sbr_result_field_bound",
    "sbr_scene_create_ex", "sbr_scene_triangle_frames", "sbr_scene_search_bvh",
    "sbr_scene_reference_bvh", "sbr_launch_directions",
)


class SbrError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Material(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("frequency", "transmission_loss", "reflection_loss",
                                           "rel_permittivity_re", "rel_permittivity_im",
                                           "rel_conductivity", "width")]


class SceneInfo(C.Structure):
    _fields_ = [("n_triangles", C.c_int), ("n_bvh_nodes", C.c_int), ("bvh_depth", C.c_int),
                ("n_coplanar", C.c_int), ("extent", C.c_double), ("device_bytes", C.c_longlong),
                ("prep_total_ms", C.c_double), ("prep_host_ms", C.c_double),
                ("prep_device_tables_ms", C.c_double), ("prep_search_bvh_ms", C.c_double),
                ("prep_reference_bvh_ms", C.c_double), ("prep_upload_ms", C.c_double)]


class Request(C.Structure):
    _fields_ = [("tx", C.c_double * 3), ("tx_coord_sys", C.c_double * 9),
                ("max_reflection", C.c_int), ("max_transmission", C.c_int),
                ("frequency", C.c_double), ("pt", C.c_double), ("use_fresnel", C.c_int),
                ("tessellation", C.c_int), ("antenna", C.c_int), ("field_precision", C.c_int),
                ("n_rx", C.c_int), ("rx", C.POINTER(C.c_double)), ("rx_on_device", C.c_int),
                ("stage_counts", C.c_int), ("field_check", C.c_int), ("pattern", C.c_void_p)]


class FieldError(C.Structure):
    _fields_ = [("components", C.c_longlong), ("over_tolerance", C.c_longlong),
                ("max_rel_mag", C.c_double), ("max_phase_rad", C.c_double),
                ("max_rel_vec", C.c_double)]


class Counts(C.Structure):
    _fields_ = [(n, C.c_longlong) for n in ("segments", "captured", "corrected", "paths", "rays",
                                             "fp64_triangle_tests", "fallback_rays",
                                             "fp64_capture_tests", "launches",
                                             "capture_candidates", "ancestor_tests",
                                             "classes", "groups", "keys",
                                             "near_edge_paths", "gpu_kernels",
                                             "fp64_field_paths", "fp64_field_receivers",
                                             "pipeline_graph")]


class Path(C.Structure):
    _fields_ = [("request", C.c_int), ("receiver", C.c_int), ("n_rays", C.c_int),
                ("heap", C.c_int), ("launch", C.c_longlong), ("ray_offset", C.c_longlong),
                ("field", C.c_double * 6), ("near_edge", C.c_int), ("reserved", C.c_int)]


class Completion(C.Structure):
    _fields_ = [("tag", C.c_longlong), ("status", C.c_int), ("scene", C.c_int),
                ("queue_ms", C.c_double), ("latency_ms", C.c_double), ("device_ms", C.c_double),
                ("counts", Counts), ("result", C.c_void_p)]


class Tuning(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("find_steps", "find_refill", "find_blocks_per_sm",
                                        "trace_blocks_per_sm", "capture_blocks_per_sm",
                                        "trace_chunk_log2", "trace_kernel",
                                        "pipeline_graph", "find_tris_per_step")]


class Timing(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("total_ms", "trace_ms", "capture_ms", "correct_ms",
                                           "field_ms", "h2d_ms", "d2h_ms", "device_ms",
                                           "capture_kernel_ms", "trace_kernel_ms",
                                           "trace_kernel_launches", "trace_kernel_first_ms")]


_lib = None
_lock = threading.Lock()


def load(path: str = LIB_PATH):
    """Loads libsbr.so (once) and declares the signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise OSError(f"{path} is not built; run sbrsolver_gb300.build.build_library()")
        lib = C.CDLL(path)
        P, I, D = C.POINTER, C.c_int, C.c_double
        vp = C.c_void_p
        sig = {
            "sbr_scene_create": [I, P(C.c_float), P(C.c_float), P(I), P(Material), I, P(vp)],
            "sbr_scene_create_from_stl": [C.c_char_p, P(I), P(Material), I, P(vp)],
            "sbr_scene_info_get": [vp, P(SceneInfo)],
            "sbr_scene_mesh_order": [vp, P(I)],
            "sbr_scene_set_mesh_order": [vp, P(I)],
            "sbr_scene_coplanar_ids": [vp, P(I)],
            "sbr_scene_destroy": [vp],
            "sbr_solve": [vp, P(Request), P(vp)],
            "sbr_solve_batch": [vp, P(Request), I, P(vp)],
            "sbr_result_counts": [vp, P(Counts)],
            "sbr_result_field": [vp, P(D)],
            "sbr_result_field_fp64": [vp, P(D)],
            "sbr_result_field_error": [vp, P(FieldError)],
            "sbr_result_paths": [vp, P(Path), P(I), P(I), P(I), P(D)],
            "sbr_result_timing": [vp, P(Timing)],
            "sbr_result_destroy": [vp],
            "sbr_receiver_field_sum_noalloc": [vp, vp, vp, I, I, I, vp, vp],
            "sbr_server_create": [P(vp), I, I, C.c_longlong, P(vp)],
            "sbr_server_submit": [vp, I, P(Request), C.c_longlong],
            "sbr_server_poll": [vp, P(Completion), I, P(I), I],
            "sbr_server_pending": [vp, P(I), P(C.c_longlong)],
            "sbr_server_destroy": [vp],
            "sbr_server_set_policy": [vp, C.c_longlong, C.c_int, C.c_double, C.c_int],
            "sbr_write_field_csv": [C.c_char_p, P(D), I, P(D)],
            "sbr_write_receivers_vtk": [C.c_char_p, P(D), I, P(D)],
            "sbr_write_paths_vtk": [C.c_char_p, P(Path), I, P(D), P(D), I],
            "sbr_write_launch_rays_vtk": [C.c_char_p, P(D), I],
            "sbr_scene_set_materials": [vp, P(I), P(Material), I],
            "sbr_stl_read": [C.c_char_p, P(I), P(C.c_float), P(C.c_float)],
            "sbr_generate_rx_line": [P(D), P(D), D, P(D), I, P(I)],
            "sbr_generate_rx_plane": [D, D, D, D, D, D, P(D), I, P(I)],
            "sbr_pattern_create": [I, I, D, D, P(C.c_float), P(vp)],
            "sbr_pattern_read": [C.c_char_p, P(vp)],
            "sbr_pattern_info": [vp, P(I), P(I), P(D), P(D)],
            "sbr_pattern_destroy": [vp],
            "sbr_fault_inject_alloc": [C.c_longlong],
            "sbr_scene_set_tuning": [vp, P(Tuning)],
            "sbr_scene_get_tuning": [vp, P(Request), I, P(Tuning)],
            "sbr_autotune": [vp, P(Request), I, I, P(Tuning), P(D)],
            "sbr_result_field_bound": [vp, P(D)],
            "sbr_scene_create_ex": [I, P(C.c_float), P(C.c_float), P(I), P(Material), I,
                                    C.c_uint, P(vp)],
            "sbr_scene_triangle_frames": [vp, P(D), P(D), P(D)],
            "sbr_scene_search_bvh": [vp, P(I), P(I), P(C.c_float), P(I)],
            "sbr_scene_reference_bvh": [vp, P(I), P(I), P(C.c_double), P(I), P(I)],
            "sbr_launch_directions": [I, P(D), C.c_longlong, P(C.c_longlong)],
        }
        for name, args in sig.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = C.c_int
        lib.sbr_last_error.restype = C.c_char_p
        lib.sbr_last_error.argtypes = []
        lib.sbr_version.restype = C.c_char_p
        lib.sbr_version.argtypes = []
        _lib = lib
        return lib


def check(status: int) -> None:
    if status != OK:
        raise SbrError(status, load().sbr_last_error().decode(errors="replace"))
