"""The C-ABI library (no GPU needed): it builds, loads, exports every symbol
include/sbr.h declares, and rejects bad arguments with a status and message."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from sbrsolver_gb300 import _lib, api, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _gpu_present():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_header_and_exports_agree(built):
    hdr = open(os.path.join(ROOT, "include", "sbr.h")).read()
    declared = set(re.findall(r"\b(sbr_[a-z0-9_]+)\s*\(", hdr))
    assert declared == set(_lib.EXPORTS)
    lib = _lib.load()
    for name in declared:
        assert hasattr(lib, name), name
    assert b"sm_103a" in lib.sbr_version()


def test_struct_layouts_match_header(tmp_path):
    """The ctypes structures have the header's sizes and field offsets (a C
    program compiled against include/sbr.h prints them)."""
    checks = {"sbr_request": (_lib.Request, ["n_rx", "rx", "stage_counts", "field_check", "pattern"]),
              "sbr_counts": (_lib.Counts, ["keys", "near_edge_paths", "gpu_kernels"]),
              "sbr_path": (_lib.Path, ["launch", "field", "near_edge"]),
              "sbr_timing": (_lib.Timing, ["device_ms", "capture_kernel_ms", "trace_kernel_launches"]),
              "sbr_field_error": (_lib.FieldError, ["max_rel_vec"]),
              "sbr_completion": (_lib.Completion, ["counts", "result"]),
              "sbr_material": (_lib.Material, ["rel_conductivity", "width"]),
              "sbr_scene_info": (_lib.SceneInfo, ["device_bytes"])}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "sbr.h"', "int main(void) {"]
    for t, (_, fields) in checks.items():
        lines.append(f'  printf("{t} %zu\\n", sizeof({t}));')
        for f in fields:
            lines.append(f'  printf("{t}.{f} %zu\\n", offsetof({t}, {f}));')
    lines.append("  return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    import subprocess
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                 check=True).stdout.splitlines())
    for t, (cls, fields) in checks.items():
        assert int(got[t]) == C.sizeof(cls), t
        for f in fields:
            assert int(got[f"{t}.{f}"]) == getattr(cls, f).offset, (t, f)


def test_null_arguments_are_rejected(built):
    lib = _lib.load()
    out = C.c_void_p()
    assert lib.sbr_scene_create(0, None, None, None, None, 0, C.byref(out)) == _lib.ERR_INVALID_ARG
    assert b"empty" in lib.sbr_last_error()
    assert lib.sbr_solve_batch(None, None, 0, C.byref(out)) == _lib.ERR_INVALID_ARG
    assert lib.sbr_result_counts(None, None) == _lib.ERR_INVALID_ARG
    assert lib.sbr_scene_destroy(None) == _lib.OK
    assert lib.sbr_result_destroy(None) == _lib.OK
    assert lib.sbr_server_set_policy(None, 1 << 30, 8, 1e9, 1) == _lib.ERR_INVALID_ARG
    assert b"set_policy" in lib.sbr_last_error()


def test_missing_stl_is_io_error(built):
    lib = _lib.load()
    out = C.c_void_p()
    m = (_lib.Material * 1)(_lib.Material(1e9, 0, 0, 5, 0, 0.1))
    st = lib.sbr_scene_create_from_stl(b"/nonexistent/x.stl", None, m, 1, C.byref(out))
    assert st == _lib.ERR_IO
    assert b"cannot open" in lib.sbr_last_error()


def test_bad_material_id_rejected(built):
    wl = scenes.small_scene()
    mesh = api.Mesh(wl.scene.tri, wl.scene.normal, np.full(wl.scene.n_tri, 7, np.int32))
    with pytest.raises(_lib.SbrError) as e:
        api.DeviceScene(mesh, [api.MaterialProperties()])
    assert e.value.status == _lib.ERR_INVALID_ARG
    assert "material id out of range" in str(e.value)


@pytest.mark.parametrize("width", [-0.1, float("nan"), float("inf")])
def test_bad_wall_width_rejected(built, width):
    wl = scenes.small_scene()
    mesh = api.Mesh(wl.scene.tri, wl.scene.normal, wl.scene.material_id)
    mats = [api.MaterialProperties(*m) for m in wl.scene.materials]
    mats[1].width = width
    with pytest.raises(_lib.SbrError) as e:
        api.DeviceScene(mesh, mats)
    assert e.value.status == _lib.ERR_INVALID_ARG
    assert "width" in str(e.value)


@pytest.mark.skipif(_gpu_present(), reason="checks the no-GPU error path")
def test_no_gpu_fails_loudly(built):
    """Without a GPU the product path returns a CUDA error; it never falls
    back to a CPU computation."""
    wl = scenes.small_scene()
    with pytest.raises(_lib.SbrError) as e:
        api.DeviceScene.from_scene(wl.scene)
    assert e.value.status in (_lib.ERR_CUDA, _lib.ERR_OOM)


def test_truncated_stl_is_io_error(built, tmp_path):
    """A binary STL cut short, or one whose header counts more facets than
    the file holds, is refused before any storage is sized from the count."""
    lib = _lib.load()
    wl = scenes.small_scene()
    whole = tmp_path / "whole.stl"
    scenes.write_stl(wl.scene, str(whole))
    data = whole.read_bytes()
    n = C.c_int()
    assert lib.sbr_stl_read(str(whole).encode(), C.byref(n), None, None) == _lib.OK
    assert n.value == wl.scene.n_tri
    cut = tmp_path / "cut.stl"
    cut.write_bytes(data[: 84 + 50 * 7 + 20])  # 7 whole facets and part of the 8th
    assert lib.sbr_stl_read(str(cut).encode(), C.byref(n), None, None) == _lib.ERR_IO
    assert b"truncated" in lib.sbr_last_error()
    huge = tmp_path / "huge.stl"  # header claims 2^32 - 1 facets
    huge.write_bytes(data[:80] + (0xFFFFFFFF).to_bytes(4, "little") + data[84:84 + 500])
    assert lib.sbr_stl_read(str(huge).encode(), C.byref(n), None, None) == _lib.ERR_IO
    assert b"4294967295" in lib.sbr_last_error()
    head = tmp_path / "head.stl"
    head.write_bytes(data[:60])
    assert lib.sbr_stl_read(str(head).encode(), C.byref(n), None, None) == _lib.ERR_IO
    out = C.c_void_p()
    m = (_lib.Material * 1)(_lib.Material(1e9, 0, 0, 5, 0, 0.1))
    assert lib.sbr_scene_create_from_stl(str(cut).encode(), None, m, 1, C.byref(out)) == _lib.ERR_IO
    assert not out.value


@pytest.mark.parametrize("where", ["vertex", "normal"])
def test_non_finite_scene_rejected(built, where):
    """NaN / inf in the triangle list is an argument error, found before any
    device work."""
    wl = scenes.small_scene()
    tri, nrm = wl.scene.tri.copy(), wl.scene.normal.copy()
    if where == "vertex":
        tri[5, 1, 2] = np.nan
    else:
        nrm[9, 0] = np.inf
    with pytest.raises(_lib.SbrError) as e:
        api.DeviceScene(api.Mesh(tri, nrm, wl.scene.material_id),
                        [api.MaterialProperties(*m) for m in wl.scene.materials])
    assert e.value.status == _lib.ERR_INVALID_ARG
    assert "finite" in str(e.value)


def test_fault_hook_arms_and_disarms(built):
    lib = _lib.load()
    assert lib.sbr_fault_inject_alloc(3) == _lib.OK
    assert lib.sbr_fault_inject_alloc(-1) == _lib.OK


def _header_prototypes():
    """Every function include/sbr.h declares: name -> parameter types."""
    hdr = open(os.path.join(ROOT, "include", "sbr.h")).read()
    hdr = re.sub(r"/\*.*?\*/", " ", hdr, flags=re.S)
    protos = {}
    for name, params in re.findall(r"\b(sbr_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", hdr):
        params = " ".join(params.split())
        protos[name] = [] if params in ("", "void") else [p.strip() for p in params.split(",")]
    return protos


def _kind_of_c(param: str):
    """(kind, bytes) of a C parameter declaration: pointers, then scalars."""
    if "*" in param:
        return ("ptr", 8)
    words = param.split()[:-1]  # drop the parameter name
    if "double" in words:
        return ("float", 8)
    if words.count("long") == 2:
        return ("signed", 8)
    if "unsigned" in words or "uint32_t" in words:
        return ("unsigned", 4)
    if "int" in words:
        return ("signed", 4)
    raise AssertionError(f"unclassified parameter type: {param!r}")


def _kind_of_ctypes(t):
    if t in (C.c_void_p, C.c_char_p) or issubclass(t, C._Pointer):
        return ("ptr", 8)
    code = t._type_
    if code == "d":
        return ("float", C.sizeof(t))
    if code in "bhilq":
        return ("signed", C.sizeof(t))
    if code in "BHILQ":
        return ("unsigned", C.sizeof(t))
    raise AssertionError(f"unclassified ctypes type: {t!r}")


def test_bindings_match_header_prototypes(built):
    """Each ctypes binding passes as many arguments as the header declares,
    each of the same kind and width (pointer, signed or unsigned integer,
    double), so a change of a C signature cannot go unnoticed by the
    Python side."""
    protos = _header_prototypes()
    assert set(protos) == set(_lib.EXPORTS)
    lib = _lib.load()
    for name, params in protos.items():
        argtypes = getattr(lib, name).argtypes
        assert argtypes is not None, name
        assert len(argtypes) == len(params), (name, params, argtypes)
        for p, t in zip(params, argtypes):
            assert _kind_of_c(p) == _kind_of_ctypes(t), (name, p, t)
