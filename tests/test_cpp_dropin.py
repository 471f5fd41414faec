"""The C++ drop-in header (include/sbr_solver.hpp): the reference's main()
written against it compiles with warnings enabled, its host-side
preprocessing runs without a GPU, and on a GPU it writes the reference's
shipped output files byte for byte."""
import hashlib
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from sbrsolver_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "sbrsolver_gb300")
SHIPPED = json.load(open(os.path.join(ROOT, "tests", "golden", "shipped_outputs.json")))


@pytest.fixture(scope="module")
def program(built, tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("cpp")
    exe = str(d / "reference_main")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror",
                    "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "reference_main.cpp"),
                    "-L", PKG, "-lsbr", f"-Wl,-rpath,{PKG}", "-o", exe], check=True)
    stl = str(d / "ground.stl")
    scenes.write_stl(scenes.reference_main_scene().scene, stl)
    return exe, stl, d


def test_preprocessing_without_gpu(program):
    exe, stl, d = program
    out = subprocess.run([exe, stl, str(d), "prep"], capture_output=True, text=True, check=True)
    first, second = out.stdout.splitlines()
    assert first.split() == ["triangles", "2", "last", "1", "(-5", "1000", "0)", "receivers",
                             "3000", "last", "(0", "2999", "3)", "plane", "121"]
    # GenerateRaysOnIcosahedron: the reference's level-2 directions, last one bit for bit
    ico = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                               "icosphere_L2.npy"))
    t = second.split()
    assert t[:3] == ["rays", str(len(ico)), "last"]
    assert [float(x) for x in t[3:]] == list(ico[-1])


@pytest.mark.gpu
def test_reference_main_through_cpp_header(program):
    exe, stl, d = program
    out = d / "out"
    out.mkdir()
    r = subprocess.run([exe, stl, str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "launches x receivers 486000" in r.stdout
    for name, meta in SHIPPED.items():
        got = hashlib.sha256((out / name).read_bytes()).hexdigest()
        assert got == meta["sha256"], name
