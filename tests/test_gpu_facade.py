"""The C++ facade (include/shy_world.hpp) drives the engine like the
reference's front-end loop, and gets what the Python binding gets."""
import json
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_front_end_loop_matches_python(shy, tmp_path):
    libdir = os.path.dirname(shy._capi.LIB_PATH)
    exe = tmp_path / "facade_loop"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "facade_loop.cpp"), "-L" + libdir, "-lshy",
                        "-Wl,-rpath," + libdir, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe), "128", "4", "300"], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    got = json.loads(out.stdout)
    w = shy.World(128, 128, seed=7)
    w.generate(7, 8)
    for _ in range(4):
        w.erode(300)
    h = w.get_field("height").astype(np.float64)
    assert w.stats().drop_steps == got["drop_steps"]
    assert h.sum() == pytest.approx(got["height_sum"], rel=1e-12)


def test_cpp_reference_sequence_matches_oracle(shy, po, tmp_path):
    """srand; frames of World::erode_sequential + Vegetation::grow through the
    facade give the oracle's plant list and heights."""
    libdir = os.path.dirname(shy._capi.LIB_PATH)
    exe = tmp_path / "facade_frames"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "facade_frames.cpp"), "-L" + libdir, "-lshy",
                        "-Wl,-rpath," + libdir, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe), "96", "30", "40", "3"], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    got = json.loads(out.stdout)
    m = po.Maps(96, 96, height=po.value_noise(96, 96, 4))
    plants, _ = po.frames(m, 3, 30, 40, 1, po.ERF_SHY)
    assert np.array_equal(np.array(got["plants"], np.float32).reshape(-1, 3), plants)
    assert m.height.astype(np.float64).sum() == got["height_sum"]
