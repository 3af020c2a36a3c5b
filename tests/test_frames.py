"""The reference's frame loop in its own random sequence: srand(s), then
frames of World::erode(n); Vegetation::grow(); with the plant agents
(source/vegetation.h:12-188) and the C-library rand() stream that spawns and
plant events share.

The oracle's restatement is pinned against fixtures made from the reference
build (tests/golden/ref_frames.json, ref_feed.json); the GPU's sequence
(shy_world_srand, shy_erode_rand, shy_vegetation_grow) must equal the
oracle's bit for bit, maps and plant list."""
import ctypes as C
import ctypes.util
import hashlib
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_restated_rand_equals_c_library(po):
    libc = C.CDLL(ctypes.util.find_library("c"))
    for seed in (0, 1, 5, 12345, 2 ** 31, 2 ** 32 - 1):
        libc.srand(C.c_uint(seed))
        want = np.array([libc.rand() for _ in range(20000)], np.int32)
        assert np.array_equal(po.crand(seed, 20000), want), seed


def test_oracle_frames_and_feed_match_reference_fixtures(po):
    with open(os.path.join(GOLDEN, "ref_frames.json")) as f:
        g = json.load(f)
    with open(os.path.join(GOLDEN, "ref_feed.json")) as f:
        gf = json.load(f)
    n = g["meta"]["map"]
    m = po.Maps(n, n, height=po.value_noise(n, n, g["terrain_seed"]))
    plants, _ = po.frames(m, g["seed"], g["frames"], g["drops"], g["order"], po.ERF_LIBM)
    assert len(plants) == g["plants"]
    assert sha(plants) == g["plants_sha"]
    for k, f in enumerate(po.FIELDS):
        assert sha(m.f[k]) == g["field_sha"][f], f
    assert sha(po.feed(m, 2, po.ERF_LIBM)) == gf["vertices_sha"]
    assert sha(po.feed(m, 0, po.ERF_LIBM)) == gf["discharge_rgba_sha"]
    assert sha(po.feed(m, 1, po.ERF_LIBM)) == gf["momentum_rgba_sha"]


def test_frame_loop_arguments(shy):
    L = shy.lib()
    assert L.shy_world_srand(None, 1) == -1
    assert L.shy_erode_rand(None, 1) == -1
    assert L.shy_vegetation_grow(None) == -1
    assert L.shy_world_set_rand_order(None, 0) == -1


def terrain(po, nx=96, ny=90):
    return (po.value_noise(nx, ny, 4) * 0.25 + 0.2).astype(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 0])
def test_gpu_frames_bitwise(shy, po, order):
    H = terrain(po)
    w = shy.World(96, 90)
    w.set_field("height", H)
    w.set_field("root_density", np.zeros_like(H))
    if order == 0:
        check = shy.lib().shy_world_set_rand_order(w._w, 0)
        assert check == 0
    w.srand(3)
    for _ in range(60):
        w.erode_rand(40)
        w.grow()
    m = po.Maps(96, 90, height=H)
    plants, acc = po.frames(m, 3, 60, 40, order, po.ERF_SHY)
    got = w.plants()
    assert len(got) == len(plants) and len(plants) > 20
    assert np.array_equal(bits(got), bits(plants))
    for k, f in enumerate(po.FIELDS):
        assert np.array_equal(bits(w.get_field(f)), bits(m.f[k])), f
    assert w.stats().drop_steps == acc.steps
    w.close()


@pytest.mark.gpu
def test_gpu_frames_resume_from_checkpoint(shy, po, tmp_path):
    H = terrain(po)
    w = shy.World(96, 90)
    w.set_field("height", H)
    w.srand(8)
    for _ in range(25):
        w.erode_rand(40)
        w.grow()
    path = tmp_path / "f.ckpt"
    w.save(path)
    for _ in range(25):
        w.erode_rand(40)
        w.grow()
    want_plants, want_h = w.plants(), w.get_field("height")
    w.close()
    r = shy.load(path)
    for _ in range(25):
        r.erode_rand(40)
        r.grow()
    assert np.array_equal(bits(r.plants()), bits(want_plants))
    assert np.array_equal(bits(r.get_field("height")), bits(want_h))
    r.close()
