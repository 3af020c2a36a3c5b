"""Checkpoint and resume: a world written with shy_world_save and reopened
with shy_world_load continues bit for bit as the original; damaged or foreign
files are refused."""
import ctypes as C

import numpy as np
import pytest

FIELDS = ("height", "discharge", "momentum_x", "momentum_y", "discharge_track", "momentum_x_track",
          "momentum_y_track", "root_density", "plant_size")
SHY_ERR_IO = -7


def test_load_refuses_missing_and_foreign_files(shy, tmp_path):
    L = shy.lib()
    h = C.c_void_p()
    assert L.shy_world_load(str(tmp_path / "none.ckpt").encode(), C.byref(h)) == SHY_ERR_IO
    bad = tmp_path / "bad.ckpt"
    bad.write_bytes(b"not a checkpoint" * 20)
    assert L.shy_world_load(str(bad).encode(), C.byref(h)) == SHY_ERR_IO
    assert b"damaged" in L.shy_last_error() or b"format" in L.shy_last_error()
    assert L.shy_world_load(None, C.byref(h)) == -1
    assert L.shy_world_save(None, b"x") == -1


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def snapshot(w):
    return {f: w.get_field(f) for f in FIELDS}, w.stats().as_dict()


@pytest.mark.gpu
def test_resume_is_bit_exact(shy, tmp_path):
    p = shy.default_params()
    p.plant_spawn_prob = 1e-2
    w = shy.World(150, 120, params=p, seed=9)
    w.generate(9, 8)
    for _ in range(3):
        w.erode(3000, 1)
        w.vegetation_step(1)
    path = tmp_path / "w.ckpt"
    w.save(path)
    for _ in range(2):
        w.erode(3000, 1)
        w.vegetation_step(1)
    a_fields, a_stats = snapshot(w)
    w.close()

    r = shy.load(path)
    assert isinstance(r, shy.World) and (r.nx, r.ny) == (150, 120)
    for _ in range(2):
        r.erode(3000, 1)
        r.vegetation_step(1)
    b_fields, b_stats = snapshot(r)
    for f in FIELDS:
        assert np.array_equal(bits(a_fields[f]), bits(b_fields[f])), f
    assert a_stats == b_stats
    assert bytes(r.params) == bytes(p)
    r.close()


@pytest.mark.gpu
def test_resume_batch_and_exact_mode(shy, tmp_path):
    b = shy.Batch([(64, 40), (33, 90)], [500, 700], [3, 4])
    for t in range(2):
        b.generate(t, 10 + t, 8)
    b.erode(2)
    path = tmp_path / "b.ckpt"
    b.save(path)
    b.erode(1)
    want = [b.get_field(t, "height") for t in range(2)]
    b.close()
    r = shy.load(path)
    assert isinstance(r, shy.Batch) and r.sizes == [(64, 40), (33, 90)]
    r.erode(1)
    for t in range(2):
        assert np.array_equal(bits(r.get_field(t, "height")), bits(want[t]))
    r.close()

    # the exact (sequential) mode resumes from the float maps
    w = shy.World(80, 80, seed=2)
    w.generate(2, 8)
    spawns = np.stack([np.arange(0, 80, 2), np.arange(79, -1, -2)], 1).astype(np.int32)
    w.erode_exact(spawns)
    w.save(path)
    w.erode_exact(spawns)
    want = w.get_field("height")
    w.close()
    r = shy.load(path)
    r.erode_exact(spawns)
    assert np.array_equal(bits(r.get_field("height")), bits(want))
    r.close()


@pytest.mark.gpu
def test_damaged_checkpoint_is_refused(shy, tmp_path):
    w = shy.World(32, 32)
    w.generate(1, 8)
    path = tmp_path / "w.ckpt"
    w.save(path)
    w.close()
    data = bytearray(path.read_bytes())
    data[len(data) // 2] ^= 0x40
    path.write_bytes(bytes(data))
    with pytest.raises(shy.ShyError) as e:
        shy.load(path)
    assert e.value.code == SHY_ERR_IO
