"""The front end's per-frame data (discharge and momentum textures, terrain
mesh; SimpleHydrology.cpp:322-355, source/cellpool.h:286-317).

The oracle's restatement is pinned against the reference: the mesh through
the reference's own updatenode, the textures through its map accessors.  The
GPU buffers must equal the oracle's bit for bit (same correctly rounded erf);
against libm's erff, which the reference calls, the textures differ by at
most one unit in the last place of erf."""
import ctypes as C

import numpy as np
import pytest

KINDS = {"discharge_rgba": 0, "momentum_rgba": 1, "vertices": 2}


def maps_with_flow(po, nx, ny, seed):
    rng = np.random.default_rng(seed)
    m = po.Maps(nx, ny, height=po.value_noise(nx, ny, seed))
    m.f[1][...] = rng.gamma(0.5, 2.0, (nx, ny)).astype(np.float32)
    m.f[2][...] = rng.normal(0, 1.5, (nx, ny)).astype(np.float32)
    m.f[3][...] = rng.normal(0, 1.5, (nx, ny)).astype(np.float32)
    return m


def test_oracle_feed_matches_reference(po):
    if not po.ref_available():
        pytest.skip("reference harness not built")
    n = 512
    m = maps_with_flow(po, n, n, 7)
    po.ref_set_maps(m)
    v = np.zeros((n, n, 12), np.float32)
    d = np.zeros((n, n, 4), np.float32)
    mo = np.zeros((n, n, 4), np.float32)
    po.ref().ref_frame(po.fptr(v), po.fptr(d), po.fptr(mo))
    for kind, ref in ((2, v), (0, d), (1, mo)):
        got = po.feed(m, kind, po.ERF_LIBM)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), kind
        shy = po.feed(m, kind, po.ERF_SHY)
        # the library's erf is correctly rounded; glibc's erff is off by one
        # ulp on some inputs: 0.5 (1 + erf) then differs by half an ulp of erf
        assert np.abs(shy.astype(np.float64) - ref).max() <= 2.0 ** -24


def test_feed_rejects_bad_arguments(shy):
    L = shy.lib()
    buf = (C.c_float * 4)()
    assert L.shy_feed(None, 0, 0, buf, 4, 0) == -1


@pytest.mark.gpu
@pytest.mark.parametrize("kind", list(KINDS))
def test_gpu_feed_bitwise(shy, po, kind):
    nx, ny = 96, 130
    m = maps_with_flow(po, nx, ny, 3)
    w = shy.World(nx, ny)
    for f in ("height", "discharge", "momentum_x", "momentum_y"):
        w.set_field(f, m.f[po.FIELDS.index(f)])
    got = w.feed(kind)
    ref = po.feed(m, KINDS[kind], po.ERF_SHY)
    assert got.shape == ref.shape
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    w.close()


@pytest.mark.gpu
def test_gpu_feed_after_erosion_and_on_device(shy, po):
    import torch
    nx, ny = 128, 100
    w = shy.World(nx, ny, seed=4)
    w.generate(4, 8)
    w.erode(2000, 2)
    m = po.Maps(nx, ny)
    for f in ("height", "discharge", "momentum_x", "momentum_y"):
        m.f[po.FIELDS.index(f)][...] = w.get_field(f)
    for kind, k in KINDS.items():
        per = 12 if kind == "vertices" else 4
        dev = torch.empty((nx, ny, per), dtype=torch.float32, device="cuda")
        w.feed(kind, out=dev)
        w.sync()
        ref = po.feed(m, k, po.ERF_SHY)
        assert np.array_equal(dev.cpu().numpy().view(np.uint32), ref.view(np.uint32)), kind
        assert np.array_equal(w.feed(kind).view(np.uint32), ref.view(np.uint32)), kind
    w.close()


@pytest.mark.gpu
def test_gpu_feed_batch_terrain_and_errors(shy, po):
    b = shy.Batch([(40, 50), (33, 64)], [100, 100], [1, 2])
    b.generate(1, 9, 8)
    got = b.feed("vertices", terrain=1)
    m = po.Maps(33, 64, height=b.get_field(1, "height"))
    assert np.array_equal(got.view(np.uint32), po.feed(m, 2).view(np.uint32))
    L = shy.lib()
    a = np.zeros(33 * 64 * 4, np.float32)
    p = a.ctypes.data_as(C.c_void_p)
    assert L.shy_feed(b._w, 1, 0, p, a.size - 1, 0) == -1   # wrong count
    assert L.shy_feed(b._w, 1, 7, p, a.size, 0) == -1       # unknown kind
    assert L.shy_feed(b._w, 2, 0, p, a.size, 0) == -1       # no such terrain
    b.close()
