"""Per-cell vegetation (Vegetation::grow, source/vegetation.h:122-188) on the
GPU against the oracle's restatement, and its coupling to erosion through
root density (source/water.h:86-87)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_vegetation_steps_bitwise_and_coupled(shy, po):
    nx, ny, seed = 128, 96, 12
    p = shy.default_params()
    p.plant_spawn_prob = 1e-2  # enough plants in a small map
    w = shy.World(nx, ny, params=p, seed=seed)
    w.generate(seed, 8)
    w.erode(2000, 3)  # some discharge, so that rivers kill plants
    m = po.Maps(nx, ny)
    for k, f in enumerate(po.FIELDS):
        m.f[k][...] = w.get_field(f)
    plant = w.get_field("plant_size").copy()
    pp = po.default_params()
    pp.plant_spawn_prob = 1e-2
    for step in range(25):
        po.vegetation_step(m, plant, seed, step, pp)
    w.vegetation_step(25)
    assert np.array_equal(bits(w.get_field("plant_size")), bits(plant))
    assert np.array_equal(bits(w.get_field("root_density")), bits(m.root_density))
    assert (plant > 0).sum() > 20
    # erosion now runs with the lower deposition rate under roots (both sides
    # start from the float heights)
    w.set_field("height", w.get_field("height"))
    w.erode(2000, 1)
    hq = None
    po.erode_batched(m, seed, 3, 2000, 1, pp, hq)
    for k, f in enumerate(po.FIELDS):
        assert np.array_equal(bits(w.get_field(f)), bits(m.f[k])), f
    w.close()
