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


def test_per_cell_statistics_match_the_plant_agents(shy):
    """The per-cell form (with batched erosion, as the large-scale workload
    runs it) against the reference's plant agents in its own frame loop
    (World::erode(512); Vegetation::grow(), SimpleHydrology.cpp:319-320):
    tests/golden/vegetation_stats.json holds eight reference runs on the
    reference's 512^2 terrain (seed 42) after 300 frames.  The reference
    makes one spawn attempt per frame at a random cell, so the per-cell
    spawn probability is 1 / 512^2.  Six per-cell runs (one batch of six
    terrains with their own seeds) must agree with the reference on every
    statistic within three standard errors of the difference of the means."""
    import json
    import os
    fx = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "vegetation_stats.json")))
    n, frames, drops = fx["config"]["map"][0], fx["config"]["frames"], fx["config"]["drops_per_frame"]
    seeds = list(range(1, 7))
    p = shy.default_params()
    p.plant_spawn_prob = 1.0 / (n * n)
    b = shy.Batch([(n, n)] * len(seeds), [drops] * len(seeds), seeds, params=p)
    for t in range(len(seeds)):
        b.init_terrain(t, 42)
    for _ in range(frames):
        b.erode(1)
        b.vegetation_step(1)
    runs = []
    for t in range(len(seeds)):
        plant = b.get_field(t, "plant_size")
        root = b.get_field(t, "root_density")
        alive = plant > 0
        runs.append({"plants": int(alive.sum()), "mean_size": float(plant[alive].mean()),
                     "root_mean": float(root.mean(dtype=np.float64)), "root_cover": float((root > 0.01).mean())})
    b.close()
    ref = fx["runs"]
    report = {}
    for k in ("plants", "mean_size", "root_mean", "root_cover"):
        a = np.array([r[k] for r in runs], np.float64)
        r = np.array([q[k] for q in ref], np.float64)
        se = np.sqrt(a.var(ddof=1) / a.size + r.var(ddof=1) / r.size)
        report[k] = (a.mean(), r.mean(), se)
        assert abs(a.mean() - r.mean()) <= 3.0 * se, (k, report[k])
    print(report)
