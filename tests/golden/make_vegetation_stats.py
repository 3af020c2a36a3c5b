"""Generate tests/golden/vegetation_stats.json: plant statistics of the
reference's frame loop, for the statistical check of the per-cell vegetation
form (shy_vegetation_step) against the reference's plant agents.

The reference's front end runs, per frame, World::erode(quad::tilesize)
then Vegetation::grow() (SimpleHydrology.cpp:319-320; source/world.h:54-88,
source/vegetation.h:122-188): 512 drops, one random spawn attempt, and every
plant grows, may die, and spreads with chance 1/20.  The CPU oracle's frame
loop (oracle/hydro_oracle.cpp, orc_frames_f32) equals the reference build
bit for bit (tests/golden/ref_frames.json).  This script runs it on the
reference's own 512^2 terrain (World::map.init seed 42) for 300 frames from
eight srand seeds and stores, per seed, the plant count, mean plant size,
mean root density and the fraction of cells with root density above 0.01.

    python tests/golden/make_vegetation_stats.py
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

N, FRAMES, DROPS, TERRAIN_SEED = 512, 300, 512, 42
SEEDS = tuple(range(1, 9))
OUT = os.path.join(HERE, "vegetation_stats.json")


def stats(plants_xy_size, root):
    """The statistics compared: plants, their mean size, root density."""
    n = int(len(plants_xy_size))
    return {"plants": n,
            "mean_size": float(np.mean(plants_xy_size[:, 2])) if n else 0.0,
            "root_mean": float(np.mean(root, dtype=np.float64)),
            "root_cover": float(np.mean(root > 0.01))}


def run(seed):
    from oracle import pyoracle as po
    m = po.Maps(N, N, height=po.terrain_init(N, N, TERRAIN_SEED))
    plants, acc = po.frames(m, seed, FRAMES, DROPS)
    out = stats(plants, m.f[7])
    out["srand"] = seed
    out["drop_steps"] = int(acc.steps)
    return out


def main():
    from oracle import pyoracle as po
    po.build()
    with mp.get_context("spawn").Pool(min(len(SEEDS), os.cpu_count() or 1)) as pool:
        res = pool.map(run, SEEDS)
    keys = ("plants", "mean_size", "root_mean", "root_cover")
    doc = {
        "what": "the reference's frame loop (World::erode(512); Vegetation::grow()) on its own 512^2 terrain, "
                "plant statistics after 300 frames for eight srand seeds (oracle restatement, bit-exact with the "
                "reference)",
        "config": {"map": [N, N], "terrain": f"World::map.init seed {TERRAIN_SEED}", "frames": FRAMES,
                   "drops_per_frame": DROPS, "srand_seeds": list(SEEDS)},
        "generator": "tests/golden/make_vegetation_stats.py",
        "runs": res,
        "mean": {k: float(np.mean([r[k] for r in res])) for k in keys},
        "std": {k: float(np.std([r[k] for r in res], ddof=1)) for k in keys},
    }
    with open(OUT, "w") as f:
        json.dump(doc, f, indent=1)
    print(json.dumps({"mean": doc["mean"], "std": doc["std"]}, indent=1))


if __name__ == "__main__":
    main()
