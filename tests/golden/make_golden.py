"""Generate the golden fixtures in this directory from the REFERENCE itself.

The reference's erosion headers are compiled unmodified into
oracle/_ref/libshyref.so (oracle/Makefile, oracle/ref_harness.cpp); this
script drives that build through its own entry points -- World::erode,
Drop::descend, World::cascade, quad::map::normal -- on the reference's
512 x 512 map and records what it returns:

  ref_traces.npz   per-step drop traces (8 floats per descend() call:
                   returned, age, pos.x, pos.y, speed.x, speed.y, volume,
                   sediment) from 12 spawns on the fresh terrain and 8 spawns
                   on the terrain after the erosion calls below, plus a
                   SHA-256 of the height map after each of those drops
  ref_erode.json   srand(1); World::erode(512) four times: SHA-256 of all 8
                   cell fields after every call, field sums, the budget
  ref_cascade.json World::cascade at 10 positions of a rough map
  ref_normals.json SHA-256 of quad::map::normal over the whole terrain
  ref_frames.json  the front end's frame loop: srand(5), then 40 times
                   World::erode(512); Vegetation::grow(); -- SHA-256 of all 8
                   cell fields and of the plant list (x, y, size per plant),
                   and the plant count
  ref_feed.json    the per-frame buffers on the map after those frames: the
                   mesh written by the reference's updatenode and the two
                   textures over its map accessors (SHA-256 each)
  ref_terrain.json the reference's own terrain, World::map.init for five
                   seeds (one child process each): SHA-256 of the 512 x 512
                   heights and every 4099th value

The input terrain is the workloads' value noise (seed 1) written over the
reference's own map after World::map.init.  Values that go through erf (the
discharge-coupled parts after the first erosion call) are the host C
library's erff; these fixtures were made with glibc 2.39 on x86-64.

Run from the repository root:  python tests/golden/make_golden.py
(`python tests/golden/make_golden.py terrain` rewrites ref_terrain.json only).
"""
import hashlib
import json
import os
import platform
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle as po  # noqa: E402

N = 512
SEED = 1


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


def main():
    po.build()
    assert po.ref_available(), "oracle/_ref/libshyref.so was not built (needs the reference checkout)"
    R = po.ref()
    assert R.ref_tilesize() == N
    order = R.ref_spawn_arg_order()
    H = po.value_noise(N, N, SEED)
    base = po.Maps(N, N, height=H)

    rng = np.random.default_rng(0)
    spawns_fresh = []
    while len(spawns_fresh) < 12:
        x, y = rng.integers(0, N, 2)
        if H[x, y] >= 0.1:
            spawns_fresh.append((float(x) + 0.5, float(y) + 0.25))
    traces = {}
    post_sha = {}
    for i, (x, y) in enumerate(spawns_fresh):
        po.ref_set_maps(base)
        traces[f"fresh_{i}"] = po.ref_drop_run(x, y)
        post_sha[f"fresh_{i}"] = sha(po.ref_get_maps().height)

    po.ref_set_maps(base)
    R.ref_srand(SEED)
    erode = {"order": order, "calls": []}
    h0 = H.astype(np.float64).sum()
    for c in range(4):
        R.ref_erode(512)
        m = po.ref_get_maps()
        erode["calls"].append({
            "sha": {f: sha(m.f[k]) for k, f in enumerate(po.FIELDS)},
            "sum": {f: float(m.f[k].astype(np.float64).sum()) for k, f in enumerate(po.FIELDS)},
        })
    eroded = po.ref_get_maps()
    erode["height_change"] = float(eroded.height.astype(np.float64).sum() - h0)

    spawns_eroded = []
    while len(spawns_eroded) < 8:
        x, y = rng.integers(0, N, 2)
        if eroded.height[x, y] >= 0.1 and eroded.discharge[x, y] > 0.0:
            spawns_eroded.append((float(x) + 0.75, float(y) + 0.5))
    for i, (x, y) in enumerate(spawns_eroded):
        po.ref_set_maps(eroded)
        traces[f"eroded_{i}"] = po.ref_drop_run(x, y)
        post_sha[f"eroded_{i}"] = sha(po.ref_get_maps().height)

    rough = po.Maps(N, N, height=(np.random.default_rng(7).random((N, N)) ** 3).astype(np.float32))
    po.ref_set_maps(rough)
    pts = [(0.5, 0.5), (511.9, 511.2), (100.0, 200.0), (300.7, 0.0), (-0.5, 3.0), (255.5, 255.5),
           (1.0, 510.0), (100.0, 200.0), (17.3, 480.9), (400.0, 400.0)]
    for x, y in pts:
        R.ref_cascade(x, y)
    cascade = {"points": pts, "height_sha": sha(po.ref_get_maps().height), "rough_seed": 7}

    nm = np.zeros((N, N, 3), np.float32)
    out = np.zeros(3, np.float32)
    po.ref_set_maps(base)
    for x in range(N):
        for y in range(N):
            R.ref_normal(x, y, po.fptr(out))
            nm[x, y] = out
    normals = {"sha": sha(nm)}

    # the frame loop: erosion and plant agents from one rand() stream
    frames = {"seed": 5, "frames": 40, "drops": 512, "terrain_seed": 11, "order": order}
    fm = po.Maps(N, N, height=po.value_noise(N, N, frames["terrain_seed"]))
    po.ref_set_maps(fm)
    R.ref_veg_clear()
    R.ref_srand(frames["seed"])
    for _ in range(frames["frames"]):
        R.ref_erode(frames["drops"])
        R.ref_veg_grow()
    fmaps = po.ref_get_maps()
    pl = np.zeros((1 << 16, 3), np.float32)
    n_pl = R.ref_veg_get(po.fptr(pl), 1 << 16)
    frames["field_sha"] = {f: sha(fmaps.f[k]) for k, f in enumerate(po.FIELDS)}
    frames["plants"] = n_pl
    frames["plants_sha"] = sha(pl[:n_pl])
    R.ref_veg_clear()

    v = np.zeros((N, N, 12), np.float32)
    d4 = np.zeros((N, N, 4), np.float32)
    m4 = np.zeros((N, N, 4), np.float32)
    R.ref_frame(po.fptr(v), po.fptr(d4), po.fptr(m4))
    feed = {"on": "the map after the frame loop of ref_frames.json", "vertices_sha": sha(v),
            "discharge_rgba_sha": sha(d4), "momentum_rgba_sha": sha(m4)}

    meta = {"generator": "tests/golden/make_golden.py", "map": N, "terrain_seed": SEED,
            "machine": platform.machine(), "libc": " ".join(platform.libc_ver())}
    np.savez_compressed(os.path.join(HERE, "ref_traces.npz"),
                        spawns_fresh=np.array(spawns_fresh, np.float32),
                        spawns_eroded=np.array(spawns_eroded, np.float32), **traces)
    with open(os.path.join(HERE, "ref_traces_post.json"), "w") as f:
        json.dump({"meta": meta, "post_height_sha": post_sha}, f, indent=1)
    with open(os.path.join(HERE, "ref_erode.json"), "w") as f:
        json.dump({"meta": meta, **erode}, f, indent=1)
    with open(os.path.join(HERE, "ref_cascade.json"), "w") as f:
        json.dump({"meta": meta, **cascade}, f, indent=1)
    with open(os.path.join(HERE, "ref_normals.json"), "w") as f:
        json.dump({"meta": meta, **normals}, f, indent=1)
    with open(os.path.join(HERE, "ref_frames.json"), "w") as f:
        json.dump({"meta": meta, **frames}, f, indent=1)
    with open(os.path.join(HERE, "ref_feed.json"), "w") as f:
        json.dump({"meta": meta, **feed}, f, indent=1)
    print("wrote fixtures:", sorted(os.listdir(HERE)))


TERRAIN_SEEDS = [1, 42, 12345, -7, 2147483647]


def terrain():
    po.build()
    assert po.ref_available(), "oracle/_ref/libshyref.so was not built (needs the reference checkout)"
    out = {}
    for s in TERRAIN_SEEDS:
        h = po.ref_terrain(s)
        assert h.shape == (N, N)
        out[str(s)] = {"height_sha": sha(h), "sample_every": 4099,
                       "sample": [float(v) for v in h.reshape(-1)[::4099]]}
    meta = {"generator": "tests/golden/make_golden.py terrain", "map": N,
            "what": "World::map.init(vertexpool, cellpool, SEED) heights, x-major",
            "machine": platform.machine()}
    with open(os.path.join(HERE, "ref_terrain.json"), "w") as f:
        json.dump({"meta": meta, "seeds": out}, f, indent=1)
    print("wrote ref_terrain.json")


if __name__ == "__main__":
    if sys.argv[1:] == ["terrain"]:
        terrain()
    else:
        main()
        terrain()
