"""Generate tests/golden/headline_stats.json: the batched mode's fidelity
fixture at the headline size (1024^2 value-noise terrain, seed 2, 65,536
drops per cycle, 20 cycles).

It runs, on the CPU oracle (oracle/hydro_oracle.cpp, whose sequential
restatement equals the reference build bit for bit):

* the reference's sequential World::erode (source/world.h:54-88), one call
  of 65,536 drops per cycle, for three spawn streams (srand seeds 1, 2, 3 of
  the C-library generator the reference's spawns use, source/world.h:69);
* the batched (lock-step) schedule the GPU runs, for the world seed 2.

For each run it stores the hypsometry, slope and log1p-discharge histograms
after cycles 10 and 20, the FP64 height budget (sum of height changes,
evaporation gain, boundary loss) and the drop-steps per cycle.  For the
batched run it also stores the SHA-256 of every field's float bits after 20
cycles, so that a GPU test can check the engine against the oracle bit for
bit at this size.  Takes about five minutes on four cores:

    python tests/golden/make_headline_stats.py
"""
from __future__ import annotations

import hashlib
import json
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

N, DROPS, CYCLES, TERRAIN_SEED, WORLD_SEED = 1024, 65536, 20, 2, 2
SPAWN_SEEDS = (1, 2, 3)
CHECKPOINTS = (10, 20)
OUT = os.path.join(HERE, "headline_stats.json")


def hists(h, d):
    """Hypsometry (40 bins on [0, 1]), slope (central differences, 40 bins
    on [0, 0.03]) and log1p discharge (40 bins on [0, 7]), as fractions of
    the cells."""
    h = np.asarray(h, np.float64)
    gx = np.zeros_like(h)
    gy = np.zeros_like(h)
    gx[1:-1] = (h[2:] - h[:-2]) / 2
    gy[:, 1:-1] = (h[:, 2:] - h[:, :-2]) / 2
    slope = np.hypot(gx, gy)
    return [(np.histogram(h, 40, (0, 1))[0] / h.size).tolist(),
            (np.histogram(slope, 40, (0, 0.03))[0] / h.size).tolist(),
            (np.histogram(np.log1p(np.asarray(d, np.float64)), 40, (0, 7))[0] / h.size).tolist()]


def sequential(spawn_seed):
    from oracle import pyoracle as po
    H = po.value_noise(N, N, TERRAIN_SEED)
    m = po.Maps(N, N, height=H)
    sp = po.rand_spawns(spawn_seed, DROPS * CYCLES, N, N, 1)
    out = {"spawn_seed": spawn_seed, "steps_per_cycle": [], "gain": 0.0, "loss": 0.0}
    for c in range(CYCLES):
        a = po.erode_seq(m, sp[c * DROPS:(c + 1) * DROPS])
        out["steps_per_cycle"].append(int(a.steps))
        out["gain"] += a.gain
        out["loss"] += a.loss
        if c + 1 in CHECKPOINTS:
            out[f"hists_c{c + 1}"] = hists(m.height, m.discharge)
    out["dh"] = float(m.height.astype(np.float64).sum() - H.astype(np.float64).sum())
    return out


def batched():
    from oracle import pyoracle as po
    H = po.value_noise(N, N, TERRAIN_SEED)
    m = po.Maps(N, N, height=H)
    hq = np.zeros((N, N), np.int64)
    out = {"world_seed": WORLD_SEED, "steps_per_cycle": [], "gain_q": 0, "loss_q": 0, "drops": 0, "oob": 0}
    for c in range(CYCLES):
        a = po.erode_batched(m, WORLD_SEED, c, DROPS, 1, hq=hq)
        out["steps_per_cycle"].append(int(a.steps))
        out["gain_q"] += int(a.gain_q)
        out["loss_q"] += int(a.loss_q)
        out["drops"] += int(a.drops)
        out["oob"] += int(a.oob)
        if c + 1 in CHECKPOINTS:
            out[f"hists_c{c + 1}"] = hists(m.height, m.discharge)
    out["dh"] = float(m.height.astype(np.float64).sum() - H.astype(np.float64).sum())
    out["sha256"] = {name: hashlib.sha256(np.ascontiguousarray(m.f[k], np.float32).tobytes()).hexdigest()
                     for k, name in enumerate(po.FIELDS)}
    return out


def _run(job):
    return batched() if job == "batched" else sequential(job)


def l1(a, b):
    return [0.5 * float(np.abs(np.asarray(x) - np.asarray(y)).sum()) for x, y in zip(a, b)]


def main():
    from oracle import pyoracle as po
    po.build()
    jobs = ["batched"] + list(SPAWN_SEEDS)
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        res = pool.map(_run, jobs)
    bat, seq = res[0], res[1:]
    summary = {}
    for cp in CHECKPOINTS:
        key = f"hists_c{cp}"
        pairs = [l1(seq[i][key], seq[j][key]) for i in range(len(seq)) for j in range(i + 1, len(seq))]
        spread = np.mean(pairs, axis=0).tolist()
        dist = np.mean([l1(bat[key], s[key]) for s in seq], axis=0).tolist()
        summary[key] = {"sequential_seed_spread_l1": spread, "batched_to_sequential_l1": dist}
    doc = {
        "what": "batched-mode fidelity at the headline size: the reference's sequential World::erode "
                "(oracle restatement, bit-exact with the reference) for three spawn streams, and the batched "
                "lock-step schedule the GPU runs; histograms are fractions of cells (hypsometry, slope, log1p "
                "discharge), L1 distances are half the summed absolute bin differences",
        "config": {"map": [N, N], "terrain": f"value noise seed {TERRAIN_SEED}, 8 octaves", "drops_per_cycle": DROPS,
                   "cycles": CYCLES, "spawn_seeds": list(SPAWN_SEEDS), "world_seed": WORLD_SEED,
                   "checkpoints": list(CHECKPOINTS)},
        "generator": "tests/golden/make_headline_stats.py",
        "sequential": seq,
        "batched_oracle": bat,
        "summary": summary,
    }
    with open(OUT, "w") as f:
        json.dump(doc, f, indent=1)
    print(json.dumps(summary, indent=1))


if __name__ == "__main__":
    main()
