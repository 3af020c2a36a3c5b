"""Launch-shape autotuner for the batched mode.

The batched kernel's launch shape -- how many CTAs (so how many drops each
CTA owns, and whether their slots fit in shared memory) and whether a
cycle's drops are ordered by spawn cell -- changes its speed, never its
results.  `autotune` tries candidate shapes on copies of a world's current
state (through a checkpoint file) and applies the fastest to the world.
"""
from __future__ import annotations

import os
import tempfile
import time

from . import Batch, World, load


def candidates(sm_count: int = 152):
    """(grid, order) pairs: every resident CTA or one per SM, and the three
    order settings (-1 automatic, 0 drop order, 1 spawn-cell order)."""
    out = []
    for grid in (0, sm_count):
        for order in (-1, 0, 1):
            out.append((grid, order))
    return out


def autotune(world, drops: int | None = None, cycles: int = 1, shapes=None, sm_count: int = 152):
    """Time `cycles` batched cycles for each launch shape on a copy of
    `world`'s state and apply the fastest shape to `world`.  `drops` is the
    drops per cycle for a single-terrain World (a Batch keeps its own).
    Returns (best_shape, {shape: seconds})."""
    if isinstance(world, World) and drops is None:
        raise ValueError("drops per cycle is needed for a World")
    shapes = list(shapes) if shapes is not None else candidates(sm_count)
    fd, path = tempfile.mkstemp(suffix=".ckpt")
    os.close(fd)
    times = {}
    try:
        world.save(path)
        for shape in shapes:
            w = load(path)
            try:
                w.set_launch(*shape)
                if isinstance(w, Batch):
                    w.erode(1)  # first launch of this shape (attribute set-up)
                else:
                    w.erode(drops, 1)
                w.sync()
                t0 = time.perf_counter()
                if isinstance(w, Batch):
                    w.erode(cycles)
                else:
                    w.erode(drops, cycles)
                w.sync()
                times[shape] = time.perf_counter() - t0
            finally:
                w.close()
    finally:
        os.remove(path)
    best = min(times, key=times.get)
    world.set_launch(*best)
    return best, times
