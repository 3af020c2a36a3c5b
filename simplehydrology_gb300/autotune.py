"""Launch-shape autotuner for the batched mode.

The batched kernel's launch shape changes its speed, never its results:

* the CTA size (64, 128 or 256 threads), hence how many drops each CTA owns
  at full residency;
* the grid (every resident CTA, or one CTA per SM), hence also the drops per
  CTA;
* whether a cycle's drops are dealt to the CTAs in spawn-cell order;
* whether a CTA's drop slots may live in shared memory (when they fit) or
  always in global memory;
* how many cycles run as one CUDA graph;
* how often the live drops are re-dealt to the CTAs, sorted by their cell
  (slots in global memory only).

`autotune` tries candidate shapes on copies of a world's current state
(through a checkpoint file), times each over `cycles` cycles with CUDA
events on the copy's stream, and applies the fastest to the world; then,
with that shape, it times each cycles-per-graph setting the same way, and
with both, each re-deal interval.
"""
from __future__ import annotations

import os
import tempfile

from . import Batch, World, load

BLOCKS = (64, 128, 256)
ORDERS = (-1, 0, 1)
GRAPHS = (0, 1, 4, 16)  # cycles per CUDA graph (0: launched one by one)
RESORTS = (-1, 0, 4, 64)  # steps between re-deals (-1: the library's default)


def sm_count(device: int | None = None) -> int:
    """The SM count of the current (or given) CUDA device."""
    import torch
    dev = torch.cuda.current_device() if device is None else device
    return int(torch.cuda.get_device_properties(dev).multi_processor_count)


def candidates(sms: int | None = None, blocks=BLOCKS, orders=ORDERS, smem=(1, 0)):
    """(grid, order, block, smem_slots) shapes: CTA sizes x (every resident
    CTA, or one per SM) x the three order settings (-1 automatic, 0 drop
    order, 1 spawn-cell order) x drop slots in shared memory where they fit
    or always in global memory."""
    sms = sm_count() if sms is None else int(sms)
    out = []
    for block in blocks:
        for grid in (0, sms):
            for order in orders:
                for sm in smem:
                    out.append((grid, order, block, sm))
    return out


def _full(shape):
    """(grid, order[, block[, smem_slots]]) with the defaults (256, 1) filled in."""
    s = tuple(shape)
    return s + (256, 1)[len(s) - 2:]


def apply(world, shape):
    """Set a (grid, order, block, smem_slots) shape on a World or Batch."""
    grid, order, block, smem = _full(shape)
    world.set_launch(grid, order)
    world.set_block(block, smem)


def _time(path, shape, graph, drops, cycles, warm, resort=-1):
    """Seconds per cycle of `cycles` cycles on a copy of the checkpoint, after
    `warm` untimed cycles (which also capture any graph)."""
    import torch
    w = load(path)
    try:
        apply(w, shape)
        w.set_graph(graph)
        w.set_resort(resort)

        def erode(n):
            if isinstance(w, Batch):
                w.erode(n)
            else:
                w.erode(drops, n)

        erode(warm)
        w.sync()
        stream = torch.cuda.ExternalStream(w.stream())
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record(stream)
        erode(cycles)
        ev[1].record(stream)
        w.sync()
        return ev[0].elapsed_time(ev[1]) / 1e3 / cycles
    finally:
        w.close()


def autotune(world, drops: int | None = None, cycles: int = 3, shapes=None, sms: int | None = None,
             graphs=GRAPHS, resorts=RESORTS):
    """Time `cycles` batched cycles (at least 3) for each launch shape on a
    copy of `world`'s state and apply the fastest shape to `world`; then time
    each cycles-per-graph setting in `graphs` with that shape (over at least
    the largest setting's cycles) and apply the fastest; then each re-deal
    interval in `resorts` with both, and apply the fastest.  `drops` is the
    drops per cycle for a single-terrain World (a Batch keeps its own).
    Returns (best_shape, {shape: seconds per cycle}); the graph choice and
    its timings are in the attribute `autotune.last_graphs`, the re-deal
    choice and its timings in `autotune.last_resorts`."""
    if isinstance(world, World) and drops is None:
        raise ValueError("drops per cycle is needed for a World")
    cycles = max(3, int(cycles))
    shapes = list(shapes) if shapes is not None else candidates(sms)
    shapes = [_full(s) for s in shapes]
    fd, path = tempfile.mkstemp(suffix=".ckpt")
    os.close(fd)
    times, gtimes, rtimes = {}, {}, {}
    try:
        world.save(path)
        for shape in shapes:
            times[shape] = _time(path, shape, 0, drops, cycles, 1)
        best = min(times, key=times.get)
        # every setting warms up over the same cycles (enough to capture the
        # largest graph) and is timed over the same later ones: later cycles
        # carry fewer drop-steps, so unequal windows would favour one setting
        gc = max([cycles] + [int(g) for g in graphs])
        gw = max([1] + [int(g) for g in graphs])
        for g in graphs:
            gtimes[int(g)] = _time(path, best, int(g), drops, gc, gw)
        graph = min(gtimes, key=gtimes.get) if gtimes else 0
        for r in resorts:
            rtimes[int(r)] = _time(path, best, graph, drops, gc, gw, int(r))
    finally:
        os.remove(path)
    apply(world, best)
    world.set_graph(graph)
    resort = min(rtimes, key=rtimes.get) if rtimes else -1
    world.set_resort(resort)
    autotune.last_graphs = (graph, gtimes)
    autotune.last_resorts = (resort, rtimes)
    return best, times


autotune.last_graphs = (0, {})
autotune.last_resorts = (-1, {})
