"""Benchmark of the erosion hot path: drop-steps/s on one GB300.

Workload (the plain-method GPU configuration): a 1024 x 1024 fp32 heightmap
of seeded fractal value noise (8 octaves, lacunarity 2, gain 0.5, normalised
to [0, 1], seed 2), 65,536 drops per cycle with uniform random spawns, the
reference's default Drop/World parameters, 32.32 fixed-point integer-atomic
scatter, lrate blend and cascade.  One step = one erosion cycle
(World::erode(65536), source/world.h:54-88).  Synthetic data: there is no
dataset; the terrain recipe stands in for the reference's FastNoiseLite map.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload plain|batch|converge|large|surrogate|surrogate-step]

`value` is device throughput with the maps resident in HBM; between timed
steps the L2 is flushed by writing a 256 MiB buffer (untimed).  `e2e` is the
same metric through the C ABI with the world state (height, discharge,
momentum) copied in from pinned host memory and back out every step.  The
reference arm runs the reference's sequential erosion on the host cores.

`roofline` takes the lock-step kernel's algorithmic bytes (72 B per
drop-step) against the HBM copy peak; `roofline_l2` takes the same bytes, and
4 integer atomics per drop-step, against the L2 peaks the library measures
on the GPU at hand (shy_measure_l2), which bound the kernel while a
terrain's cell state fits in L2.  `cycle_gbs` adds the 80 B per cell of the
end-of-cycle pass over the whole step time.

`--workload converge` measures the plain method's time to converged
discharge (within 5 % log-L2 of the discharge after 4 x 500 cycles).

`--workload surrogate` trains the learned warm-start on the device and
compares the time to converged discharge with and without it (`--warm-scales`
tries scaled warm starts; `--save-net` / `--load-net` keep the network);
`--workload surrogate-conv` times the largest convolution per tile setting;
`--workload surrogate-step` times its training step alone (TFLOP/s).

`--workload large` runs the large-scale configuration: 8192^2, 4,194,304
drops per cycle, per-cell vegetation every cycle.

`--workload batch` runs the batched-terrain configuration instead: 64
terrains, sides log-uniform in [128, 1024], 0.25 drops per cell per cycle,
one lock-step launch per cycle; with N ranks each erodes a disjoint share of
whole terrains.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX = NY = 1024
DROPS = 65536
SEED = 2
METRIC = "drop-steps/s"
WORKLOAD = "plain method, GPU batched: 1024x1024 value-noise terrain, 65536 drops/cycle"
# algorithmic bytes: 72 B per drop-step (5 own-cell f32 fields, 4 neighbour
# heights and h2 = 40 B read; height delta and 3 tracks = 32 B of scatter) and
# 80 B per cell per cycle (tracks read + reset, 3 fields read + write, height)
BYTES_PER_STEP = 72
BYTES_PER_CELL_CYCLE = 80
FALLBACK_HBM_GBS = 6800.0


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def profiled_traffic(name="lockstep_kernel_1024.md"):
    """Per-launch DRAM bytes of the lock-step kernel from a committed ncu summary."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch:"):
                    return float(line.split(":", 1)[1])
    except Exception:
        pass
    return None


class ClockSampler:
    """nvidia-smi samples during the timed region (200 ms period)."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
def dist_setup(n_gpus):
    if n_gpus <= 1 or "RANK" not in os.environ:
        return 0, 1, None
    import torch
    import torch.distributed as dist
    rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, world, dist


def cpu_baseline_sample(seconds=10.0):
    """The oracle's restatement of the reference's sequential World::erode
    (pinned bit for bit against the reference) timed on one host core on a
    bounded sample of the workload: 1024^2 terrain, drops in batches of 512."""
    import numpy as np
    from oracle import pyoracle as po
    po.build()
    H = po.value_noise(NX, NY, SEED)
    m = po.Maps(NX, NY, height=H)
    rng = np.random.default_rng(SEED)
    steps = drops = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        sp = np.stack([rng.integers(0, NX, 512), rng.integers(0, NY, 512)], 1)
        a = po.erode_seq(m, sp)
        steps += a.steps
        drops += 512
    dt = time.perf_counter() - t0
    return {"value": steps / dt, "unit": METRIC, "cores": 1, "kind": "port",
            "sample": f"{drops} drops of World::erode on the 1024^2 terrain ({steps} drop-steps, {dt:.1f} s, 1 thread)"}


class PlainWorkload:
    """One terrain: the 1024^2 / 65,536-drop configuration (or a smaller
    profiling case).  One step = one World::erode(drops) cycle."""

    def __init__(self, shy, n, drops):
        self.w = shy.World(n, n, seed=SEED)
        self.w.generate(SEED, 8)
        self.h0 = self.w.get_field("height")
        self.zero = self.h0 * 0.0
        self.drops = drops
        self.cells = n * n
        self.config = {"workload": WORKLOAD if (n, drops) == (1024, 65536) else
                       f"profiling case: {n}x{n} value-noise terrain, {drops} drops/cycle",
                       "map": [n, n], "drops_per_cycle": drops}

    def erode(self):
        self.w.erode(self.drops)

    def reset(self):
        self.w.set_field("height", self.h0)
        for f in ("discharge", "momentum_x", "momentum_y"):
            self.w.set_field(f, self.zero)
        self.w.set_cycle(0)

    def host_buffers(self, torch):
        bufs = {}
        for f in FIELDS:
            b = torch.empty(self.h0.shape, dtype=torch.float32, pin_memory=True).numpy()
            b[...] = self.h0 if f == "height" else 0.0
            bufs[f] = b
        return bufs

    def upload(self, bufs):
        self.w.set_state(0, **bufs)

    def download(self, bufs):
        self.w.get_state(0, out=bufs)


class LargeWorkload(PlainWorkload):
    """The large-scale configuration: an 8192^2 terrain, 4,194,304 drops per
    cycle, per-cell vegetation (spawn probability 1e-4 per cell per cycle)
    coupled to erosion through the root density.  One step = one erosion
    cycle followed by one vegetation step."""

    def __init__(self, shy, n, drops):
        super().__init__(shy, n, drops)
        self.config = {"workload": f"large scale: {n}x{n} value-noise terrain, {drops} drops/cycle, "
                                   "per-cell vegetation each cycle", "map": [n, n], "drops_per_cycle": drops}

    def erode(self):
        self.w.erode(self.drops)
        self.w.vegetation_step(1)

    def reset(self):
        super().reset()
        self.w.set_field("root_density", self.zero)
        self.w.set_field("plant_size", self.zero)


class BatchWorkload:
    """This rank's share of the batched-terrain configuration: 64 terrains
    with sides log-uniform in [128, 1024], 0.25 drops per cell per cycle, all
    eroded by one lock-step launch per cycle.  Terrains are split over ranks
    whole (no exchange).  One step = one cycle of every terrain."""

    def __init__(self, shy, rank, world_size, n_terrains):
        from simplehydrology_gb300 import sharding
        self.specs = sharding.rank_terrains(sharding.batch_workload(n_terrains), world_size, rank)
        self.w = shy.Batch([(t.nx, t.ny) for t in self.specs], [t.drops for t in self.specs],
                           [t.seed for t in self.specs])
        self.h0 = []
        for i, t in enumerate(self.specs):
            self.w.generate(i, t.seed, 8)
            self.h0.append(self.w.get_field(i, "height"))
        self.cells = sum(t.cells for t in self.specs)
        self.config = {"workload": f"batched terrains: {n_terrains} value-noise terrains, sides log-uniform in "
                                   f"[128, 1024], 0.25 drops/cell/cycle, one launch per cycle",
                       "terrains_this_rank": len(self.specs), "cells_this_rank": self.cells,
                       "drops_per_cycle_this_rank": sum(t.drops for t in self.specs)}

    def erode(self):
        self.w.erode(1)

    def reset(self):
        for i, t in enumerate(self.specs):
            self.w.set_field(i, "height", self.h0[i])
            z = self.h0[i] * 0.0
            for f in ("discharge", "momentum_x", "momentum_y"):
                self.w.set_field(i, f, z)
        self.w.set_cycle(0)

    def host_buffers(self, torch):
        # every terrain's cells back to back, one pinned array per field: the
        # whole batch's state moves in one call each way (shy_world_set_state)
        import numpy as np
        flat = np.concatenate([np.asarray(h, np.float32).reshape(-1) for h in self.h0])
        bufs = {}
        for f in FIELDS:
            b = torch.empty(flat.shape, dtype=torch.float32, pin_memory=True).numpy()
            b[...] = flat if f == "height" else 0.0
            bufs[f] = b
        return bufs

    def upload(self, bufs):
        self.w.set_state_all(**bufs)

    def download(self, bufs):
        self.w.get_state_all(out=bufs)


FIELDS = ("height", "discharge", "momentum_x", "momentum_y")


def run_ours(args):
    import torch

    import simplehydrology_gb300 as shy
    from simplehydrology_gb300 import build as shybuild
    from simplehydrology_gb300 import sharding

    shybuild.build()
    rank, world_size, dist = dist_setup(args.gpus)
    dev = torch.cuda.current_device()

    if args.workload == "batch":
        wl = BatchWorkload(shy, rank, world_size, args.terrains)
    elif args.workload == "large":
        wl = LargeWorkload(shy, 8192 if args.map == NX else args.map,
                           4194304 if args.drops == DROPS else args.drops)
    else:
        wl = PlainWorkload(shy, args.map, args.drops)
    w = wl.w
    if args.resort is not None:
        w.set_resort(args.resort)

    # optional: the launch-shape autotuner on the initial state (each
    # candidate timed over 3 cycles on a checkpoint copy); the bench then
    # runs with the fastest shape
    tune = None
    if args.autotune:
        from simplehydrology_gb300 import autotune
        best, times = autotune.autotune(w, None if args.workload == "batch" else wl.drops, cycles=3)
        graph, gtimes = autotune.autotune.last_graphs
        tune = {"best": list(best), "ms_per_cycle": {"x".join(str(v) for v in k): round(t * 1e3, 4)
                                                      for k, t in sorted(times.items(), key=lambda kv: kv[1])},
                "shape": "grid x order x block x smem_slots (grid 0: every resident CTA)",
                "cycles_per_graph": graph, "ms_per_cycle_by_graph": {g: round(t * 1e3, 4) for g, t in gtimes.items()},
                "resort": autotune.autotune.last_resorts[0],
                "ms_per_cycle_by_resort": {r: round(t * 1e3, 4) for r, t in autotune.autotune.last_resorts[1].items()}}

    # warm-up on the same workload, then restart from the initial terrain
    for _ in range(args.warmup):
        wl.erode()
    wl.reset()
    w.reset_stats()

    stream = torch.cuda.ExternalStream(w.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    stops = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    w.enable_timing(True)
    ph0, it0 = w.lockstep_profile()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    with ClockSampler(dev) as clk:
        wall0 = time.perf_counter()
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xFF)        # untimed L2 flush
                starts[k].record(stream)
            wl.erode()
            with torch.cuda.stream(stream):
                stops[k].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, stops)]
    dev_s = sum(step_ms) / 1e3
    st = w.stats()
    tm = w.timing()
    ph1, it1 = w.lockstep_profile()
    w.enable_timing(False)
    steps_total = st.drop_steps
    steps_all, dev_s_max = sharding.aggregate(steps_total, dev_s, dist)
    value = steps_all / dev_s_max

    # roofline of the dominant kernel (the lock-step drops kernel): the
    # algorithmic bytes against the HBM copy peak, and against the L2 peaks
    # that bound it when the cell state fits in L2
    n_launch = max(1, tm.launches[0])
    avg_ms = tm.ms[0] / n_launch
    bytes_per_launch = BYTES_PER_STEP * steps_total / n_launch
    achieved = bytes_per_launch / (avg_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    # the committed captures cover the default 1024^2 / 65,536-drop workload
    # and the default large workload (its three timed cycles, re-deal on)
    plain_default = args.workload == "plain" and (args.map, args.drops) == (1024, 65536)
    large_default = args.workload == "large" and (args.map, args.drops) == (NX, DROPS) and args.resort is None
    traffic = (profiled_traffic() if plain_default else
               profiled_traffic("lockstep_kernel_8192_dram.md") if large_default else None)
    l2 = shy.measure_l2(dev)
    kernel_s = tm.ms[0] / 1e3
    atomics = 4.0 * steps_total / kernel_s
    cycle_bytes = BYTES_PER_STEP * steps_total + BYTES_PER_CELL_CYCLE * wl.cells * args.steps

    # end to end through the C ABI with pinned host buffers: each step copies
    # the world state in, erodes one cycle and copies it back out
    # the same cycles as the device-timed steps (the terrain, hence the
    # drop-steps per cycle, changes from cycle to cycle)
    e2e_steps = 0 if args.no_e2e else args.steps
    e2e_value, nbytes = None, 0
    if e2e_steps:
        bufs = wl.host_buffers(torch)
        wl.reset()
        w.reset_stats()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(e2e_steps):
            wl.upload(bufs)
            wl.erode()
            wl.download(bufs)
        e2e_s = time.perf_counter() - t0
        e2e_units, e2e_s = sharding.aggregate(w.stats().drop_steps, e2e_s, dist)
        e2e_value = e2e_units / e2e_s
        nbytes = wl.cells * 4 * len(FIELDS)

    # the whole workload beside the headline window: cycles 0 .. whole-1
    # from the initial terrain, device time (later cycles carry fewer
    # drop-steps as the terrain wears down)
    whole = None
    if args.workload == "plain" and args.whole_cycles > 0:
        # one World::erode call of every cycle, run as CUDA graphs of 16
        # cycles (the graph is captured by an untimed call first)
        w.set_graph(16)
        wl.reset()
        w.erode(wl.drops, 16)
        wl.reset()
        w.reset_stats()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            ev[0].record(stream)
        w.erode(wl.drops, args.whole_cycles)
        with torch.cuda.stream(stream):
            ev[1].record(stream)
        torch.cuda.synchronize()
        w.set_graph(0)
        whole_s = ev[0].elapsed_time(ev[1]) / 1e3
        ws_ = w.stats()
        whole = {"cycles": args.whole_cycles, "value": ws_.drop_steps / whole_s, "unit": METRIC,
                 "ms_per_cycle": whole_s * 1e3 / args.whole_cycles,
                 "drop_steps_per_cycle": ws_.drop_steps / args.whole_cycles,
                 "timing": "one shy_erode call of all cycles from the initial terrain, CUDA graphs of 16 cycles, "
                           "device time (CUDA events), no L2 flush"}

    config = dict(wl.config)
    config.update({"step": "one erosion cycle",
                   "cycles_timed": f"0-{args.steps - 1} of the workload, from the initial terrain",
                   "l2": "flushed between steps (256 MiB write, untimed)",
                   "redeal_steps": (args.resort if args.resort is not None else
                                    "library default: 16 with spawn-ordered slots in global memory, else none"),
                   "parallelism": (("terrain shards" if args.workload == "batch" else "replicas") +
                                   f" x{world_size}") if world_size > 1 else "single GPU"})
    out = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world_size,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_s_max * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded value-noise terrain, counter-based spawns)",
        "config": config,
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "steps": e2e_steps},
        "gpu_launches": int(sum(tm.launches)),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                     "kernel": "lockstep_kernel", "avg_launch_ms": avg_ms,
                     "algorithmic_bytes_per_launch": bytes_per_launch},
        "roofline_l2": {"achieved_gbs": achieved, "read_peak_gbs": l2["read_gbs"],
                        "frac": achieved / l2["read_gbs"],
                        "atomics_per_s": atomics, "red_peak_per_s": l2["red_per_s"],
                        "atomic_frac": atomics / l2["red_per_s"],
                        "random_sector_reads_peak_per_s": l2["random_sector_reads_per_s"],
                        "l2_bytes": l2["l2_bytes"], "peak_source": "shy_measure_l2 on this GPU"},
        "cycle_gbs": cycle_bytes / dev_s / 1e9,
        "kernel_ms": {"drops": tm.ms[0], "cycle_end": tm.ms[1], "relax": tm.ms[2]},
        "lockstep": {"iterations": it1 - it0,
                     "phase_ms": dict(zip(["descend", "wait_descend", "scan", "wait_scan", "settle", "wait_settle"],
                                          [b - a for a, b in zip(ph0, ph1)]))},
        "drop_steps": steps_total, "wall_s": wall,
    }
    if whole:
        out["whole_workload"] = whole
    if tune:
        out["autotune"] = tune
    out["clocks"] = clk.summary()
    if rank == 0 and world_size == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_sample(args.cpu_seconds)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out))


# ---------------------------------------------------------------------------
def _ref_worker(args):
    """One host core: the oracle's sequential World::erode on `n` drops per step."""
    idx, steps, warmup, n = args
    import numpy as np
    from oracle import pyoracle as po
    H = po.value_noise(NX, NY, SEED)
    m = po.Maps(NX, NY, height=H)
    rng = np.random.default_rng(1000 + idx)
    out = []
    for k in range(warmup + steps):
        sp = np.stack([rng.integers(0, NX, n), rng.integers(0, NY, n)], 1)
        t0 = time.perf_counter()
        a = po.erode_seq(m, sp)
        out.append((time.perf_counter() - t0, a.steps))
    return out[warmup:]


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp

    from oracle import pyoracle as po
    po.build()
    cores = os.cpu_count() or 1
    per = max(1, 4096 // cores)  # 4096 drops per step across all cores
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        t0 = time.perf_counter()
        res = pool.map(_ref_worker, [(i, args.steps, args.warmup, per) for i in range(cores)])
        wall = time.perf_counter() - t0
    steps = sum(s for r in res for _, s in r)
    busy = max(sum(t for t, _ in r) for r in res)
    value = steps / busy
    sample = (f"{args.steps} steps of {per} drops x {cores} host processes of the sequential "
              f"World::erode restatement (bit-exact with the reference) on the 1024^2 terrain")
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": busy * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded value-noise terrain)",
        "config": {"workload": WORKLOAD, "map": [NX, NY], "drops_per_step": per * cores,
                   "step": "a bounded sample of one erosion cycle"},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": wall,
    }
    print(json.dumps(out))


def run_converge(args):
    """Time to converged discharge of the plain method: the discharge map
    after k cycles against the one after `--ref-cycles` cycles (4 x the
    500-cycle workload by default), distance ||log1p(D_k) - log1p(D*)|| /
    ||log1p(D*)||; converged at the first k where it is at most 5 %.  The
    batched mode is deterministic, so one run gives D* and every D_k; the
    time is the device time of the first k cycles (CUDA events)."""
    import numpy as np
    import torch

    import simplehydrology_gb300 as shy
    from simplehydrology_gb300 import build as shybuild
    shybuild.build()
    dev = torch.cuda.current_device()
    n, drops = args.map, args.drops
    w = shy.World(n, n, seed=SEED)
    w.generate(SEED, 8)
    stream = torch.cuda.ExternalStream(w.stream())
    snaps, ms, diag = [], [], []
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    every = args.check_every
    steps0 = 0
    for c0 in range(0, args.ref_cycles, every):
        k = min(every, args.ref_cycles - c0)
        with torch.cuda.stream(stream):
            ev[0].record(stream)
        w.erode(drops, k)
        with torch.cuda.stream(stream):
            ev[1].record(stream)
        torch.cuda.synchronize()
        ms.append(ev[0].elapsed_time(ev[1]))
        d = w.get_field("discharge").astype(np.float64)
        snaps.append(np.log1p(d))
        h = w.get_field("height")
        st = w.stats()
        diag.append({"cycle": c0 + k, "height_mean": round(float(h.mean()), 5),
                     "cells_ge_0.1": round(float((h >= 0.1).mean()), 4), "discharge_mean": float(d.mean()),
                     "drop_steps_per_cycle": (st.drop_steps - steps0) / k})
        steps0 = st.drop_steps
    ref = snaps[-1]
    norm = float(np.linalg.norm(ref))
    # D* is meaningless once the terrain has worn below the spawn threshold
    # everywhere (source/world.h:71): no drop spawns and discharge decays to 0
    degenerate = diag[-1]["cells_ge_0.1"] == 0.0 or diag[-1]["drop_steps_per_cycle"] == 0
    dist = [float(np.linalg.norm(s - ref)) / norm if norm > 0 else float("inf") for s in snaps[:-1]]
    k_conv = None if degenerate else next((i for i, d in enumerate(dist) if d <= 0.05), None)
    cycles = (k_conv + 1) * every if k_conv is not None else None
    t = sum(ms[:k_conv + 1]) / 1e3 if k_conv is not None else None
    out = {"metric": "time to converged discharge (<=5% log-L2), plain method", "value": t, "unit": "s",
           "higher_is_better": False, "cycles_to_converge": cycles, "reference_cycles": args.ref_cycles,
           "log_l2_at_checks": [round(d, 5) for d in dist[:: max(1, len(dist) // 20)]],
           "diagnostics": diag[:: max(1, len(diag) // 20)],
           "ms_per_cycle": sum(ms) / args.ref_cycles, "n_gpus": 1, "dtype": "f32",
           "data": "synthetic (seeded value-noise terrain, counter-based spawns)",
           "config": {"workload": f"plain method, GPU batched: {n}x{n} value-noise terrain, {drops} drops/cycle",
                      "check_every_cycles": every},
           "surrogate": "compared in --workload surrogate"}
    if degenerate:
        out["degenerate"] = ("after %d cycles no cell is at height >= 0.1, so every spawn is skipped "
                             "(source/world.h:71) and the reference discharge D* has decayed to ~0" % args.ref_cycles)
    print(json.dumps(out))


def _discharge_run(shy, seed, n, drops, cycles, warm=None, spawn_seed=None, scale=1.0):
    """A plain run of `cycles` cycles on the value-noise terrain of `seed`
    from zero maps, or from the surrogate's maps when `warm` is given; the
    spawns follow `spawn_seed` (default `seed`).
    Returns (discharge after each cycle, device ms of each cycle, warm-start
    seconds: the prediction and the device-to-device map write, wall clock)."""
    import torch
    w = shy.World(n, n, seed=seed if spawn_seed is None else spawn_seed)
    w.generate(seed, 8)
    t_warm = 0.0
    if warm is not None:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        warm.warm_start(w, scale=scale)
        w.sync()
        t_warm = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(w.stream())
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ds, ms = [], []
    for _ in range(cycles):
        ev[0].record(stream)
        w.erode(drops, 1)
        ev[1].record(stream)
        ds.append(w.get_field("discharge"))
        ms.append(ev[0].elapsed_time(ev[1]))
    w.close()
    return ds, ms, t_warm


def run_surrogate(args):
    """The learned warm-start against the plain method: time to converged
    discharge on 1024^2 terrains.

    The plain method's discharge is a blend with lrate 0.1 of each cycle's
    tracks (source/world.h:83-85), so from zero maps it takes tens of cycles
    to settle, and it carries the spawn order's noise: two plain runs of one
    terrain with different spawns stay about 0.4 log-L2 apart.  So D* of a
    terrain is the mean discharge of cycles horizon+1 .. horizon+10 averaged
    over `spawn_runs` plain runs with different spawns, and each run is
    compared with the D* of the other runs (leave one out), never with one
    that contains itself.  A run's distance at cycle k is the log-L2 between
    the mean discharge of its last min(k, 10) cycles and that D*.  The floor
    is the distance the plain runs reach at the horizon; a run has converged
    at the first k where its distance is within 5 % of that floor
    (distance <= 1.05 x floor).  The strict reading, distance <= 0.05, is
    reported too.  The warm run starts from the surrogate's maps (written
    device to device) and its time includes the prediction.

    The surrogate is trained first, on pairs the batched GPU particle method
    generates: 256^2 value-noise terrains (seeds 10000+i), input the initial
    heightmap, targets the maps after `horizon` cycles at the same drop
    density (4,096 drops per cycle), averaged over `spawn_runs` spawn
    orders.  Evaluation terrains are 1024^2, seeds 20000+i."""
    import numpy as np
    import torch

    import simplehydrology_gb300 as shy
    from simplehydrology_gb300 import build as shybuild
    from simplehydrology_gb300 import surrogate as sg
    shybuild.build()
    torch.cuda.init()
    clock = ClockSampler(torch.cuda.current_device())
    clock.__enter__()
    horizon, theta, n_tr, n_val = args.horizon, 0.05, args.train_terrains, 64
    runs = args.spawn_runs
    side = args.train_side
    if side != 256:  # fewer, larger terrains, trained on random 256^2 crops
        n_tr, n_val = max(1, n_tr * 256 * 256 // (side * side)), max(1, 64 * 256 * 256 // (side * side))
    t0 = time.perf_counter()
    H, D, MX, MY = sg.make_pairs((0 if args.load_net else n_tr) + n_val, size=side, cycles=horizon,
                                 seed0=10000 + (n_tr if args.load_net else 0),
                                 per_launch=max(16, 64 * 256 * 256 // (side * side)), spawn_runs=runs)
    if args.load_net:  # the held-out pairs only; the network comes from the file
        pad = [np.zeros((n_tr,) + a.shape[1:], np.float32) for a in (H, D, MX, MY)]
        H, D, MX, MY = (np.concatenate([p_, a]) for p_, a in zip(pad, (H, D, MX, MY)))
    gen_s = time.perf_counter() - t0
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    batch = 16
    if args.load_net:
        net = sg.Surrogate(seed=0)
        net.load_state_dict(dict(np.load(args.load_net, allow_pickle=True)["state"].item()))
        losses, train_ms, launches0 = [], 0.0, net.launches
    else:
        norm = sg.Norm.fit(H[:n_tr], D[:n_tr], MX[:n_tr], MY[:n_tr])
        net = sg.Surrogate(seed=0, norm=norm)
        net.autotune(batch, 256, 256)
        launches0 = net.launches
        ev[0].record()
        losses = sg.train(net, H[:n_tr], D[:n_tr], MX[:n_tr], MY[:n_tr], epochs=args.epochs, batch=batch,
                          lr=2e-3, crop=256 if side != 256 else None,
                          steps_per_epoch=args.train_terrains // batch)
        ev[1].record()
        torch.cuda.synchronize()
        net.status()
        train_ms = ev[0].elapsed_time(ev[1])
        if args.save_net:
            np.savez(args.save_net, state=np.array(net.state_dict(), dtype=object))
    steps = args.epochs * (args.train_terrains // batch)
    train_flops = steps * batch * 256 * 256 * sg.flops_per_pixel(True) if train_ms else 0.0
    # held-out 256^2 pairs: the prediction against the particle method's maps
    val_pred, _, _ = net.predict(torch.from_numpy(H[n_tr:]).cuda())
    vp = val_pred.cpu().numpy()
    val = {"terrains": n_val, "log_l2_prediction": float(np.mean([sg.log_l2(vp[i], D[n_tr + i])
                                                                  for i in range(n_val)])),
           "log_l2_zero_maps": 1.0}

    # the dominant convolution shape alone: dec2a forward (384 -> 128 channels,
    # 3x3) at the training batch, level 2 of 256^2 (16 x 64 x 64 pixels)
    ws = net.workspace(batch, 256, 256, True)
    conv_flops = 2.0 * batch * 64 * 64 * 9 * 384 * 128
    reps, conv_paths = 20, {}
    for path, label in ((1, "staged"), (0, "tma")):
        shy._capi.check(shy.lib().shy_sg_set_conv_path(path))
        for _ in range(3):
            net._conv(ws, "dec2a", ws.cat[2], 384, ws.z["dec2a"], 128, 0, ws.a["dec2a"], 128, 0, sg.ACT_GELU)
        ev[0].record()
        for _ in range(reps):
            net._conv(ws, "dec2a", ws.cat[2], 384, ws.z["dec2a"], 128, 0, ws.a["dec2a"], 128, 0, sg.ACT_GELU)
        ev[1].record()
        torch.cuda.synchronize()
        conv_paths[label] = ev[0].elapsed_time(ev[1]) / reps
    net.status()
    conv_ms = conv_paths["tma"]
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            bf16_peak, peak_src = float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        bf16_peak, peak_src = 1900.0, "fallback"

    # warm start against plain on 1024^2 terrains
    n, drops, total = 1024, 65536, horizon + 10

    def window(ds, k):
        return np.mean(ds[max(0, k - 10):k], axis=0)

    def first(dist, bound):
        return next((k + 1 for k, d in enumerate(dist) if d <= bound), None)

    scales = [float(v) for v in args.warm_scales.split(",")]
    per = []
    for i in range(args.eval_terrains):
        seed = 20000 + i
        plain = [_discharge_run(shy, seed, n, drops, total, spawn_seed=seed + sg.SPAWN_STRIDE * r)
                 for r in range(runs)]
        finals = [np.mean(ds[horizon:], axis=0) for ds, _, _ in plain]
        # D* of run r: the other runs' mean (leave one out)
        dstar = [np.mean([f for q, f in enumerate(finals) if q != r], axis=0) for r in range(runs)]
        floor = float(np.mean([sg.log_l2(window(plain[r][0], horizon), dstar[r]) for r in range(runs)]))
        dp, mp, _ = plain[0]
        pred = net.predict(torch.from_numpy(_initial_height(shy, seed, n)[None]).cuda())[0][0].cpu().numpy()
        dist_p = [sg.log_l2(window(dp, k), dstar[0]) for k in range(1, total + 1)]
        d_pred = sg.log_l2(pred, dstar[0])
        bound = (1.0 + theta) * floor
        kp = first(dist_p, bound)
        tp = sum(mp[:kp]) / 1e3 if kp else None
        row = {"seed": seed, "floor": floor, "bound": bound, "cycles_plain": kp, "plain_s": tp,
               "log_l2_prediction": d_pred, "prediction_worth_plain_cycles": first(dist_p, d_pred),
               "strict_5pct_plain": first(dist_p, theta),
               "log_l2_plain_window": [round(d, 4) for d in dist_p[::5]],
               "ms_per_cycle": sum(mp) / len(mp), "warm": {}}
        for scale in scales:  # the spawn order of run 0
            dw_, mw, t_warm = _discharge_run(shy, seed, n, drops, total, warm=net, scale=scale)
            dist_w = [sg.log_l2(window(dw_, k), dstar[0]) for k in range(1, total + 1)]
            kw = first(dist_w, bound)
            tw = t_warm + sum(mw[:kw]) / 1e3 if kw else None
            row["warm"][str(scale)] = {"cycles_warm": kw, "warm_s": tw, "warm_start_s": t_warm,
                                       "speedup": (tp / tw) if tp and tw else None,
                                       "strict_5pct_warm": first(dist_w, theta),
                                       "log_l2_warm_window": [round(d, 4) for d in dist_w[::5]]}
        first_scale = row["warm"][str(scales[0])]
        row.update({k: first_scale[k] for k in ("cycles_warm", "warm_s", "warm_start_s", "speedup",
                                                 "strict_5pct_warm", "log_l2_warm_window")})
        per.append(row)
    clock.__exit__()
    tps = [r["plain_s"] for r in per if r["plain_s"]]
    tws = [r["warm_s"] for r in per if r["warm_s"]]
    by_scale = {}
    for sc in scales:
        ws_ = [r["warm"][str(sc)]["warm_s"] for r in per]
        done = [w_ for w_ in ws_ if w_]
        by_scale[str(sc)] = {"converged_terrains": len(done),
                             "warm_s": statistics.mean(done) if done else None,
                             "speedup": (statistics.mean(tps) / statistics.mean(done)) if tps and done and
                             len(done) == len(per) else None}
    # what the prediction is worth: the plain cycles' device time to the
    # prediction's distance from D*, against the warm start's cost
    lv = [(r["prediction_worth_plain_cycles"] * r["ms_per_cycle"] / 1e3, r["warm_start_s"]) for r in per
          if r["prediction_worth_plain_cycles"]]
    out = {"metric": "time to converged discharge (within 5% of the plain runs' floor, log-L2), plain vs "
                     "surrogate warm start", "unit": "s",
           "value": statistics.mean(tws) if tws else None,
           "plain_s": statistics.mean(tps) if tps else None,
           "warm_s": statistics.mean(tws) if tws else None,
           "speedup": (statistics.mean(tps) / statistics.mean(tws)) if tps and tws else None,
           "target_speedup": 3.0,
           "warm_scales": by_scale,
           "prediction_level": {"plain_s": statistics.mean(a for a, _ in lv) if lv else None,
                                "warm_start_s": statistics.mean(b for _, b in lv) if lv else None,
                                "speedup": (statistics.mean(a for a, _ in lv) / statistics.mean(b for _, b in lv))
                                if lv else None},
           "higher_is_better": False, "n_gpus": 1, "dtype": "bf16 (f32 accumulate)",
           "data": "synthetic (seeded value-noise terrains; training pairs from the GPU particle method)",
           "config": {"workload": "learned warm-start: U-Net (1.36 M parameters, 4 levels, channels 32-256) "
                                  "trained on 256x256 terrains, evaluated on 1024x1024 at 65536 drops/cycle",
                      "horizon_cycles": horizon, "threshold": theta, "window_cycles": 10, "spawn_runs": runs,
                      "dstar": "mean over the other spawn runs of the mean discharge of cycles "
                               "horizon+1..horizon+10",
                      "converged": "log-L2 to D* <= (1 + threshold) x the plain runs' floor",
                      "eval_terrains": args.eval_terrains,
                      "train_terrains": n_tr, "train_side": side, "epochs": args.epochs, "batch": batch},
           "training": {"pairs_s": gen_s, "train_s": train_ms / 1e3, "steps": steps,
                        "tflops": train_flops / (train_ms / 1e3) / 1e12 if train_ms else None,
                        "loaded_from": args.load_net or None,
                        "loss_by_epoch": [round(v, 5) for v in losses],
                        "launches": net.launches - launches0, "validation": val},
           "roofline": {"bound": "tensor", "kernel": "conv_tma_kernel (384->128, 3x3, 16x64x64 pixels)",
                        "achieved": conv_flops / (conv_ms / 1e3) / 1e12, "peak": bf16_peak, "unit": "TFLOP/s",
                        "frac": conv_flops / (conv_ms / 1e3) / 1e12 / bf16_peak, "peak_source": peak_src,
                        "avg_launch_ms": conv_ms, "traffic": None,
                        "tflops_by_staging": {k: conv_flops / (v / 1e3) / 1e12 for k, v in conv_paths.items()}},
           "terrains": per, "clocks": clock.summary()}
    print(json.dumps(out))


def run_surrogate_step(args):
    """Training throughput of the surrogate: one step = forward, loss,
    backward and AdamW on a batch of 16 256^2 maps (seeded random heights
    and targets; the kernels' work does not depend on the values).  FLOPs
    are the convolutions' 2 x multiply-adds (forward, input and weight
    gradients)."""
    import torch

    import simplehydrology_gb300 as shy
    from simplehydrology_gb300 import build as shybuild
    from simplehydrology_gb300 import surrogate as sg
    shybuild.build()
    batch, side = 16, 256
    g = torch.Generator(device="cuda").manual_seed(SEED)
    h = torch.rand((batch, side, side), device="cuda", generator=g)
    t = torch.randn((batch, side, side, 3), device="cuda", generator=g)
    net = sg.Surrogate(seed=SEED)
    tuned = net.autotune(batch, side, side)
    for _ in range(args.warmup):
        net.train_step(h, t, 1e-4)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    launches0 = net.launches
    with ClockSampler(torch.cuda.current_device()) as clock:
        ev[0].record()
        for _ in range(args.steps):
            net.train_step(h, t, 1e-4)
        ev[1].record()
        torch.cuda.synchronize()
    net.status()
    ms = ev[0].elapsed_time(ev[1]) / args.steps
    flops = batch * side * side * sg.flops_per_pixel(True)
    # inference on one 1024^2 map: features, forward, decode (device time)
    h1 = torch.rand((1, 1024, 1024), device="cuda", generator=g)
    for _ in range(2):
        net.predict(h1)
    ev[0].record()
    for _ in range(10):
        net.predict(h1)
    ev[1].record()
    torch.cuda.synchronize()
    infer_ms = ev[0].elapsed_time(ev[1]) / 10
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak, src = float(json.load(f)["bf16_tflops_sustained"]), "measured (sustained)"
    except Exception:
        peak, src = 1700.0, "fallback (sustained)"
    tf = flops / (ms / 1e3) / 1e12
    print(json.dumps({
        "metric": "surrogate training throughput", "value": tf, "unit": "TFLOP/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "dtype": "bf16 (f32 accumulate)", "data": "synthetic (seeded random heights and targets)",
        "config": {"workload": "surrogate U-Net training step, 16 x 256x256 maps, AdamW",
                   "params": sg.param_count(), "gflop_per_step": flops / 1e9},
        "gpu_launches": (net.launches - launches0),
        "inference_1024": {"ms": infer_ms,
                           "tflops": 1024 * 1024 * sg.flops_per_pixel(False) / (infer_ms / 1e3) / 1e12},
        "autotune": {f"{n}/{k}": "x".join(str(c) for c in v[0]) for (n, k), v in tuned.items()},
        "roofline": {"bound": "tensor", "achieved": tf, "peak": peak, "unit": "TFLOP/s", "frac": tf / peak,
                     "peak_source": src, "kernel": "whole training step (convolutions 80 % of its time)",
                     "traffic": None},
        "clocks": clock.summary()}))


def run_surrogate_conv(args):
    """The surrogate's largest convolution alone -- dec2a forward, 384 -> 128
    channels, 3x3, at the training batch (16 x 64 x 64 pixels, 58.0 GFLOP)
    with GELU -- for each TMA tile setting (pixels, stages, taps per stage),
    or only the one given by --tile/--stages/--tap-rows.  CUDA events over
    --steps launches after --warmup."""
    import torch

    import simplehydrology_gb300 as shy
    from simplehydrology_gb300 import build as shybuild
    from simplehydrology_gb300 import surrogate as sg
    shybuild.build()
    net = sg.Surrogate(seed=SEED)
    net.prep_weights()
    batch = 16
    ws = net.workspace(batch, 256, 256, True)
    flops = 2.0 * batch * 64 * 64 * 9 * 384 * 128
    if args.tile:
        cands = [(args.tile, args.stages_conv, args.tap_rows)]
    else:
        cands = [c for c in sg.CONV_TILES]
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    res = {}
    for px, st, rows in cands:
        shy._capi.check(shy.lib().shy_sg_set_conv_tile(px, st))
        shy._capi.check(shy.lib().shy_sg_set_conv_tap_rows(rows))
        for _ in range(args.warmup):
            net._conv(ws, "dec2a", ws.cat[2], 384, ws.z["dec2a"], 128, 0, ws.a["dec2a"], 128, 0, sg.ACT_GELU)
        ev[0].record()
        for _ in range(args.steps):
            net._conv(ws, "dec2a", ws.cat[2], 384, ws.z["dec2a"], 128, 0, ws.a["dec2a"], 128, 0, sg.ACT_GELU)
        ev[1].record()
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / args.steps
        res[f"{px}x{st}x{rows}"] = {"ms": ms, "tflops": flops / (ms / 1e3) / 1e12}
    net.status()
    shy._capi.check(shy.lib().shy_sg_set_conv_tile(0, 0))
    shy._capi.check(shy.lib().shy_sg_set_conv_tap_rows(3))
    best = max(res, key=lambda k: res[k]["tflops"])
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak, src = float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        peak, src = 1900.0, "fallback"
    print(json.dumps({"metric": "largest surrogate convolution throughput", "value": res[best]["tflops"],
                      "unit": "TFLOP/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "higher_is_better": True, "dtype": "bf16 (f32 accumulate)", "data": "synthetic",
                      "config": {"workload": "dec2a forward, 16 x 64 x 64 pixels, 384 -> 128, 3x3, GELU",
                                 "best": best},
                      "roofline": {"bound": "tensor", "achieved": res[best]["tflops"], "peak": peak,
                                   "unit": "TFLOP/s", "frac": res[best]["tflops"] / peak, "peak_source": src,
                                   "kernel": "conv_tma_kernel", "traffic": None},
                      "by_tile": res}))


def _initial_height(shy, seed, n):
    w = shy.World(n, n, seed=seed)
    w.generate(seed, 8)
    h = w.get_field("height")
    w.close()
    return h


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    # smaller cases for profiling captures; the bench line itself uses the defaults
    ap.add_argument("--map", type=int, default=NX)
    ap.add_argument("--drops", type=int, default=DROPS)
    ap.add_argument("--no-e2e", action="store_true")
    # the batched-terrain configuration (not the default bench line)
    # default: the single-terrain workload on one GPU; with N > 1 the
    # batched-terrain workload, sharded by whole terrain across the ranks
    ap.add_argument("--workload", default=None, choices=["plain", "batch", "converge", "large", "surrogate",
                                                           "surrogate-step", "surrogate-conv"])
    # --workload surrogate-conv: one tile setting (default: every candidate)
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--stages-conv", type=int, default=0)
    ap.add_argument("--tap-rows", type=int, default=3)
    ap.add_argument("--ref-cycles", type=int, default=2000)
    ap.add_argument("--check-every", type=int, default=10)
    ap.add_argument("--terrains", type=int, default=64)
    # --workload surrogate
    ap.add_argument("--horizon", type=int, default=50)
    ap.add_argument("--train-terrains", type=int, default=4096)
    ap.add_argument("--epochs", type=int, default=24)
    ap.add_argument("--eval-terrains", type=int, default=4)
    ap.add_argument("--spawn-runs", type=int, default=4)
    ap.add_argument("--warm-scales", default="1.0",
                    help="comma-separated scales of the warm start's maps (the first one fills the main keys)")
    ap.add_argument("--save-net", default="", help="--workload surrogate: save the trained network (.npz)")
    ap.add_argument("--load-net", default="", help="--workload surrogate: use this network instead of training")
    ap.add_argument("--train-side", type=int, default=256)
    ap.add_argument("--resort", type=int, default=None,
                    help="steps between re-deals of the live drops (-1 automatic, 0 never); default: automatic")
    ap.add_argument("--autotune", action="store_true",
                    help="run the launch-shape autotuner first and bench the fastest shape")
    ap.add_argument("--whole-cycles", type=int, default=500,
                    help="cycles of the whole-workload average reported beside the headline (0: skip)")
    args = ap.parse_args()
    if args.workload is None:
        args.workload = "batch" if args.gpus > 1 else "plain"
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "converge":
        run_converge(args)
    elif args.workload == "surrogate":
        run_surrogate(args)
    elif args.workload == "surrogate-step":
        run_surrogate_step(args)
    elif args.workload == "surrogate-conv":
        run_surrogate_conv(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
