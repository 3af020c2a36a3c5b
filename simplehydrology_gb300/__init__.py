"""simplehydrology_gb300 -- the SimpleHydrology erosion path on one GB300 GPU.

The engine is libshy.so (CUDA, sm_103a) behind the C ABI in include/shy.h.
This module mirrors the reference's erosion interface on top of it:

  World(nx, ny).erode(cycles)   World::erode(int cycles)      source/world.h:54-88
  World.erode_exact(spawns)     World::erode with given spawns, sequential
  World.cascade(pos)            World::cascade(vec2)           source/world.h:90-168
  Drop(world, pos).descend()    Drop::descend()                source/water.h:58-156
  World.height/discharge/normal quad::map accessors            source/cellpool.h:413-447

Arrays are numpy float32 of shape (nx, ny), x-major like the reference.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from ._capi import (ERF_DEVICE, ERF_HOST_LIBM, FEED_KINDS, FIELD_NAMES, DropState, L2Probe, Params, ShyError,
                    Stats, Timing, check, default_params, lib)

__all__ = ["World", "Batch", "Drop", "Params", "Stats", "Timing", "ShyError", "default_params",
           "lib", "load", "measure_l2", "check_conversions", "ERF_DEVICE", "ERF_HOST_LIBM", "FIELD_NAMES"]


def measure_l2(device: int = 0) -> dict:
    """L2 peaks of one device from the library's microbenchmarks (shy_measure_l2)."""
    out = L2Probe()
    check(lib().shy_measure_l2(int(device), C.byref(out)))
    return out.as_dict()


def check_conversions():
    """Mismatch counts of the kernels' fast arithmetic against the library's
    restatements: (float -> 32.32, 32.32 -> float, float-float erf, float
    evaporation division, float edge height); all 0 on a conforming device
    (shy_check_conversions)."""
    out = (C.c_uint64 * 5)()
    check(lib().shy_check_conversions(out))
    return tuple(int(v) for v in out)


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _field_index(field):
    if isinstance(field, str):
        return FIELD_NAMES.index(field)
    return int(field)


class _Handle:
    def __init__(self):
        self._w = C.c_void_p()

    def close(self):
        if self._w:
            lib().shy_world_destroy(self._w)
            self._w = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # counters and timing
    def stats(self) -> Stats:
        s = Stats()
        check(lib().shy_world_stats(self._w, C.byref(s)))
        return s

    def reset_stats(self):
        check(lib().shy_world_reset_stats(self._w))

    def enable_timing(self, on=True):
        check(lib().shy_world_enable_timing(self._w, 1 if on else 0))

    def timing(self) -> Timing:
        t = Timing()
        check(lib().shy_world_timing(self._w, C.byref(t)))
        return t

    def lockstep_profile(self):
        """(phase_ms[6], iterations) of the batched kernel, seen by its first CTA."""
        ph = (C.c_double * 6)()
        it = C.c_uint64()
        check(lib().shy_world_lockstep_profile(self._w, ph, C.byref(it)))
        return list(ph), it.value

    def vegetation_step(self, steps: int = 1):
        """Vegetation::grow(), per cell (source/vegetation.h:122-188)."""
        check(lib().shy_vegetation_step(self._w, steps))

    def set_launch(self, grid: int = 0, order: int = -1):
        """At most `grid` CTAs for the batched kernel (0: all resident); slots
        in spawn-cell order (-1: when the state outgrows L2, 0 never, 1 always)."""
        check(lib().shy_world_set_launch(self._w, grid, order))

    def set_block(self, threads: int = 256, smem_slots: int = 1):
        """Threads per CTA of the batched kernel (64, 128 or 256) and whether
        drop slots may live in shared memory (1) or always in global (0)."""
        check(lib().shy_world_set_block(self._w, threads, smem_slots))

    def set_resort(self, steps: int = -1):
        """Every `steps` lock-step steps, sort the live drops by their cell and
        deal them to the CTAs again (slots in global memory only; -1: every
        16 steps with spawn-ordered slots, else never; 0 never)."""
        check(lib().shy_world_set_resort(self._w, steps))

    def set_settle(self, mode: int = -1):
        """With re-deals: 1 the first drop registered in a cell settles the
        cell's whole step, 0 every drop its own change, -1 (default) 1 when
        the slots outgrow L2."""
        check(lib().shy_world_set_settle(self._w, mode))

    def set_graph(self, cycles_per_graph: int = 0):
        """Run batched cycles as CUDA graphs of this many cycles (0: none)."""
        check(lib().shy_world_set_graph(self._w, cycles_per_graph))

    def set_cycle(self, cycle: int):
        check(lib().shy_world_set_cycle(self._w, cycle))

    def cycle(self) -> int:
        """The cycle index the next batched cycle uses for its spawns."""
        c = C.c_uint64()
        check(lib().shy_world_get_cycle(self._w, C.byref(c)))
        return c.value

    def sync(self):
        check(lib().shy_world_sync(self._w))

    def stream(self) -> int:
        s = C.c_void_p()
        check(lib().shy_world_stream(self._w, C.byref(s)))
        return s.value or 0

    # ---- the state a front end exchanges every frame, in one call each way ----
    _STATE = ("height", "discharge", "momentum_x", "momentum_y")

    def _state_args(self, terrain, arrays, writable):
        nx, ny = self._terrain_shape(terrain)
        ptrs = []
        for name in self._STATE:
            a = arrays.get(name)
            if a is None:
                ptrs.append(None)
                continue
            if writable:
                if a.dtype != np.float32 or a.shape != (nx, ny) or not a.flags.c_contiguous:
                    raise ValueError(f"{name}: want a contiguous float32 array of shape {(nx, ny)}")
            else:
                a = np.ascontiguousarray(a, np.float32).reshape(nx, ny)
                arrays[name] = a
            ptrs.append(_fptr(a))
        return ptrs, nx * ny

    def set_state(self, terrain: int = 0, **fields):
        """height / discharge / momentum_x / momentum_y of one terrain in one
        call (shy_terrain_set_state); fields not given are left unchanged."""
        unknown = set(fields) - set(self._STATE)
        if unknown:
            raise ValueError(f"unknown fields {sorted(unknown)}")
        arrays = dict(fields)
        ptrs, n = self._state_args(terrain, arrays, False)
        check(lib().shy_terrain_set_state(self._w, terrain, *ptrs, n))

    def get_state(self, terrain: int = 0, out=None):
        """The four state fields of one terrain (shy_terrain_get_state), into
        `out` (a dict of float32 arrays) when given."""
        nx, ny = self._terrain_shape(terrain)
        if out is None:
            out = {name: np.empty((nx, ny), np.float32) for name in self._STATE}
        ptrs, n = self._state_args(terrain, out, True)
        check(lib().shy_terrain_get_state(self._w, terrain, *ptrs, n))
        return out

    def _cells_total(self):
        sizes = getattr(self, "sizes", None) or [(self.nx, self.ny)]
        return sum(int(x) * int(y) for x, y in sizes)

    def set_state_all(self, **fields):
        """Every terrain's height / discharge / momentum_x / momentum_y in one
        call (shy_world_set_state): float32 arrays of all cells, terrain after
        terrain in creation order, each x-major; fields not given are left
        unchanged."""
        unknown = set(fields) - set(self._STATE)
        if unknown:
            raise ValueError(f"unknown fields {sorted(unknown)}")
        n = self._cells_total()
        keep, ptrs = [], []
        for name in self._STATE:
            a = fields.get(name)
            if a is None:
                ptrs.append(None)
                continue
            a = np.ascontiguousarray(a, np.float32).reshape(n)
            keep.append(a)
            ptrs.append(_fptr(a))
        check(lib().shy_world_set_state(self._w, *ptrs, n))

    def get_state_all(self, out=None):
        """The four state fields of every terrain (shy_world_get_state), as
        flat arrays laid out like set_state_all's, into `out` when given."""
        n = self._cells_total()
        if out is None:
            out = {name: np.empty(n, np.float32) for name in self._STATE}
        ptrs = []
        for name in self._STATE:
            a = out.get(name)
            if a is None:
                ptrs.append(None)
                continue
            if a.dtype != np.float32 or a.size != n or not a.flags.c_contiguous:
                raise ValueError(f"{name}: want a contiguous float32 array of {n} elements")
            ptrs.append(_fptr(a))
        check(lib().shy_world_get_state(self._w, *ptrs, n))
        return out

    def _device_args(self, terrain, tensors):
        nx, ny = self._terrain_shape(terrain)
        ptrs = []
        for name in self._STATE:
            t = tensors.get(name)
            if t is None:
                ptrs.append(None)
                continue
            import torch
            if (not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float32
                    or not t.is_contiguous() or t.numel() != nx * ny):
                raise ValueError(f"{name}: want a contiguous float32 CUDA tensor of {nx * ny} elements")
            ptrs.append(t.data_ptr())
        return ptrs, nx * ny

    def set_state_device(self, terrain: int = 0, **tensors):
        """set_state from torch CUDA tensors, device to device
        (shy_terrain_set_state_device); the tensors' producing work must have
        finished (synchronize its stream first)."""
        unknown = set(tensors) - set(self._STATE)
        if unknown:
            raise ValueError(f"unknown fields {sorted(unknown)}")
        ptrs, n = self._device_args(terrain, tensors)
        check(lib().shy_terrain_set_state_device(self._w, terrain, *ptrs, n))

    def get_state_device(self, terrain: int = 0, out=None):
        """The four state fields of one terrain as torch CUDA tensors (nx, ny),
        device to device (shy_terrain_get_state_device), into `out` when given."""
        import torch
        nx, ny = self._terrain_shape(terrain)
        if out is None:
            out = {name: torch.empty((nx, ny), dtype=torch.float32, device="cuda") for name in self._STATE}
        ptrs, n = self._device_args(terrain, out)
        check(lib().shy_terrain_get_state_device(self._w, terrain, *ptrs, n))
        return out

    def save(self, path):
        """Write the world's state to a checkpoint file (shy_world_save)."""
        check(lib().shy_world_save(self._w, str(path).encode()))

    def feed(self, kind: str, terrain: int = 0, out=None):
        """The front end's per-frame buffer `kind` (discharge_rgba, momentum_rgba
        or vertices) of one terrain, as a numpy array (nx, ny, 4 or 12).  `out`
        may be a torch CUDA tensor of that shape (float32, contiguous), which
        is filled on the device."""
        k, per = FEED_KINDS[kind]
        nx, ny = self._terrain_shape(terrain)
        if out is not None and hasattr(out, "data_ptr"):
            if tuple(out.shape) != (nx, ny, per) or not out.is_contiguous() or out.element_size() != 4:
                raise ValueError("out must be a contiguous float32 tensor of shape (nx, ny, %d)" % per)
            check(lib().shy_feed(self._w, terrain, k, C.c_void_p(out.data_ptr()), nx * ny * per, 1))
            return out
        a = np.empty((nx, ny, per), np.float32)
        check(lib().shy_feed(self._w, terrain, k, a.ctypes.data_as(C.c_void_p), a.size, 0))
        return a

    def _terrain_shape(self, terrain):
        nx, ny, d = C.c_int(), C.c_int(), C.c_int()
        check(lib().shy_terrain_size(self._w, terrain, C.byref(nx), C.byref(ny), C.byref(d)))
        return nx.value, ny.value

    @property
    def params(self) -> Params:
        p = Params()
        check(lib().shy_world_get_params(self._w, C.byref(p)))
        return p

    @params.setter
    def params(self, p: Params):
        check(lib().shy_world_set_params(self._w, C.byref(p)))


class World(_Handle):
    """One terrain: the reference's class World (source/world.h:17-36)."""

    def __init__(self, nx: int, ny: int, params: Params | None = None, seed: int = 1):
        super().__init__()
        p = C.byref(params) if params is not None else None
        check(lib().shy_world_create(nx, ny, p, seed, C.byref(self._w)))
        self.nx, self.ny = nx, ny

    # ---- fields ----
    def set_field(self, field, values):
        a = np.ascontiguousarray(values, dtype=np.float32).reshape(self.nx, self.ny)
        check(lib().shy_world_set_field(self._w, _field_index(field), _fptr(a), a.size))

    def get_field(self, field, out=None):
        if out is None:
            out = np.empty((self.nx, self.ny), np.float32)
        check(lib().shy_world_get_field(self._w, _field_index(field), _fptr(out), out.size))
        return out

    def generate(self, seed: int, octaves: int = 8):
        """Seeded fractal value-noise heights, normalised to [0, 1], on the GPU."""
        check(lib().shy_terrain_generate(self._w, 0, seed, octaves))

    def init_terrain(self, seed: int):
        """The reference's own terrain for `seed`: quad::map::init's OpenSimplex2
        FBm layers, min-max normalised (source/cellpool.h:323-411), on the GPU."""
        check(lib().shy_terrain_init(self._w, 0, seed))

    def set_erf_source(self, source: int):
        check(lib().shy_world_set_erf_source(self._w, source))

    # ---- erosion (source/world.h:54-168, source/water.h:58-156) ----
    def erode(self, cycles: int, repeat: int = 1):
        """World::erode(cycles): `cycles` drops, batched, `repeat` times."""
        check(lib().shy_erode(self._w, cycles, repeat))

    def erode_exact(self, spawns):
        sp = np.ascontiguousarray(np.asarray(spawns, np.int32).reshape(-1, 2))
        check(lib().shy_erode_exact(self._w, sp.ctypes.data_as(C.POINTER(C.c_int32)), len(sp)))

    # ---- the reference's frame loop in its own random sequence ----
    def srand(self, seed: int):
        """srand(seed) for the world's C-library random stream."""
        check(lib().shy_world_srand(self._w, seed))

    def erode_rand(self, drops: int):
        """World::erode(drops), sequential, spawns from the world's stream."""
        check(lib().shy_erode_rand(self._w, drops))

    def grow(self):
        """Vegetation::grow() on the world's plant list."""
        check(lib().shy_vegetation_grow(self._w))

    def plants(self):
        """The plant list as (n, 3) float32: x, y, size."""
        n = C.c_int()
        check(lib().shy_plants(self._w, None, 0, C.byref(n)))
        out = np.zeros((n.value, 3), np.float32)
        if n.value:
            check(lib().shy_plants(self._w, _fptr(out), n.value, C.byref(n)))
        return out

    def cascade(self, pos):
        check(lib().shy_cascade(self._w, float(pos[0]), float(pos[1])))

    def drop_run(self, x, y, max_records=1024):
        tr = np.zeros((max_records, 8), np.float32)
        n = C.c_int()
        check(lib().shy_drop_run(self._w, float(x), float(y), _fptr(tr), max_records, C.byref(n)))
        return tr[:min(n.value, max_records)].copy()

    def normals(self):
        out = np.empty((self.nx, self.ny, 3), np.float32)
        check(lib().shy_normals(self._w, _fptr(out), out.size))
        return out

    # ---- quad::map accessors (source/cellpool.h:413-447), from a host copy ----
    def oob(self, p):
        x, y = int(p[0]), int(p[1])
        return x < 0 or y < 0 or x >= self.nx or y >= self.ny

    def height(self, p):
        if self.oob(p):
            return 0.0
        return float(self.get_field("height")[int(p[0]), int(p[1])])

    def discharge(self, p):
        """erf(0.4 * discharge) (source/cellpool.h:242-244, 439-443)."""
        if self.oob(p):
            return 0.0
        from math import erf
        return erf(0.4 * float(self.get_field("discharge")[int(p[0]), int(p[1])]))


class Drop:
    """struct Drop (source/water.h:12-39) descending on a World."""

    def __init__(self, world: World, pos):
        self.world = world
        self.state = DropState()
        self.state.age = 0
        self.state.pos[0], self.state.pos[1] = float(pos[0]), float(pos[1])
        self.state.speed[0] = self.state.speed[1] = 0.0
        self.state.volume = 1.0
        self.state.sediment = 0.0

    def descend(self) -> bool:
        more = C.c_int()
        check(lib().shy_drop_descend(self.world._w, C.byref(self.state), C.byref(more)))
        return bool(more.value)

    @property
    def pos(self):
        return (self.state.pos[0], self.state.pos[1])

    @property
    def speed(self):
        return (self.state.speed[0], self.state.speed[1])

    @property
    def volume(self):
        return self.state.volume

    @property
    def sediment(self):
        return self.state.sediment

    @property
    def age(self):
        return self.state.age


class Batch(_Handle):
    """Many independent terrains eroded in one lock-step launch per cycle."""

    def __init__(self, sizes, drops_per_cycle, seeds, params: Params | None = None):
        super().__init__()
        n = len(sizes)
        nx = (C.c_int * n)(*[int(s[0]) for s in sizes])
        ny = (C.c_int * n)(*[int(s[1]) for s in sizes])
        dr = (C.c_int * n)(*[int(d) for d in drops_per_cycle])
        sd = (C.c_uint64 * n)(*[int(s) for s in seeds])
        p = C.byref(params) if params is not None else None
        check(lib().shy_batch_create(n, nx, ny, dr, sd, p, C.byref(self._w)))
        self.sizes = [(int(s[0]), int(s[1])) for s in sizes]

    def __len__(self):
        return len(self.sizes)

    def set_field(self, t, field, values):
        nx, ny = self.sizes[t]
        a = np.ascontiguousarray(values, dtype=np.float32).reshape(nx, ny)
        check(lib().shy_terrain_set_field(self._w, t, _field_index(field), _fptr(a), a.size))

    def get_field(self, t, field, out=None):
        nx, ny = self.sizes[t]
        if out is None:
            out = np.empty((nx, ny), np.float32)
        elif out.dtype != np.float32 or out.shape != (nx, ny) or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous float32 array of the terrain's shape")
        check(lib().shy_terrain_get_field(self._w, t, _field_index(field), _fptr(out), out.size))
        return out

    def generate(self, t, seed: int, octaves: int = 8):
        check(lib().shy_terrain_generate(self._w, t, seed, octaves))

    def init_terrain(self, t, seed: int):
        check(lib().shy_terrain_init(self._w, t, seed))

    def erode(self, cycles: int = 1):
        check(lib().shy_batch_erode(self._w, cycles))


def load(path):
    """A world resumed from a checkpoint file (shy_world_load): a World for a
    single terrain, a Batch otherwise."""
    h = C.c_void_p()
    check(lib().shy_world_load(str(path).encode(), C.byref(h)))
    n = C.c_int()
    check(lib().shy_batch_size(h, C.byref(n)))
    sizes = []
    for t in range(n.value):
        nx, ny, d = C.c_int(), C.c_int(), C.c_int()
        check(lib().shy_terrain_size(h, t, C.byref(nx), C.byref(ny), C.byref(d)))
        sizes.append((nx.value, ny.value))
    if n.value == 1:
        obj = World.__new__(World)
        _Handle.__init__(obj)
        obj.nx, obj.ny = sizes[0]
    else:
        obj = Batch.__new__(Batch)
        _Handle.__init__(obj)
        obj.sizes = sizes
    obj._w = h
    return obj
