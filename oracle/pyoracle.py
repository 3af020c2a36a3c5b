"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE, not product code.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  It loads

* liboracle.so        -- the restatement of the reference's erosion algorithm
                         (hydro_oracle.cpp), and
* _ref/libshyref.so   -- the reference's own erosion headers compiled
                         unmodified (ref_harness.cpp), where it was built.

Maps are numpy arrays of shape (nx, ny), x-major like the reference
(math::flatten, source/include/math.h:11-14).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libshyref.so")

ERF_LIBM = 0
ERF_SHY = 1

FIELDS = ("height", "discharge", "momentum_x", "momentum_y",
          "discharge_track", "momentum_x_track", "momentum_y_track", "root_density")


class Params(C.Structure):
    """Mirror of shy_params (include/shy.h)."""
    _fields_ = [
        ("evap_rate", C.c_float), ("deposition_rate", C.c_float), ("min_vol", C.c_float),
        ("max_age", C.c_float), ("entrainment", C.c_float), ("gravity", C.c_float),
        ("momentum_transfer", C.c_float), ("lrate", C.c_float), ("max_diff", C.c_float),
        ("settling", C.c_float), ("map_scale", C.c_float), ("plant_max_size", C.c_float),
        ("plant_grow_rate", C.c_float), ("plant_max_steep", C.c_float),
        ("plant_max_discharge", C.c_float), ("plant_max_height", C.c_float),
        ("plant_spawn_prob", C.c_float), ("plant_death_prob", C.c_float),
        ("plant_spread_prob", C.c_float), ("cascade_weight", C.c_float),
        ("cascade_passes", C.c_int), ("reserved", C.c_int * 7),
    ]


class Drop(C.Structure):
    """Mirror of shy_drop (include/shy.h)."""
    _fields_ = [("age", C.c_int), ("pos", C.c_float * 2), ("speed", C.c_float * 2),
                ("volume", C.c_float), ("sediment", C.c_float)]


class Acc(C.Structure):
    _fields_ = [("drops", C.c_uint64), ("skipped", C.c_uint64), ("oob", C.c_uint64),
                ("steps", C.c_uint64), ("gain", C.c_double), ("loss", C.c_double),
                ("gain_q", C.c_int64), ("loss_q", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class GridF32(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("f", C.POINTER(C.c_float) * 8)]


class GridF64(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("f", C.POINTER(C.c_double) * 8)]


# The reference checkout the harness compiles from: SHY_REFERENCE, else the
# place this build's container mounts it (absent on machines without it).
REFERENCE_DIR = os.environ.get("SHY_REFERENCE", "/root/reference")


def build(quiet: bool = True) -> None:
    """Build liboracle.so (and the reference harness where the checkout exists)."""
    cmd = ["make", "-C", HERE]
    if os.path.isfile(os.path.join(REFERENCE_DIR, "source", "world.h")):
        cmd.append("REF=" + REFERENCE_DIR)
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        L.orc_params_default.argtypes = [P(Params)]
        L.orc_erode_seq_f32.argtypes = [P(GridF32), P(Params), P(C.c_int32), C.c_int, C.c_int, P(Acc)]
        L.orc_erode_seq_f64.argtypes = [P(GridF64), P(Params), P(C.c_int32), C.c_int, C.c_int, P(Acc)]
        L.orc_drop_run_f32.argtypes = [P(GridF32), P(Params), C.c_float, C.c_float, P(C.c_float),
                                       C.c_int, C.c_int, P(Acc)]
        L.orc_drop_run_f64.argtypes = [P(GridF64), P(Params), C.c_double, C.c_double, P(C.c_float),
                                       C.c_int, C.c_int, P(Acc)]
        L.orc_drop_descend_f32.argtypes = [P(GridF32), P(Params), P(Drop), C.c_int, P(Acc)]
        L.orc_cascade_f32.argtypes = [P(GridF32), P(Params), C.c_float, C.c_float]
        L.orc_normals_f32.argtypes = [P(GridF32), P(Params), P(C.c_float)]
        L.orc_feed_f32.argtypes = [P(GridF32), P(Params), C.c_int, C.c_int, P(C.c_float)]
        L.orc_crand.argtypes = [C.c_uint, C.c_int, P(C.c_int)]
        L.orc_frames_f32.argtypes = [P(GridF32), P(Params), C.c_uint, C.c_int, C.c_int, C.c_int, C.c_int,
                                     P(C.c_float), C.c_int, P(Acc)]
        L.orc_frames_f32.restype = C.c_int
        L.orc_rand_spawns.argtypes = [C.c_uint, C.c_int, C.c_int, C.c_int, C.c_int, P(C.c_int32)]
        L.orc_erode_batched_f32.argtypes = [P(GridF32), P(Params), C.c_uint64, C.c_uint64, C.c_int,
                                            C.c_int, P(Acc), P(C.c_int64), C.c_int]
        L.orc_value_noise.argtypes = [C.c_int, C.c_int, C.c_uint64, C.c_int, P(C.c_float)]
        L.orc_terrain_init.argtypes = [C.c_int, C.c_int, C.c_int32, P(C.c_float)]
        L.orc_vegetation_step_f32.argtypes = [P(GridF32), P(C.c_float), P(Params), C.c_uint64, C.c_uint64]
        L.orc_erff_libm.argtypes = [C.c_float]
        L.orc_erff_libm.restype = C.c_float
        L.orc_erff_shy.argtypes = [C.c_float]
        L.orc_erff_shy.restype = C.c_float
        L.orc_erf_shy_d.argtypes = [C.c_double]
        L.orc_erf_shy_d.restype = C.c_double
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    """The reference's erosion code, compiled unmodified (512 x 512 map)."""
    global _ref
    if _ref is None:
        R = C.CDLL(REF_PATH)
        P = C.POINTER
        R.ref_init.argtypes = [C.c_uint]
        R.ref_set_field.argtypes = [C.c_int, P(C.c_float)]
        R.ref_get_field.argtypes = [C.c_int, P(C.c_float)]
        R.ref_srand.argtypes = [C.c_uint]
        R.ref_erode.argtypes = [C.c_int]
        R.ref_cascade.argtypes = [C.c_float, C.c_float]
        R.ref_normal.argtypes = [C.c_int, C.c_int, P(C.c_float)]
        R.ref_descend_trace.argtypes = [C.c_float, C.c_float, P(C.c_float), C.c_int]
        R.ref_veg_get.argtypes = [P(C.c_float), C.c_int]
        R.ref_frame.argtypes = [P(C.c_float), P(C.c_float), P(C.c_float)]
        R.ref_init(1)
        _ref = R
    return _ref


def ref_terrain(seed):
    """quad::map::init's heights for `seed` (the reference's int SEED) from the
    reference build, as a (512, 512) array.  The reference builds its map once
    per process, so each seed runs in a child process."""
    code = ("import ctypes as C, sys, numpy as np\n"
            "R = C.CDLL(sys.argv[1]); n = R.ref_tilesize()\n"
            "R.ref_init.argtypes = [C.c_uint]; R.ref_init(int(sys.argv[2]) & 0xffffffff)\n"
            "o = np.empty(n * n, np.float32)\n"
            "R.ref_get_field(0, o.ctypes.data_as(C.POINTER(C.c_float)))\n"
            "sys.stdout.buffer.write(o.tobytes())\n")
    out = subprocess.run([sys.executable, "-c", code, REF_PATH, str(seed)], capture_output=True,
                         check=True).stdout
    a = np.frombuffer(out, np.float32)
    n = int(round(len(a) ** 0.5))
    return a.reshape(n, n).copy()


def fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def ipptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def default_params() -> Params:
    p = Params()
    lib().orc_params_default(C.byref(p))
    return p


class Maps:
    """The eight quad::cell fields (source/cellpool.h:207-220) as (nx, ny) arrays."""

    def __init__(self, nx, ny, dtype=np.float32, height=None):
        self.nx, self.ny = nx, ny
        self.dtype = np.dtype(dtype)
        self.f = [np.zeros((nx, ny), dtype=self.dtype) for _ in range(8)]
        self.hq_valid = False
        if height is not None:
            self.f[0][...] = height

    def copy(self, dtype=None):
        m = Maps(self.nx, self.ny, dtype or self.dtype)
        for i in range(8):
            m.f[i][...] = self.f[i]
        return m

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        if name in FIELDS:
            return self.f[FIELDS.index(name)]
        raise AttributeError(name)

    def grid(self):
        if self.dtype == np.float32:
            g = GridF32()
            g.nx, g.ny = self.nx, self.ny
            for i in range(8):
                assert self.f[i].flags.c_contiguous
                g.f[i] = fptr(self.f[i])
        else:
            g = GridF64()
            g.nx, g.ny = self.nx, self.ny
            for i in range(8):
                g.f[i] = dptr(self.f[i])
        return g


def value_noise(nx, ny, seed, octaves=8):
    out = np.empty((nx, ny), np.float32)
    lib().orc_value_noise(nx, ny, seed, octaves, fptr(out))
    return out


def terrain_init(nx, ny, seed):
    """quad::map::init's terrain for an nx x ny map (source/cellpool.h:323-411)."""
    out = np.empty((nx, ny), np.float32)
    lib().orc_terrain_init(nx, ny, seed, fptr(out))
    return out


def erode_seq(maps: Maps, spawns, params=None, erf_mode=ERF_LIBM):
    """World::erode(len(spawns)) with the given spawn cells, in place."""
    params = params or default_params()
    sp = np.ascontiguousarray(np.asarray(spawns, np.int32).reshape(-1, 2))
    acc = Acc()
    g = maps.grid()
    fn = lib().orc_erode_seq_f32 if maps.dtype == np.float32 else lib().orc_erode_seq_f64
    fn(C.byref(g), C.byref(params), ipptr(sp), len(sp), erf_mode, C.byref(acc))
    return acc


def drop_run(maps: Maps, x, y, params=None, erf_mode=ERF_LIBM, max_records=1024):
    """Drop d(pos); while (d.descend()); -> (trace[n, 8], Acc)."""
    params = params or default_params()
    tr = np.zeros((max_records, 8), np.float32)
    acc = Acc()
    g = maps.grid()
    fn = lib().orc_drop_run_f32 if maps.dtype == np.float32 else lib().orc_drop_run_f64
    n = fn(C.byref(g), C.byref(params), x, y, fptr(tr), max_records, erf_mode, C.byref(acc))
    return tr[:min(n, max_records)].copy(), acc


def cascade(maps: Maps, x, y, params=None):
    params = params or default_params()
    g = maps.grid()
    lib().orc_cascade_f32(C.byref(g), C.byref(params), x, y)


def normals(maps: Maps, params=None):
    params = params or default_params()
    out = np.zeros((maps.nx, maps.ny, 3), np.float32)
    g = maps.grid()
    lib().orc_normals_f32(C.byref(g), C.byref(params), fptr(out))
    return out


def feed(maps: Maps, kind, erf_mode=ERF_SHY, params=None):
    """The front end's per-frame buffer: kind 0 discharge texture, 1 momentum
    texture (4 floats per cell), 2 mesh vertices (12 floats per cell)."""
    params = params or default_params()
    out = np.zeros((maps.nx, maps.ny, 12 if kind == 2 else 4), np.float32)
    g = maps.grid()
    lib().orc_feed_f32(C.byref(g), C.byref(params), kind, erf_mode, fptr(out))
    return out


def crand(seed, n):
    """n outputs of the restated C-library rand() after srand(seed)."""
    out = np.zeros(n, np.int32)
    lib().orc_crand(seed, n, out.ctypes.data_as(C.POINTER(C.c_int)))
    return out


def frames(maps: Maps, seed, n_frames, drops, order=1, erf_mode=ERF_LIBM, params=None, max_plants=1 << 20):
    """The reference's frame loop (World::erode(drops); Vegetation::grow()) from
    srand(seed); returns the plant list (n, 3) and the counters."""
    params = params or default_params()
    out = np.zeros((max_plants, 3), np.float32)
    acc = Acc()
    g = maps.grid()
    n = lib().orc_frames_f32(C.byref(g), C.byref(params), seed, n_frames, drops, order, erf_mode, fptr(out),
                             max_plants, C.byref(acc))
    return out[:min(n, max_plants)].copy(), acc


def rand_spawns(seed, n, nx, ny, order):
    out = np.zeros((n, 2), np.int32)
    lib().orc_rand_spawns(seed, n, nx, ny, order, ipptr(out))
    return out


def erode_batched(maps: Maps, seed, cycle0, drops, cycles, params=None, hq=None):
    """Batched (lock-step) cycles in place.  `hq`, an (nx, ny) int64 array,
    carries the fixed-point heights between calls: pass the same array to a
    later call to continue exactly where this one stopped (it is filled on
    the first call, when maps.hq_valid is not set)."""
    params = params or default_params()
    acc = Acc()
    g = maps.grid()
    hq_ptr = None
    hq_in = 0
    if hq is not None:
        assert hq.dtype == np.int64 and hq.flags.c_contiguous and hq.size == maps.nx * maps.ny
        hq_ptr = hq.ctypes.data_as(C.POINTER(C.c_int64))
        hq_in = 1 if getattr(maps, "hq_valid", False) else 0
    lib().orc_erode_batched_f32(C.byref(g), C.byref(params), seed, cycle0, drops, cycles,
                                C.byref(acc), hq_ptr, hq_in)
    if hq is not None:
        maps.hq_valid = True
    return acc


def vegetation_step(maps: Maps, plant, seed, step, params=None):
    """One per-cell vegetation step; `plant` (nx, ny) float32 sizes, in place."""
    params = params or default_params()
    assert plant.dtype == np.float32 and plant.flags.c_contiguous
    g = maps.grid()
    lib().orc_vegetation_step_f32(C.byref(g), fptr(plant), C.byref(params), seed, step)


# ---- the compiled reference (512 x 512) -----------------------------------

def ref_set_maps(maps: Maps):
    R = ref()
    for i in range(8):
        a = np.ascontiguousarray(maps.f[i], dtype=np.float32)
        R.ref_set_field(i, fptr(a))


def ref_get_maps(nx=512, ny=512) -> Maps:
    R = ref()
    m = Maps(nx, ny)
    for i in range(8):
        R.ref_get_field(i, fptr(m.f[i]))
    return m


def ref_drop_run(x, y, max_records=1024):
    tr = np.zeros((max_records, 8), np.float32)
    n = ref().ref_descend_trace(x, y, fptr(tr), max_records)
    return tr[:min(n, max_records)].copy()
