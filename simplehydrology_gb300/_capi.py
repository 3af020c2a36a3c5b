"""ctypes declarations of the C ABI in include/shy.h and include/shy_surrogate.h.

The library is loaded from this package directory (built in place by
simplehydrology_gb300/build.py).  There is no fallback: if libshy.so is
missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libshy.so")

SHY_OK = 0
SHY_ERR_INVALID_ARG = -1
SHY_ERR_OUT_OF_MEMORY = -2
SHY_ERR_CUDA = -3
SHY_ERR_NO_DEVICE = -4
SHY_ERR_TIMEOUT = -5
SHY_ERR_STATE = -6

FIELD_HEIGHT = 0
FIELD_DISCHARGE = 1
FIELD_MOMENTUM_X = 2
FIELD_MOMENTUM_Y = 3
FIELD_DISCHARGE_TRACK = 4
FIELD_MOMENTUM_X_TRACK = 5
FIELD_MOMENTUM_Y_TRACK = 6
FIELD_ROOT_DENSITY = 7
FIELD_PLANT_SIZE = 8
FIELD_COUNT = 9
FIELD_NAMES = ("height", "discharge", "momentum_x", "momentum_y", "discharge_track",
               "momentum_x_track", "momentum_y_track", "root_density", "plant_size")

KERNEL_DROPS, KERNEL_APPLY, KERNEL_CASCADE, KERNEL_OTHER = 0, 1, 2, 3

ERF_DEVICE = 0
ERF_HOST_LIBM = 1
# shy_feed kinds and floats per cell
FEED_KINDS = {"discharge_rgba": (0, 4), "momentum_rgba": (1, 4), "vertices": (2, 12)}


class Params(C.Structure):
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


class DropState(C.Structure):
    _fields_ = [("age", C.c_int), ("pos", C.c_float * 2), ("speed", C.c_float * 2),
                ("volume", C.c_float), ("sediment", C.c_float)]


class Stats(C.Structure):
    _fields_ = [("cycles", C.c_uint64), ("drops", C.c_uint64), ("drops_skipped", C.c_uint64),
                ("drops_oob", C.c_uint64), ("drop_steps", C.c_uint64), ("evap_gain", C.c_double),
                ("boundary_loss", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Timing(C.Structure):
    _fields_ = [("ms", C.c_double * 4), ("launches", C.c_uint64 * 4), ("steps_timed", C.c_uint64)]


class L2Probe(C.Structure):
    _fields_ = [("l2_bytes", C.c_uint64), ("buffer_bytes", C.c_uint64), ("read_gbs", C.c_double),
                ("random_sector_reads_per_s", C.c_double), ("red_per_s", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ShyError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"shy error {code}: {msg}")
        self.code = code


class SgConvDesc(C.Structure):
    _fields_ = [("batch", C.c_int32), ("height", C.c_int32), ("width", C.c_int32),
                ("cin", C.c_int32), ("cout", C.c_int32), ("ksize", C.c_int32),
                ("tile", C.c_int32), ("stages", C.c_int32), ("tap_rows", C.c_int32)]


class SgAdamw(C.Structure):
    _fields_ = [("lr", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float),
                ("weight_decay", C.c_float), ("bc1", C.c_float), ("bc2", C.c_float)]


class SgNorm(C.Structure):
    _fields_ = [("height_mean", C.c_float), ("height_scale", C.c_float), ("slope_scale", C.c_float),
                ("out_mean", C.c_float * 3), ("out_scale", C.c_float * 3)]


W = C.c_void_p
P = C.POINTER
FP = P(C.c_float)

# name -> (restype, argtypes); every entry point of include/shy.h
SIGNATURES = {
    "shy_version": (C.c_int, []),
    "shy_last_error": (C.c_char_p, []),
    "shy_params_default": (C.c_int, [P(Params)]),
    "shy_world_create": (C.c_int, [C.c_int, C.c_int, P(Params), C.c_uint64, P(W)]),
    "shy_world_destroy": (C.c_int, [W]),
    "shy_world_set_params": (C.c_int, [W, P(Params)]),
    "shy_world_get_params": (C.c_int, [W, P(Params)]),
    "shy_world_size": (C.c_int, [W, P(C.c_int), P(C.c_int)]),
    "shy_world_set_field": (C.c_int, [W, C.c_int, FP, C.c_size_t]),
    "shy_world_get_field": (C.c_int, [W, C.c_int, FP, C.c_size_t]),
    "shy_world_sync": (C.c_int, [W]),
    "shy_terrain_set_state": (C.c_int, [W, C.c_int, FP, FP, FP, FP, C.c_size_t]),
    "shy_terrain_get_state": (C.c_int, [W, C.c_int, FP, FP, FP, FP, C.c_size_t]),
    "shy_world_set_state": (C.c_int, [W, FP, FP, FP, FP, C.c_size_t]),
    "shy_world_get_state": (C.c_int, [W, FP, FP, FP, FP, C.c_size_t]),
    "shy_terrain_set_state_device": (C.c_int, [W, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_size_t]),
    "shy_terrain_get_state_device": (C.c_int, [W, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_size_t]),
    "shy_world_stream": (C.c_int, [W, P(C.c_void_p)]),
    "shy_world_stats": (C.c_int, [W, P(Stats)]),
    "shy_world_reset_stats": (C.c_int, [W]),
    "shy_world_set_cycle": (C.c_int, [W, C.c_uint64]),
    "shy_world_get_cycle": (C.c_int, [W, C.POINTER(C.c_uint64)]),
    "shy_world_enable_timing": (C.c_int, [W, C.c_int]),
    "shy_world_timing": (C.c_int, [W, P(Timing)]),
    "shy_world_set_erf_source": (C.c_int, [W, C.c_int]),
    "shy_world_lockstep_profile": (C.c_int, [W, P(C.c_double), P(C.c_uint64)]),
    "shy_world_set_launch": (C.c_int, [W, C.c_int, C.c_int]),
    "shy_world_set_block": (C.c_int, [W, C.c_int, C.c_int]),
    "shy_world_set_graph": (C.c_int, [W, C.c_int]),
    "shy_world_set_resort": (C.c_int, [W, C.c_int]),
    "shy_world_set_settle": (C.c_int, [W, C.c_int]),
    "shy_debug_stall_waits": (C.c_int, [C.c_uint64]),
    "shy_erode": (C.c_int, [W, C.c_int, C.c_int]),
    "shy_erode_exact": (C.c_int, [W, P(C.c_int32), C.c_int]),
    "shy_drop_descend": (C.c_int, [W, P(DropState), P(C.c_int)]),
    "shy_drop_run": (C.c_int, [W, C.c_float, C.c_float, FP, C.c_int, P(C.c_int)]),
    "shy_cascade": (C.c_int, [W, C.c_float, C.c_float]),
    "shy_normals": (C.c_int, [W, FP, C.c_size_t]),
    "shy_batch_create": (C.c_int, [C.c_int, P(C.c_int), P(C.c_int), P(C.c_int), P(C.c_uint64),
                                   P(Params), P(W)]),
    "shy_batch_erode": (C.c_int, [W, C.c_int]),
    "shy_batch_size": (C.c_int, [W, P(C.c_int)]),
    "shy_terrain_size": (C.c_int, [W, C.c_int, P(C.c_int), P(C.c_int), P(C.c_int)]),
    "shy_terrain_set_field": (C.c_int, [W, C.c_int, C.c_int, FP, C.c_size_t]),
    "shy_terrain_get_field": (C.c_int, [W, C.c_int, C.c_int, FP, C.c_size_t]),
    "shy_terrain_erode_exact": (C.c_int, [W, C.c_int, P(C.c_int32), C.c_int]),
    "shy_terrain_generate": (C.c_int, [W, C.c_int, C.c_uint64, C.c_int]),
    "shy_terrain_init": (C.c_int, [W, C.c_int, C.c_int32]),
    "shy_vegetation_step": (C.c_int, [W, C.c_int]),
    "shy_world_set_vegetation_step": (C.c_int, [W, C.c_uint64]),
    "shy_erode_noalloc": (C.c_int, [C.c_int, C.c_int, P(Params), C.c_uint64, C.c_uint64, C.c_int, C.c_int,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    P(Stats)]),
    "shy_measure_l2": (C.c_int, [C.c_int, P(L2Probe)]),
    "shy_check_conversions": (C.c_int, [P(C.c_uint64)]),
    "shy_feed": (C.c_int, [W, C.c_int, C.c_int, C.c_void_p, C.c_size_t, C.c_int]),
    "shy_world_save": (C.c_int, [W, C.c_char_p]),
    "shy_world_srand": (C.c_int, [W, C.c_uint32]),
    "shy_world_set_rand_order": (C.c_int, [W, C.c_int]),
    "shy_erode_rand": (C.c_int, [W, C.c_int]),
    "shy_vegetation_grow": (C.c_int, [W]),
    "shy_plants": (C.c_int, [W, FP, C.c_int, P(C.c_int)]),
    "shy_world_load": (C.c_int, [C.c_char_p, P(W)]),
    # include/shy_surrogate.h: device pointers and a stream handle
    "shy_sg_conv_forward": (C.c_int, [P(SgConvDesc), W, C.c_int32, W, W, W, C.c_int32, C.c_int32, W,
                                      C.c_int32, C.c_int32, C.c_int32, W]),
    "shy_sg_conv_wgrad": (C.c_int, [P(SgConvDesc), W, C.c_int32, W, C.c_int32, W, W]),
    "shy_sg_conv_input_grad": (C.c_int, [P(SgConvDesc), W, C.c_int32, W, W, C.c_int32, C.c_int32, W, W]),
    "shy_sg_bias_grad": (C.c_int, [C.c_int64, C.c_int32, W, C.c_int32, W, W]),
    "shy_sg_gelu_backward": (C.c_int, [C.c_int64, C.c_int32, W, C.c_int32, C.c_int32, W, C.c_int32, C.c_int32,
                                       W, W, W]),
    "shy_sg_pool_forward": (C.c_int, [C.c_int32] * 4 + [W, C.c_int32, C.c_int32, W, C.c_int32, C.c_int32, W]),
    "shy_sg_pool_backward": (C.c_int, [C.c_int32] * 4 + [W, C.c_int32, C.c_int32, W, C.c_int32, C.c_int32, W]),
    "shy_sg_upsample_forward": (C.c_int, [C.c_int32] * 4 + [W, C.c_int32, C.c_int32, W, C.c_int32, C.c_int32,
                                                            W]),
    "shy_sg_upsample_backward": (C.c_int, [C.c_int32] * 4 + [W, C.c_int32, C.c_int32, W, C.c_int32, C.c_int32,
                                                             W]),
    "shy_sg_weight_prep": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, W, W, W, W]),
    "shy_sg_adamw": (C.c_int, [C.c_int64, W, W, W, W, P(SgAdamw), W]),
    "shy_sg_features": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, W, P(SgNorm), W, W]),
    "shy_sg_loss": (C.c_int, [C.c_int64, W, C.c_int32, W, FP, W, W, W]),
    "shy_sg_decode": (C.c_int, [C.c_int64, W, C.c_int32, P(SgNorm), W, W, W, W]),
    "shy_sg_set_conv_path": (C.c_int, [C.c_int32]),
    "shy_sg_set_conv_tile": (C.c_int, [C.c_int32, C.c_int32]),
    "shy_sg_set_conv_tap_rows": (C.c_int, [C.c_int32]),
    "shy_sg_set_wgrad_tile": (C.c_int, [C.c_int32, C.c_int32]),
    "shy_sg_status": (C.c_int, []),
}

_lib = None


def lib():
    """The loaded libshy.so (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with simplehydrology_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc):
    if rc != SHY_OK:
        msg = lib().shy_last_error()
        raise ShyError(rc, msg.decode() if msg else "")
    return rc


def default_params() -> Params:
    p = Params()
    check(lib().shy_params_default(C.byref(p)))
    return p
