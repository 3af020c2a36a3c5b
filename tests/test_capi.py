"""The C ABI library without a GPU: it loads, exports every entry point that
include/shy.h and include/shy_surrogate.h declare, and validates arguments
before touching a device."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", h) for h in ("shy.h", "shy_surrogate.h")]


def declared():
    src = "".join(open(h).read() for h in HEADERS)
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\**(shy_\w+)\s*\(", src, flags=re.M)))


def test_header_declares_entry_points():
    names = declared()
    assert "shy_erode" in names and "shy_world_create" in names and len(names) >= 30


def test_library_exports_every_declared_symbol(shy):
    out = subprocess.run(["nm", "-D", "--defined-only", shy._capi.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r" T (shy_\w+)", out))
    missing = [n for n in declared() if n not in exported]
    assert not missing, missing
    # and the Python binding covers all of them
    assert not [n for n in declared() if n not in shy._capi.SIGNATURES]


def test_defaults_are_the_reference_values(shy):
    p = shy.default_params()
    # source/water.h:43-50, source/world.h:42-44, source/cellpool.h:165,
    # source/vegetation.h:38-42
    assert (p.evap_rate, p.deposition_rate, p.min_vol, p.max_age) == (
        C.c_float(0.001).value, C.c_float(0.1).value, C.c_float(0.01).value, 500.0)
    assert (p.entrainment, p.gravity, p.momentum_transfer) == (10.0, 1.0, 1.0)
    assert (p.lrate, p.max_diff, p.settling) == (C.c_float(0.1).value, C.c_float(0.01).value,
                                                 C.c_float(0.8).value)
    assert p.map_scale == 80.0
    assert (p.plant_max_size, p.plant_grow_rate, p.plant_max_steep, p.plant_max_discharge,
            p.plant_max_height) == (1.5, C.c_float(0.05).value, C.c_float(0.8).value,
                                    C.c_float(0.3).value, C.c_float(0.8).value)
    assert p.cascade_passes == 0


def test_oracle_defaults_match_library(shy, po):
    a, b = shy.default_params(), po.default_params()
    assert bytes(a) == bytes(b)


@pytest.mark.parametrize("nx,ny", [(0, 5), (5, 0), (-1, 3), (1 << 16, 1 << 16)])
def test_create_rejects_bad_sizes(shy, nx, ny):
    w = C.c_void_p()
    rc = shy.lib().shy_world_create(nx, ny, None, 1, C.byref(w))
    assert rc == -1 and not w.value
    assert b"size" in shy.lib().shy_last_error()


def test_null_arguments(shy):
    L = shy.lib()
    assert L.shy_world_create(8, 8, None, 1, None) == -1
    assert L.shy_params_default(None) == -1
    assert L.shy_erode(None, 10, 1) == -1
    assert L.shy_world_get_field(None, 0, None, 0) == -1
    assert L.shy_world_destroy(None) == 0
    p = shy.default_params()
    p.evap_rate = 2.0
    w = C.c_void_p()
    assert L.shy_world_create(8, 8, C.byref(p), 1, C.byref(w)) == -1
    n = (C.c_int * 1)(4)
    assert L.shy_batch_create(1, n, n, None, None, None, C.byref(w)) == -1


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="a GPU is present")
def test_no_device_is_an_error_not_a_fallback(shy):
    w = C.c_void_p()
    rc = shy.lib().shy_world_create(64, 64, None, 1, C.byref(w))
    assert rc == -4 and not w.value
    with pytest.raises(shy.ShyError):
        shy.World(64, 64)


def test_cpp_facade_compiles(shy, tmp_path):
    """include/shy_world.hpp (the reference's World/Drop names over the C ABI)
    compiles and links against libshy.so with the host C++ compiler."""
    exe = tmp_path / "facade_loop"
    src = os.path.join(ROOT, "tests", "cpp", "facade_loop.cpp")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), src,
                        "-L" + os.path.dirname(shy._capi.LIB_PATH), "-lshy",
                        "-Wl,-rpath," + os.path.dirname(shy._capi.LIB_PATH), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("field,value", [("evap_rate", float("nan")), ("map_scale", float("inf")),
                                         ("max_age", float("nan")), ("evap_rate", 1.0)])
def test_noalloc_rejects_invalid_parameters_on_the_host(shy, field, value):
    """The no-allocation entry point applies the allocating path's parameter
    checks (a NaN fails them) before it touches a device or a map."""
    L = shy.lib()
    p = shy.default_params()
    setattr(p, field, value)
    x = C.c_void_p(1)  # never dereferenced: the parameter checks come first
    rc = L.shy_erode_noalloc(64, 64, C.byref(p), 1, 0, 100, 1, x, x, x, x, x, None, None)
    assert rc == -1 and b"invalid parameters" in L.shy_last_error()


def test_new_entry_points_check_their_arguments_on_the_host(shy):
    """Launch shape, CUDA graphs, device state and cycle calls refuse a null
    world (and bad values) with SHY_ERR_INVALID_ARG before touching a device."""
    L = shy.lib()
    assert L.shy_world_set_block(None, 256, 1) == -1
    assert L.shy_world_set_graph(None, 4) == -1
    assert L.shy_world_set_resort(None, 16) == -1
    assert L.shy_world_set_settle(None, 1) == -1
    assert L.shy_world_set_state(None, None, None, None, None, 0) == -1
    assert L.shy_world_get_state(None, None, None, None, None, 0) == -1
    c = C.c_uint64()
    assert L.shy_world_get_cycle(None, C.byref(c)) == -1
    assert L.shy_terrain_set_state_device(None, 0, None, None, None, None, 0) == -1
    assert L.shy_terrain_get_state_device(None, 0, None, None, None, None, 0) == -1
    assert L.shy_debug_stall_waits(20_000_000_000) == -1
    assert L.shy_debug_stall_waits(0) == 0
    assert L.shy_sg_set_conv_tile(384, 0) == -1 and b"512" in L.shy_last_error()
    assert L.shy_sg_set_conv_tile(512, 3) == 0 and L.shy_sg_set_conv_tile(0, 0) == 0
