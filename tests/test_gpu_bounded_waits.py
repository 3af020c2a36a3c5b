"""Failure detection without a GPU fault: the library's bounded device waits
run out cleanly and the context stays usable.

With the test hook shy_debug_stall_waits on, the first grid barrier of a
batched cycle, and the first pipeline wait of a surrogate TMA convolution,
wait for an event that never happens (an arrival that never comes, an
mbarrier nothing arrives at), give up after the hook's limit and take the
kernel's give-up path.  The call must report SHY_ERR_TIMEOUT; then, with
the hook off, the same world and the same convolution must give the
oracle's results again."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHY_ERR_TIMEOUT = -5
STALL_NS = 2_000_000  # 2 ms


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.fixture
def stall(shy):
    L = shy.lib()
    assert L.shy_debug_stall_waits(STALL_NS) == 0
    yield L
    assert L.shy_debug_stall_waits(0) == 0


def test_hook_rejects_long_stalls(shy):
    L = shy.lib()
    assert L.shy_debug_stall_waits(20_000_000_000) == -1
    assert L.shy_debug_stall_waits(0) == 0


@pytest.mark.parametrize("redeal", [False, True])
def test_batched_barrier_times_out_then_world_recovers(shy, po, stall, redeal):
    """Both instantiations of the lock-step kernel: slots in shared memory,
    and slots in global memory with the live drops re-dealt every step."""
    nx, ny, drops, seed = 96, 80, 600, 11
    H = po.value_noise(nx, ny, 3)
    w = shy.World(nx, ny, seed=seed)
    if redeal:
        w.set_launch(0, 1)
        w.set_block(256, 0)
        w.set_resort(1)
        w.set_settle(1)
    w.set_field("height", H)
    with pytest.raises(shy.ShyError) as ei:
        w.erode(drops, 1)
    assert ei.value.code == SHY_ERR_TIMEOUT
    assert b"timed out" in stall.shy_last_error()
    # hook off: the same world, reset to the same start and cycle index,
    # erodes like the oracle again
    assert stall.shy_debug_stall_waits(0) == 0
    w.set_field("height", H)
    for f in ("discharge", "momentum_x", "momentum_y"):
        w.set_field(f, np.zeros((nx, ny), np.float32))
    w.set_cycle(0)
    w.reset_stats()
    w.erode(drops, 2)
    m = po.Maps(nx, ny, height=H)
    acc = po.erode_batched(m, seed, 0, drops, 2)
    for k, name in enumerate(po.FIELDS):
        assert np.array_equal(bits(w.get_field(name)), bits(m.f[k])), name
    assert w.stats().drop_steps == acc.steps
    w.close()


def test_noalloc_barrier_times_out_then_recovers(shy, stall):
    torch = pytest.importorskip("torch")
    nx, ny, drops, seed = 64, 64, 800, 4
    p = shy.default_params()
    w = shy.World(nx, ny, params=p, seed=seed)
    w.generate(seed, 8)
    h0 = w.get_field("height")
    maps = {f: torch.zeros((nx, ny), dtype=torch.float32, device="cuda")
            for f in ("height", "discharge", "momentum_x", "momentum_y", "root_density")}

    def call():
        maps["height"].copy_(torch.from_numpy(h0))
        for f in ("discharge", "momentum_x", "momentum_y"):
            maps[f].zero_()
        torch.cuda.synchronize()
        return stall.shy_erode_noalloc(nx, ny, C.byref(p), seed, 0, drops, 1,
                                       *[maps[f].data_ptr() for f in ("height", "discharge", "momentum_x",
                                                                      "momentum_y", "root_density")],
                                       None, None)

    assert call() == SHY_ERR_TIMEOUT
    assert stall.shy_debug_stall_waits(0) == 0
    assert call() == 0, stall.shy_last_error()
    w.erode(drops, 1)
    for f in ("height", "discharge", "momentum_x", "momentum_y"):
        assert np.array_equal(bits(maps[f].cpu().numpy()), bits(w.get_field(f))), f
    w.close()


def test_surrogate_convolution_wait_times_out_then_recovers(shy, stall):
    torch = pytest.importorskip("torch")
    from oracle import surrogate_oracle as so
    from simplehydrology_gb300._capi import SgConvDesc
    L = stall
    assert L.shy_sg_set_conv_path(0) == 0  # the TMA path, where the hook sits
    B, H, W, ci, co, k = 1, 16, 16, 32, 64, 3
    rng = np.random.default_rng(5)
    x = so.bf16(rng.standard_normal((B, H, W, ci)))
    wt = so.bf16(rng.standard_normal((co, k * k, ci)) / np.sqrt(k * k * ci))
    P = B * H * W
    xd = torch.from_numpy(x.reshape(P, ci).astype(np.float32)).cuda().to(torch.bfloat16)
    wd = torch.from_numpy(wt.ravel().astype(np.float32)).cuda().to(torch.bfloat16)
    z = torch.full((P, co), 7.0, device="cuda")
    d = SgConvDesc(B, H, W, ci, co, k)

    def conv():
        z.fill_(7.0)
        rc = L.shy_sg_conv_forward(C.byref(d), C.c_void_p(xd.data_ptr()), ci, C.c_void_p(wd.data_ptr()), None,
                                   C.c_void_p(z.data_ptr()), co, 0, None, 0, 0, 0, None)
        assert rc == 0, L.shy_last_error()
        torch.cuda.synchronize()
        return L.shy_sg_status()

    assert conv() == SHY_ERR_TIMEOUT
    assert torch.all(z == 7.0), "a convolution that gave up must skip its epilogue"
    assert L.shy_debug_stall_waits(0) == 0
    assert conv() == 0, L.shy_last_error()
    want = so.conv(x, wt).reshape(P, co)
    bound = so.conv(np.abs(x), np.abs(wt)).reshape(P, co)
    got = z.double().cpu().numpy()
    assert np.all(np.abs(got - want) <= 1e-5 * bound + 1e-6)
