"""shy_erode_noalloc -- batched erosion for callers that cannot allocate
device memory (for example a plugin whose host application's own allocator
holds the GPU) -- against the allocating entry point shy_erode.

Both run the same lock-step cycles; the no-allocation call keeps all of its
working memory in one fixed array inside the library and works on maps the
caller already holds on the device.  The results must match bit for bit on
two calls in a row (the tolerance of every batched-mode test here).  This
file is collected last so that a stop at its first failure has already run
every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_noalloc_matches_allocating_entry_point_two_calls(shy):
    torch = pytest.importorskip("torch")
    L = shy.lib()
    nx, ny, drops, seed = 200, 160, 6000, 5
    p = shy.default_params()
    w = shy.World(nx, ny, params=p, seed=seed)
    w.generate(seed, 8)
    h0 = w.get_field("height")
    dev = torch.device("cuda", 0)
    maps = {f: torch.zeros((nx, ny), dtype=torch.float32, device=dev)
            for f in ("height", "discharge", "momentum_x", "momentum_y", "root_density")}
    maps["height"].copy_(torch.from_numpy(h0))
    torch.cuda.synchronize()
    for call in range(2):
        st = shy.Stats()
        rc = L.shy_erode_noalloc(nx, ny, C.byref(p), seed, call, drops, 1,
                                 maps["height"].data_ptr(), maps["discharge"].data_ptr(),
                                 maps["momentum_x"].data_ptr(), maps["momentum_y"].data_ptr(),
                                 maps["root_density"].data_ptr(), None, C.byref(st))
        assert rc == 0, L.shy_last_error()
        # the allocating path, from the same float maps (a fresh start each call)
        w.set_field("height", w.get_field("height"))
        w.reset_stats()
        w.erode(drops, 1)
        for f in ("height", "discharge", "momentum_x", "momentum_y"):
            got = maps[f].cpu().numpy()
            assert np.array_equal(bits(got), bits(w.get_field(f))), (call, f)
        ws = w.stats()
        assert st.drop_steps == ws.drop_steps and st.drops == ws.drops and st.drops_oob == ws.drops_oob
        assert st.drop_steps > 0
    w.close()


def test_noalloc_rejects_requests_beyond_its_scratch(shy):
    L = shy.lib()
    p = shy.default_params()
    x = C.c_void_p(1)  # never dereferenced: the size checks come first
    rc = L.shy_erode_noalloc(512, 512, C.byref(p), 1, 0, 100, 1, x, x, x, x, x, None, None)
    assert rc == -1 and b"scratch" in L.shy_last_error()
    rc = L.shy_erode_noalloc(64, 64, C.byref(p), 1, 0, 1 << 20, 1, x, x, x, x, x, None, None)
    assert rc == -1 and b"drops" in L.shy_last_error()


def test_noalloc_rejects_host_maps(shy):
    """A host array passed as a map is refused with an error code before any
    kernel runs (it would otherwise be read by the device)."""
    torch = pytest.importorskip("torch")
    L = shy.lib()
    p = shy.default_params()
    nx, ny = 64, 64
    dev = [torch.zeros((nx, ny), dtype=torch.float32, device="cuda") for _ in range(4)]
    host = np.zeros((nx, ny), np.float32)
    ptrs = [t.data_ptr() for t in dev]
    for i in range(5):
        args = ptrs[:i] + [host.ctypes.data] + ptrs[i:]
        rc = L.shy_erode_noalloc(nx, ny, C.byref(p), 1, 0, 100, 1, *args[:5], None, None)
        assert rc == -1 and b"device memory" in L.shy_last_error(), (i, L.shy_last_error())
