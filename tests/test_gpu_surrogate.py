"""The surrogate's device kernels (include/shy_surrogate.h) against the FP64
oracle (oracle/surrogate_oracle.py), through the C ABI.

Tolerances: the tensor-core convolutions multiply bf16 operands exactly and
accumulate in f32, so they must agree with the float64 result on the same
bf16 inputs to within 1e-5 of the sum of the terms' magnitudes.  Results
stored as bf16 must agree to within one bf16 rounding (2^-8 relative).  The
whole network, with bf16 storage emulated in the oracle, must agree to 2 %
relative L2 (rounding flips propagate through 14 layers); the pure-FP64
figures are reported next to it."""
import ctypes as C

import numpy as np
import pytest

from oracle import surrogate_oracle as so

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

BF16_REL = 2.0 ** -8


@pytest.fixture(scope="module")
def sg(shy):
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from simplehydrology_gb300 import surrogate
    return surrogate


def lib():
    from simplehydrology_gb300 import _capi
    return _capi.lib()


def ok(rc):
    from simplehydrology_gb300 import _capi
    _capi.check(rc)


_alive = []


@pytest.fixture(autouse=True)
def _release():
    yield
    torch.cuda.synchronize()
    _alive.clear()


def p(t):
    """Device pointer of a tensor, which stays referenced until the test
    ends (a temporary freed before its kernel runs could be reused)."""
    if t is None:
        return None
    _alive.append(t)
    return C.c_void_p(t.data_ptr())


def dev(a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to("cuda").to(dtype)


def host(t):
    return t.float().cpu().numpy().astype(np.float64)


def status():
    ok(lib().shy_sg_status())


CONV_CASES = [  # batch, h, w, cin, cout, k, x pixel stride
    (1, 12, 12, 16, 32, 3, 16),    # 144 pixels: a partial M tile; kc 16
    (2, 8, 16, 32, 16, 1, 48),     # the head's shape; strided input
    (1, 16, 8, 96, 96, 3, 96),     # kc 32, N tile 96
    (1, 8, 8, 384, 128, 3, 384),   # kc 64, 54 K chunks
    (2, 4, 4, 128, 256, 3, 128),   # two N tiles of 128
    (1, 16, 16, 32, 192, 3, 32),   # two N tiles of 96
]


@pytest.fixture(params=[0, 3, 1, 2], ids=["tma", "tma-tap-by-tap", "staged", "persistent"])
def conv_path(request, sg):
    """The operand-staging paths of the convolutions (3: the TMA path with one
    input box per tap); the TMA path is restored after."""
    path = 0 if request.param == 3 else request.param
    ok(lib().shy_sg_set_conv_path(path))
    ok(lib().shy_sg_set_conv_tap_rows(1 if request.param == 3 else 3))
    yield path
    ok(lib().shy_sg_set_conv_path(0))
    ok(lib().shy_sg_set_conv_tap_rows(3))


@pytest.fixture(params=[(0, 0), (256, 2), (256, 3), (128, 4), (512, 2), (512, 3)],
                ids=["auto", "256px2", "256px3", "128px4", "512px2", "512px3"])
def conv_tile(request, sg):
    """The TMA convolution's pixel tiles and depths; the automatic choice is restored after."""
    ok(lib().shy_sg_set_conv_tile(*request.param))
    yield request.param
    ok(lib().shy_sg_set_conv_tile(0, 0))


@pytest.mark.parametrize("case", CONV_CASES)
def test_conv_forward_matches_oracle(sg, conv_path, conv_tile, case):
    if conv_path == 1 and conv_tile != (0, 0):
        pytest.skip("the tile applies to the TMA paths only")
    B, H, W, ci, co, k, xs = case
    rng = np.random.default_rng(sum(case))
    x = so.bf16(rng.standard_normal((B, H, W, xs)))
    w = so.bf16(rng.standard_normal((co, k * k, ci)) / np.sqrt(k * k * ci))
    b = rng.standard_normal(co).astype(np.float32).astype(np.float64)
    P = B * H * W
    xd, wd, bd = dev(x.reshape(P, xs), torch.bfloat16), dev(w.ravel(), torch.bfloat16), dev(b, torch.float32)
    zs, zo, as_, ao = co + 8, 4, co + 16, 8
    z = torch.full((P, zs), 7.0, device="cuda")
    a = torch.zeros((P, as_), dtype=torch.bfloat16, device="cuda")
    from simplehydrology_gb300._capi import SgConvDesc
    d = SgConvDesc(B, H, W, ci, co, k)
    if conv_path == 2 and conv_tile[0] == 512:
        # the persistent path double-buffers its accumulators: four of them
        # would not fit in tensor memory, so the call is refused up front
        rc = lib().shy_sg_conv_forward(C.byref(d), p(xd), xs, p(wd), p(bd), p(z), zs, zo, p(a), as_, ao, 1, None)
        assert rc == -1 and b"512" in lib().shy_last_error()
        return
    ok(lib().shy_sg_conv_forward(C.byref(d), p(xd), xs, p(wd), p(bd), p(z), zs, zo, p(a), as_, ao, 1, None))
    status()
    want = so.conv(x[..., :ci], w, b).reshape(P, co)
    bound = so.conv(np.abs(x[..., :ci]), np.abs(w)).reshape(P, co) + np.abs(b)
    zg = host(z)
    assert np.all(np.abs(zg[:, zo:zo + co] - want) <= 1e-5 * bound + 1e-6)
    assert np.all(zg[:, :zo] == 7.0) and np.all(zg[:, zo + co:] == 7.0), "wrote outside its channels"
    ag = host(a)
    g = so.gelu(zg[:, zo:zo + co])
    assert np.all(np.abs(ag[:, ao:ao + co] - g) <= BF16_REL * np.abs(g) + 1e-6)
    assert np.all(ag[:, :ao] == 0) and np.all(ag[:, ao + co:] == 0)


@pytest.fixture(params=[(0, 0), (64, 3), (128, 2)], ids=["auto", "64px", "128px"])
def wgrad_tile(request, sg):
    """The TMA weight gradient's pixel tiles and depths; the automatic choice is restored after."""
    ok(lib().shy_sg_set_wgrad_tile(*request.param))
    yield request.param
    ok(lib().shy_sg_set_wgrad_tile(0, 0))


@pytest.mark.parametrize("case", CONV_CASES)
def test_weight_gradient_matches_oracle(sg, conv_path, wgrad_tile, case):
    if conv_path != 0 and wgrad_tile != (0, 0):
        pytest.skip("the weight gradient's tile is covered on the TMA path")
    B, H, W, ci, co, k, xs = case
    rng = np.random.default_rng(sum(case) + 1)
    x = so.bf16(rng.standard_normal((B, H, W, xs)))
    dz = so.bf16(rng.standard_normal((B, H, W, co)))
    P = B * H * W
    dw0 = rng.standard_normal((co, k * k, ci)).astype(np.float32).astype(np.float64)
    dw = dev(dw0.ravel(), torch.float32)
    # every device tensor stays referenced until the kernel has run
    xd, dzd = dev(x.reshape(P, xs), torch.bfloat16), dev(dz.reshape(P, co), torch.bfloat16)
    from simplehydrology_gb300._capi import SgConvDesc
    d = SgConvDesc(B, H, W, ci, co, k)
    ok(lib().shy_sg_conv_wgrad(C.byref(d), p(xd), xs, p(dzd), co, p(dw), None))
    status()
    want = dw0 + so.conv_wgrad(x[..., :ci], dz, k)
    bound = np.abs(dw0) + so.conv_wgrad(np.abs(x[..., :ci]), np.abs(dz), k)
    got = host(dw).reshape(co, k * k, ci)
    assert np.all(np.abs(got - want) <= 1e-5 * bound + 1e-6)


@pytest.mark.parametrize("case", CONV_CASES[:4])
def test_input_gradient_through_flipped_weights(sg, conv_path, case):
    B, H, W, ci, co, k, _ = case
    rng = np.random.default_rng(sum(case) + 2)
    w32 = rng.standard_normal((co, k * k, ci)).astype(np.float32)
    dz = so.bf16(rng.standard_normal((B, H, W, co)))
    wd = dev(w32.ravel(), torch.float32)
    wb = torch.empty(w32.size, dtype=torch.bfloat16, device="cuda")
    wf = torch.empty(w32.size, dtype=torch.bfloat16, device="cuda")
    ok(lib().shy_sg_weight_prep(co, k, ci, p(wd), p(wb), p(wf), None))
    wq = so.bf16(w32)
    assert np.array_equal(host(wb).reshape(co, k * k, ci), wq)
    assert np.array_equal(host(wf).reshape(ci, k * k, co), so.flip(wq))
    P = B * H * W
    dx = torch.zeros((P, ci), device="cuda")
    dzd = dev(dz.reshape(P, co), torch.bfloat16)
    from simplehydrology_gb300._capi import SgConvDesc
    d = SgConvDesc(B, H, W, co, ci, k)
    ok(lib().shy_sg_conv_forward(C.byref(d), p(dzd), co, p(wf), None, p(dx), ci, 0, None, 0, 0, 0, None))
    status()
    want = so.conv_dgrad(dz, wq).reshape(P, ci)
    bound = so.conv_dgrad(np.abs(dz), np.abs(wq)).reshape(P, ci)
    assert np.all(np.abs(host(dx) - want) <= 1e-5 * bound + 1e-6)


@pytest.mark.parametrize("case", [CONV_CASES[0], CONV_CASES[2], CONV_CASES[4]])
def test_input_gradient_fused_with_gelu_backward(sg, conv_path, case):
    """shy_sg_conv_input_grad: the input gradient times gelu'(z_prev), in bf16."""
    B, H, W, ci, co, k, _ = case
    rng = np.random.default_rng(sum(case) + 3)
    w32 = rng.standard_normal((co, k * k, ci)).astype(np.float32) / np.sqrt(k * k * co)
    dz = so.bf16(rng.standard_normal((B, H, W, co)))
    P = B * H * W
    zs = ci + 4
    zprev = (rng.standard_normal((P, zs)) * 2).astype(np.float32).astype(np.float64)
    wd = dev(w32.ravel(), torch.float32)
    wb = torch.empty(w32.size, dtype=torch.bfloat16, device="cuda")
    wf = torch.empty(w32.size, dtype=torch.bfloat16, device="cuda")
    ok(lib().shy_sg_weight_prep(co, k, ci, p(wd), p(wb), p(wf), None))
    out = torch.zeros((P, ci), dtype=torch.bfloat16, device="cuda")
    from simplehydrology_gb300._capi import SgConvDesc
    d = SgConvDesc(B, H, W, co, ci, k)
    ok(lib().shy_sg_conv_input_grad(C.byref(d), p(dev(dz.reshape(P, co), torch.bfloat16)), co, p(wf),
                                    p(dev(zprev, torch.float32)), zs, 4, p(out), None))
    status()
    dx = so.conv_dgrad(dz, so.bf16(w32)).reshape(P, ci)
    bound = so.conv_dgrad(np.abs(dz), np.abs(so.bf16(w32))).reshape(P, ci)
    gg = so.gelu_grad(zprev[:, 4:4 + ci])
    want = dx * gg
    got = host(out)
    # gelu' in f32 carries an absolute error of ~1e-7 where 1 + erf cancels (z << 0)
    assert np.all(np.abs(got - want) <= BF16_REL * np.abs(want) + (1e-5 * bound + 1e-6) * np.abs(gg)
                  + 1e-6 * np.abs(dx))


def test_elementwise_kernels_match_oracle(sg):
    rng = np.random.default_rng(11)
    B, H, W, c = 2, 8, 12, 32
    P = B * H * W
    # pooling from a channel slice of a wider tensor
    x = so.bf16(rng.standard_normal((B, H, W, 3 * c)))
    y = torch.zeros((P // 4, c), dtype=torch.bfloat16, device="cuda")
    ok(lib().shy_sg_pool_forward(B, H, W, c, p(dev(x.reshape(P, 3 * c), torch.bfloat16)), 3 * c, 2 * c, p(y), c,
                                 0, None))
    want = so.pool(x[..., 2 * c:]).reshape(-1, c)
    assert np.all(np.abs(host(y) - want) <= BF16_REL * np.abs(want))
    dy = rng.standard_normal((B, H // 2, W // 2, c)).astype(np.float32).astype(np.float64)
    dx0 = rng.standard_normal((B, H, W, 3 * c)).astype(np.float32).astype(np.float64)
    dx = dev(dx0.reshape(P, 3 * c), torch.float32)
    ok(lib().shy_sg_pool_backward(B, H, W, c, p(dev(dy.reshape(-1, c), torch.float32)), c, 0, p(dx), 3 * c, 2 * c,
                                  None))
    want = dx0.copy()
    want[..., 2 * c:] += so.pool_bwd(dy)
    np.testing.assert_allclose(host(dx), want.reshape(P, 3 * c), rtol=1e-6, atol=1e-7)
    # upsampling into a channel slice, and its adjoint
    xc = so.bf16(rng.standard_normal((B, H, W, 2 * c)))
    yf = torch.zeros((4 * P, 3 * c), dtype=torch.bfloat16, device="cuda")
    ok(lib().shy_sg_upsample_forward(B, H, W, 2 * c, p(dev(xc.reshape(P, 2 * c), torch.bfloat16)), 2 * c, 0, p(yf),
                                     3 * c, 0, None))
    got = host(yf).reshape(B, 2 * H, 2 * W, 3 * c)
    assert np.array_equal(got[..., :2 * c], so.up(xc)) and np.all(got[..., 2 * c:] == 0)
    dyf = rng.standard_normal((B, 2 * H, 2 * W, 3 * c)).astype(np.float32).astype(np.float64)
    dxc = torch.zeros((P, 2 * c), device="cuda")
    ok(lib().shy_sg_upsample_backward(B, H, W, 2 * c, p(dev(dyf.reshape(-1, 3 * c), torch.float32)), 3 * c, 0,
                                      p(dxc), 2 * c, 0, None))
    np.testing.assert_allclose(host(dxc), so.up_bwd(dyf[..., :2 * c]).reshape(P, 2 * c), rtol=1e-6, atol=1e-6)
    # GELU backward from strided f32 inputs
    da = rng.standard_normal((P, 3 * c)).astype(np.float32).astype(np.float64)
    z = (rng.standard_normal((P, c)) * 3).astype(np.float32).astype(np.float64)
    dz = torch.empty((P, c), dtype=torch.bfloat16, device="cuda")
    dbg = dev(np.full(c, 0.5), torch.float32)
    ok(lib().shy_sg_gelu_backward(P, c, p(dev(da, torch.float32)), 3 * c, c, p(dev(z, torch.float32)), c, 0, p(dz),
                                  p(dbg), None))
    want = da[:, c:2 * c] * so.gelu_grad(z)
    got = host(dz)
    assert np.all(np.abs(got - want) <= BF16_REL * np.abs(want) + 1e-6 * np.abs(da[:, c:2 * c]))
    np.testing.assert_allclose(host(dbg), 0.5 + got.sum(0), rtol=1e-5, atol=1e-4)
    # bias gradient
    g = so.bf16(rng.standard_normal((P, 48)))
    for ch in (32, 48, 16):  # dividing 256 or not
        db0 = np.ones(ch)
        db = dev(db0, torch.float32)
        ok(lib().shy_sg_bias_grad(P, ch, p(dev(g, torch.bfloat16)), 48, p(db), None))
        np.testing.assert_allclose(host(db), db0 + g[:, :ch].sum(0), rtol=1e-5, atol=1e-4)
    status()


def test_loss_features_decode_adamw_match_oracle(sg, shy):
    rng = np.random.default_rng(12)
    B, H, W = 2, 16, 24
    P = B * H * W
    zh = rng.standard_normal((P, 16)).astype(np.float32).astype(np.float64)
    t = rng.standard_normal((P, 3)).astype(np.float32).astype(np.float64)
    wts = (1.0, 0.5, 0.25)
    dz = torch.empty((P, 16), dtype=torch.bfloat16, device="cuda")
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    ok(lib().shy_sg_loss(P, p(dev(zh, torch.float32)), 16, p(dev(t, torch.float32)), (C.c_float * 3)(*wts), p(dz),
                         p(loss), None))
    L, g = so.loss(zh.reshape(1, 1, P, 16), t.reshape(1, 1, P, 3), wts)
    assert float(loss.item()) == pytest.approx(L, rel=1e-6)
    g = g.reshape(P, 16)
    assert np.all(np.abs(host(dz) - g) <= BF16_REL * np.abs(g) + 1e-12)

    norm = sg.Norm(0.4, 3.0, 50.0, (0.1, 0.2, -0.1), (2.0, 0.5, 0.25))
    h = rng.random((B, H, W)).astype(np.float32)
    x = torch.empty((P, 16), dtype=torch.bfloat16, device="cuda")
    ok(lib().shy_sg_features(B, H, W, p(dev(h, torch.float32)), C.byref(norm.c()), p(x), None))
    want = so.features(h, {"height_mean": 0.4, "height_scale": 3.0, "slope_scale": 50.0}).reshape(P, 16)
    assert np.all(np.abs(host(x) - want) <= 2 * BF16_REL * np.abs(want) + 1e-5)

    outs = [torch.empty(P, device="cuda") for _ in range(3)]
    ok(lib().shy_sg_decode(P, p(dev(zh, torch.float32)), 16, C.byref(norm.c()), *[p(o) for o in outs], None))
    np.testing.assert_allclose(host(outs[0]), np.maximum(0, np.expm1(zh[:, 0] * 2.0 + 0.1)), rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(host(outs[1]), zh[:, 1] * 0.5 + 0.2, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(host(outs[2]), zh[:, 2] * 0.25 - 0.1, rtol=1e-6, atol=1e-6)

    n = 1000
    p0 = rng.standard_normal(n)
    pd, md, vd = dev(p0, torch.float32), torch.zeros(n, device="cuda"), torch.zeros(n, device="cuda")
    q, m, v = p0.astype(np.float32).astype(np.float64), np.zeros(n), np.zeros(n)
    for step in range(1, 4):
        gr = rng.standard_normal(n).astype(np.float32).astype(np.float64)
        a = shy._capi.SgAdamw(1e-2, 0.9, 0.999, 1e-8, 0.01, 1 - 0.9 ** step, 1 - 0.999 ** step)
        ok(lib().shy_sg_adamw(n, p(pd), p(dev(gr, torch.float32)), p(md), p(vd), C.byref(a), None))
        q, m, v = so.adamw(q, gr, m, v, 1e-2, 0.9, 0.999, 1e-8, 0.01, step)
    np.testing.assert_allclose(host(pd), q, rtol=1e-5, atol=1e-6)
    status()


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30))


@pytest.mark.parametrize("path", [0, 2], ids=["tma", "persistent"])
def test_network_gradients_match_oracle(sg, path):
    """One training step's loss and every layer's gradient, device against
    the oracle with bf16 storage emulated (and against pure FP64)."""
    ok(lib().shy_sg_set_conv_path(path))
    try:
        _network_gradients_match_oracle(sg)
    finally:
        ok(lib().shy_sg_set_conv_path(0))


def _network_gradients_match_oracle(sg):
    params = so.init_params(21)
    rng = np.random.default_rng(22)
    B, H, W = 2, 32, 16
    h = rng.random((B, H, W)).astype(np.float32)
    target = rng.standard_normal((B, H, W, 3)).astype(np.float32)
    norm = sg.Norm(0.5, 3.0, 20.0)
    net = sg.Surrogate(init=params, norm=norm)
    ws = net.workspace(B, H, W, True)
    net.features(ws, dev(h, torch.float32))
    ws.target.copy_(dev(target.reshape(-1, 3), torch.float32))
    wts = (1.0, 0.5, 0.25)
    net.loss_and_grads(ws, wts)
    net.status()
    x = so.features(h, {"height_mean": 0.5, "height_scale": 3.0, "slope_scale": 20.0})
    report = {}
    for emulate, tol in ((True, 2e-2), (False, 1e-1)):
        on = so.Net(params, bf16_storage=emulate)
        zh = on.forward(x)
        L, g = so.loss(zh, target.astype(np.float64), wts)
        grads = on.backward(g)
        errs = {"zh": rel_l2(host(ws.zh).reshape(zh.shape)[..., :3], zh[..., :3]),
                "loss": abs(float(ws.loss.item()) - L) / L}
        for name, *_ in so.LAYERS:
            gw, gb = net.grads_of(name)
            errs[name] = max(rel_l2(gw.astype(np.float64), grads[name][0]),
                             rel_l2(gb.astype(np.float64), grads[name][1]))
        report["bf16 emulated" if emulate else "fp64"] = errs
        worst = max(errs.values())
        assert worst <= tol, (emulate, errs)
    print(report)


def test_training_reduces_the_loss(sg):
    """AdamW on the device fits a fixed batch: the loss falls tenfold."""
    B, H, W = 4, 32, 32
    yy, xx = np.meshgrid(np.linspace(0, 1, H), np.linspace(0, 1, W), indexing="ij")
    h = np.stack([0.5 + 0.3 * np.sin(3 * xx + i) * np.cos(2 * yy - i) for i in range(B)]).astype(np.float32)
    t = np.stack([h - 0.5, np.gradient(h, axis=1) * 10, np.gradient(h, axis=2) * 10], axis=-1).astype(np.float32)
    net = sg.Surrogate(seed=3, norm=sg.Norm(0.5, 4.0, 30.0))
    hd, td = dev(h, torch.float32), dev(t, torch.float32)
    losses = []
    for i in range(150):
        losses.append(net.train_step(hd, td, lr=2e-3).clone())
    first, last = float(losses[0].item()), float(losses[-1].item())
    net.status()
    assert last < 0.1 * first, (first, last)


def test_trained_network_beats_the_method_without_it(sg):
    """Trained on pairs from the GPU particle method, the network's maps for
    held-out terrains are closer to the particle method's (log-L2) than zero
    maps (the plain method's start) and than the training set's mean map
    (the best terrain-blind guess)."""
    n_tr, n_te = 96, 8
    H, D, MX, MY = sg.make_pairs(n_tr + n_te, size=128, cycles=30, seed0=500)
    norm = sg.Norm.fit(H[:n_tr], D[:n_tr], MX[:n_tr], MY[:n_tr])
    net = sg.Surrogate(seed=1, norm=norm)
    losses = sg.train(net, H[:n_tr], D[:n_tr], MX[:n_tr], MY[:n_tr], epochs=12, batch=8, lr=2e-3)
    net.status()
    pred = net.predict(torch.from_numpy(H[n_tr:]).cuda())[0].cpu().numpy()
    err = np.mean([sg.log_l2(pred[i], D[n_tr + i]) for i in range(n_te)])
    mean_map = D[:n_tr].mean(0)
    blind = np.mean([sg.log_l2(mean_map, D[n_tr + i]) for i in range(n_te)])
    zero = np.mean([sg.log_l2(0 * mean_map, D[n_tr + i]) for i in range(n_te)])
    print({"loss_by_epoch": losses, "prediction": err, "mean_map": blind, "zero_maps": zero})
    assert losses[-1] < losses[0]
    assert err < blind < zero == 1.0


def test_cpp_host_runs_the_c_abi(sg, tmp_path):
    """tests/cpp/surrogate_conv.cpp: a C++ program (CUDA runtime for memory,
    libshy for the kernels) runs a convolution and its weight gradient and
    checks them against host loops."""
    import os
    import subprocess
    from simplehydrology_gb300 import _capi
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    libdir = os.path.dirname(_capi.LIB_PATH)
    cuda = "/usr/local/cuda"
    exe = tmp_path / "surrogate_conv"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(root, "include"), "-I" + cuda + "/include",
                        os.path.join(root, "tests", "cpp", "surrogate_conv.cpp"), "-L" + libdir, "-lshy",
                        "-L" + cuda + "/lib64", "-lcudart", "-Wl,-rpath," + libdir, "-Wl,-rpath," + cuda + "/lib64",
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok")


def test_autotune_picks_a_tile_per_call(sg):
    """The autotuner times the candidates of every convolution call and the
    step afterwards runs on its choices (each candidate's numerics are
    checked above)."""
    net = sg.Surrogate(seed=4, norm=sg.Norm(0.5, 3.0, 20.0))
    tuned = net.autotune(2, 32, 32, reps=2)
    assert len(tuned) == 3 * len(sg.LAYERS) - 1
    for (name, kind), (cand, ms) in tuned.items():
        assert cand in (sg.WGRAD_TILES if kind == "wgrad" else sg.CONV_TILES)
        assert ms > 0
        assert net.tune[(name, kind)] == cand
    h = torch.rand((2, 32, 32), device="cuda")
    t = torch.randn((2, 32, 32, 3), device="cuda")
    loss = float(net.train_step(h, t, 1e-3).item())
    net.status()
    assert np.isfinite(loss)


def test_device_state_calls_match_host_ones(sg, shy):
    """shy_terrain_get/set_state_device move the same bits as the host state
    calls, with no host copy of the data."""
    w = shy.World(96, 80, seed=3)
    w.generate(3, 8)
    w.erode(500, 2)
    host = w.get_state()
    dev_ = w.get_state_device()
    for k, v in host.items():
        assert np.array_equal(dev_[k].cpu().numpy().view(np.uint32), v.view(np.uint32)), k
    w2 = shy.World(96, 80, seed=3)
    w2.set_state_device(**dev_)
    back = w2.get_state()
    for k, v in host.items():
        assert np.array_equal(back[k].view(np.uint32), v.view(np.uint32)), k
    with pytest.raises(ValueError):  # host tensors are refused before the call
        w2.set_state_device(discharge=torch.zeros(96 * 80))
    w.close()
    w2.close()


def _small_net(sg):
    n_tr = 32
    H, D, MX, MY = sg.make_pairs(n_tr, size=128, cycles=20, seed0=700)
    norm = sg.Norm.fit(H, D, MX, MY)
    net = sg.Surrogate(seed=2, norm=norm)
    sg.train(net, H, D, MX, MY, epochs=4, batch=8, lr=2e-3)
    net.status()
    return net


def test_warm_start_is_device_to_device_and_writes_the_prediction(sg, shy):
    net = _small_net(sg)
    w = shy.World(128, 128, seed=9)
    w.generate(9, 8)
    net.warm_start(w)
    h = torch.from_numpy(w.get_field("height")[None]).cuda()
    d, mx, my = net.predict(h)
    torch.cuda.synchronize()
    for name, t in (("discharge", d), ("momentum_x", mx), ("momentum_y", my)):
        assert np.array_equal(w.get_field(name).view(np.uint32), t[0].cpu().numpy().view(np.uint32)), name
    w.close()


def test_judged_warm_start_falls_back_to_the_plain_method(sg, shy):
    """A prediction the particle method moves by more than the threshold is
    discarded: the world ends bit for bit where the plain method alone ends."""
    net = _small_net(sg)
    drops, k = 1024, 3
    w = shy.World(128, 128, seed=21)
    w.generate(21, 8)
    res = net.warm_start_judged(w, drops, probe_cycles=k, threshold=1e-6)
    assert not res["accepted"] and res["log_l2"] > 1e-6
    plain = shy.World(128, 128, seed=21)
    plain.generate(21, 8)
    plain.erode(drops, k)
    for f in ("height", "discharge", "momentum_x", "momentum_y"):
        assert np.array_equal(w.get_field(f).view(np.uint32), plain.get_field(f).view(np.uint32)), f
    assert w.cycle() == plain.cycle() == k
    w.close()
    plain.close()


def test_judged_warm_start_keeps_an_accepted_prediction(sg, shy):
    """Within the threshold the warm start stands: the world continues from
    the probe cycles run after the prediction."""
    net = _small_net(sg)
    drops, k = 1024, 3
    w = shy.World(128, 128, seed=22)
    w.generate(22, 8)
    res = net.warm_start_judged(w, drops, probe_cycles=k, threshold=10.0)
    assert res["accepted"]
    ref = shy.World(128, 128, seed=22)
    ref.generate(22, 8)
    net.warm_start(ref)
    ref.erode(drops, k)
    for f in ("height", "discharge", "momentum_x", "momentum_y"):
        assert np.array_equal(w.get_field(f).view(np.uint32), ref.get_field(f).view(np.uint32)), f
    w.close()
    ref.close()
