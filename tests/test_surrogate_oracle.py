"""The surrogate's FP64 oracle against torch's float64 CPU operators and
autograd, and the surrogate's host-side pieces.  No GPU."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.nn.functional as F  # noqa: E402

from oracle import surrogate_oracle as so  # noqa: E402


def nchw(x):
    return torch.from_numpy(np.ascontiguousarray(x.transpose(0, 3, 1, 2)))


def nhwc(t):
    return t.detach().numpy().transpose(0, 2, 3, 1)


def torch_w(w):
    cout, taps, cin = w.shape
    k = int(round(taps ** 0.5))
    return torch.from_numpy(np.ascontiguousarray(w.reshape(cout, k, k, cin).transpose(0, 3, 1, 2)))


@pytest.mark.parametrize("k", [1, 3])
def test_conv_and_its_gradients_match_torch(k):
    rng = np.random.default_rng(1)
    x = rng.standard_normal((2, 6, 10, 16))
    w = rng.standard_normal((32, k * k, 16))
    b = rng.standard_normal(32)
    dz = rng.standard_normal((2, 6, 10, 32))
    xt = nchw(x).requires_grad_(True)
    wt = torch_w(w).requires_grad_(True)
    zt = F.conv2d(xt, wt, torch.from_numpy(b), padding=k // 2)
    np.testing.assert_allclose(so.conv(x, w, b), nhwc(zt), rtol=1e-12, atol=1e-10)
    zt.backward(nchw(dz))
    np.testing.assert_allclose(so.conv_dgrad(dz, w), nhwc(xt.grad), rtol=1e-12, atol=1e-10)
    gw = wt.grad.numpy().transpose(0, 2, 3, 1).reshape(32, k * k, 16)
    np.testing.assert_allclose(so.conv_wgrad(x, dz, k), gw, rtol=1e-12, atol=1e-9)


def test_resampling_and_gelu_match_torch():
    rng = np.random.default_rng(2)
    x = rng.standard_normal((2, 8, 6, 16))
    np.testing.assert_allclose(so.pool(x), nhwc(F.avg_pool2d(nchw(x), 2)), rtol=1e-13)
    np.testing.assert_allclose(so.up(x), nhwc(F.interpolate(nchw(x), scale_factor=2, mode="nearest")))
    xt = nchw(x).requires_grad_(True)
    dy = rng.standard_normal((2, 4, 3, 16))
    F.avg_pool2d(xt, 2).backward(nchw(dy))
    np.testing.assert_allclose(so.pool_bwd(dy), nhwc(xt.grad), rtol=1e-13)
    xt = nchw(x).requires_grad_(True)
    dy = rng.standard_normal((2, 16, 12, 16))
    F.interpolate(xt, scale_factor=2, mode="nearest").backward(nchw(dy))
    np.testing.assert_allclose(so.up_bwd(dy), nhwc(xt.grad), rtol=1e-13)
    z = torch.linspace(-6, 6, 1001, dtype=torch.float64, requires_grad=True)
    F.gelu(z).sum().backward()
    np.testing.assert_allclose(so.gelu(z.detach().numpy()), F.gelu(z).detach().numpy(), rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(so.gelu_grad(z.detach().numpy()), z.grad.numpy(), rtol=1e-12, atol=1e-14)


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.standard_normal(10000) * 10.0 ** rng.integers(-8, 8, 10000),
                        np.array([0.0, -0.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 65504.0])])
    want = torch.from_numpy(x.astype(np.float32)).to(torch.bfloat16).to(torch.float64).numpy()
    np.testing.assert_array_equal(so.bf16(x), want)


def torch_unet(params, x):
    """The oracle's U-Net in torch float64 (NCHW)."""
    def conv(name, t, act=True):
        w, b = params[name]
        z = F.conv2d(t, w, b, padding=w.shape[-1] // 2)
        return F.gelu(z) if act else z

    e0 = conv("enc0b", conv("enc0a", x))
    e1 = conv("enc1b", conv("enc1a", F.avg_pool2d(e0, 2)))
    e2 = conv("enc2b", conv("enc2a", F.avg_pool2d(e1, 2)))
    m = conv("mid", F.avg_pool2d(e2, 2))
    up = lambda t: F.interpolate(t, scale_factor=2, mode="nearest")  # noqa: E731
    d2 = conv("dec2b", conv("dec2a", torch.cat([up(m), e2], 1)))
    d1 = conv("dec1b", conv("dec1a", torch.cat([up(d2), e1], 1)))
    d0 = conv("dec0b", conv("dec0a", torch.cat([up(d1), e0], 1)))
    return conv("head", d0, act=False)


def test_unet_backward_matches_torch_autograd():
    params = so.init_params(5)
    rng = np.random.default_rng(6)
    h = rng.random((2, 16, 16))
    norm = {"height_mean": 0.5, "height_scale": 3.0, "slope_scale": 20.0}
    x = so.features(h, norm)
    target = rng.standard_normal((2, 16, 16, 3))
    weights = (1.0, 0.5, 0.25)
    net = so.Net(params)
    zh = net.forward(x)
    L, g = so.loss(zh, target, weights)
    grads = net.backward(g)

    tp = {n: (torch_w(w).requires_grad_(True), torch.from_numpy(b).requires_grad_(True))
          for n, (w, b) in params.items()}
    zt = torch_unet(tp, nchw(x))
    np.testing.assert_allclose(zh, nhwc(zt), rtol=1e-10, atol=1e-12)
    e = zt[:, :3] - nchw(target)
    wv = torch.tensor(weights, dtype=torch.float64).view(1, 3, 1, 1)
    lt = (wv * e * e).sum() / (3 * 2 * 16 * 16)
    lt.backward()
    assert L == pytest.approx(float(lt.detach()), rel=1e-12)
    for name, ci, co, k in so.LAYERS:
        gw = tp[name][0].grad.numpy().transpose(0, 2, 3, 1).reshape(co, k * k, ci)
        np.testing.assert_allclose(grads[name][0], gw, rtol=1e-9, atol=1e-14, err_msg=name)
        np.testing.assert_allclose(grads[name][1], tp[name][1].grad.numpy(), rtol=1e-9, atol=1e-14, err_msg=name)


def test_adamw_matches_torch():
    rng = np.random.default_rng(7)
    p0 = rng.standard_normal(50)
    p = torch.tensor(p0, requires_grad=True)
    opt = torch.optim.AdamW([p], lr=1e-2, betas=(0.9, 0.99), eps=1e-8, weight_decay=0.1)
    q, m, v = p0.copy(), np.zeros(50), np.zeros(50)
    for t in range(1, 6):
        g = rng.standard_normal(50)
        p.grad = torch.tensor(g)
        opt.step()
        q, m, v = so.adamw(q, g, m, v, 1e-2, 0.9, 0.99, 1e-8, 0.1, t)
    # torch applies the decay as p *= 1 - lr*wd before the Adam step, the
    # oracle (and the kernel) as lr*wd*p inside the same update
    np.testing.assert_allclose(q, p.detach().numpy(), rtol=1e-3, atol=1e-5)


def test_layer_table_and_counts_agree_with_the_oracle():
    from simplehydrology_gb300 import surrogate as sg
    assert sg.LAYERS == so.LAYERS
    assert sg.param_count() == sum(w.size + b.size for w, b in so.init_params(0).values()) == 1_361_040
    # forward multiply-adds per level-0 pixel, from the layer shapes
    macs = sum(9 * ci * co / 4 ** lvl for (ci, co, lvl) in
               [(16, 32, 0), (32, 32, 0), (32, 64, 1), (64, 64, 1), (64, 128, 2), (128, 128, 2), (128, 256, 3),
                (384, 128, 2), (128, 128, 2), (192, 64, 1), (64, 64, 1), (96, 32, 0), (32, 32, 0)]) + 32 * 16
    assert sg.flops_per_pixel(False) == pytest.approx(2 * macs)
    assert sg.flops_per_pixel(True) == pytest.approx(6 * macs - 2 * 9 * 16 * 32)


def test_norm_targets_round_trip():
    from simplehydrology_gb300 import surrogate as sg
    rng = np.random.default_rng(8)
    h = rng.random((3, 8, 8))
    d = rng.random((3, 8, 8)) * 5
    mx, my = rng.standard_normal((2, 3, 8, 8))
    n = sg.Norm.fit(h, d, mx, my)
    t = n.targets(d, mx, my).astype(np.float64)
    back = t * np.asarray(n.out_scale) + np.asarray(n.out_mean)
    np.testing.assert_allclose(np.expm1(back[..., 0]), d, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(back[..., 1], mx, rtol=1e-5, atol=1e-6)


def test_entry_points_validate_before_touching_a_device(shy):
    lib = shy._capi.lib()
    d = shy._capi.SgConvDesc(1, 8, 8, 8, 16, 3)  # cin not a multiple of 16
    rc = lib.shy_sg_conv_forward(C.byref(d), C.c_void_p(16), 16, C.c_void_p(16), None, C.c_void_p(16), 16, 0,
                                 None, 0, 0, 0, None)
    assert rc == shy._capi.SHY_ERR_INVALID_ARG
    d = shy._capi.SgConvDesc(1, 8, 8, 16, 16, 5)  # kernel size
    assert lib.shy_sg_conv_wgrad(C.byref(d), C.c_void_p(16), 16, C.c_void_p(16), 16, C.c_void_p(16),
                                 None) == shy._capi.SHY_ERR_INVALID_ARG
    # misaligned bf16 tensor
    assert lib.shy_sg_pool_forward(1, 8, 8, 16, C.c_void_p(18), 16, 0, C.c_void_p(32), 16, 0,
                                   None) == shy._capi.SHY_ERR_INVALID_ARG
    assert lib.shy_sg_pool_forward(1, 7, 8, 16, C.c_void_p(16), 16, 0, C.c_void_p(32), 16, 0,
                                   None) == shy._capi.SHY_ERR_INVALID_ARG
    assert "shy_sg_pool_forward" in lib.shy_last_error().decode()


def test_unet_gradients_match_finite_differences():
    """Central differences of the oracle's loss against its backward pass,
    for a few weights and biases of the first, middle and last layers."""
    params = so.init_params(9)
    rng = np.random.default_rng(10)
    x = so.features(rng.random((1, 16, 16)), {"height_mean": 0.5, "height_scale": 3.0, "slope_scale": 20.0})
    target = rng.standard_normal((1, 16, 16, 3))

    def loss_of(p):
        net = so.Net(p)
        return so.loss(net.forward(x), target, (1.0, 1.0, 1.0))[0]

    net = so.Net(params)
    zh = net.forward(x)
    _, g = so.loss(zh, target, (1.0, 1.0, 1.0))
    grads = net.backward(g)
    eps = 1e-6
    for name in ("enc0a", "mid", "dec1a", "head"):
        w, b = params[name]
        for idx in [tuple(rng.integers(0, n) for n in w.shape) for _ in range(3)]:
            wp, wm = w.copy(), w.copy()
            wp[idx] += eps
            wm[idx] -= eps
            fd = (loss_of({**params, name: (wp, b)}) - loss_of({**params, name: (wm, b)})) / (2 * eps)
            assert fd == pytest.approx(grads[name][0][idx], rel=1e-5, abs=1e-9), (name, idx)
        j = int(rng.integers(0, b.size))
        bp, bm = b.copy(), b.copy()
        bp[j] += eps
        bm[j] -= eps
        fd = (loss_of({**params, name: (w, bp)}) - loss_of({**params, name: (w, bm)})) / (2 * eps)
        assert fd == pytest.approx(grads[name][1][j], rel=1e-5, abs=1e-9), (name, j)


class _StubNet:
    """Stands in for Surrogate in train(): records each step's batch on the CPU."""

    def __init__(self, norm):
        self.torch = torch
        self.dev = torch.device("cpu")
        self.norm = norm
        self.steps = []

    def train_step(self, h, t, lr):
        self.steps.append((h.clone(), t.clone(), lr))
        return torch.zeros(1, dtype=torch.float64)


def test_training_loop_crops_flips_and_schedule():
    from simplehydrology_gb300 import surrogate as sg
    rng = np.random.default_rng(11)
    n, side = 3, 32
    H = rng.random((n, side, side)).astype(np.float32)
    D = rng.random((n, side, side)).astype(np.float32) * 3
    MX, MY = rng.standard_normal((2, n, side, side)).astype(np.float32)
    norm = sg.Norm.fit(H, D, MX, MY)
    net = _StubNet(norm)
    losses = sg.train(net, H, D, MX, MY, epochs=2, batch=4, lr=1e-3, seed=5, crop=16, steps_per_epoch=3)
    assert len(losses) == 2 and len(net.steps) == 6
    mean, scale = np.asarray(norm.out_mean), np.asarray(norm.out_scale)
    for h, t, lr in net.steps:
        assert tuple(h.shape) == (4, 16, 16) and tuple(t.shape) == (4, 16, 16, 3)
        for i in range(4):
            hi, raw = h[i].numpy(), t[i].numpy() * scale + mean
            # the crop is a window at a multiple of 8 of some map, flipped along rows and/or columns
            found = False
            for k in range(n):
                for oy in range(0, side - 15, 8):
                    for ox in range(0, side - 15, 8):
                        for fy in (False, True):
                            for fx in (False, True):
                                w = H[k, oy:oy + 16, ox:ox + 16]
                                w = w[::-1] if fy else w
                                w = w[:, ::-1] if fx else w
                                if not np.array_equal(w, hi):
                                    continue
                                sl = (k, slice(oy, oy + 16), slice(ox, ox + 16))
                                mx, my = MX[sl], MY[sl]
                                d = D[sl]
                                if fy:
                                    d, mx, my = d[::-1], -mx[::-1], my[::-1]
                                if fx:
                                    d, mx, my = d[:, ::-1], mx[:, ::-1], -my[:, ::-1]
                                np.testing.assert_allclose(np.expm1(raw[..., 0]), d, rtol=1e-4, atol=1e-5)
                                np.testing.assert_allclose(raw[..., 1], mx, rtol=1e-4, atol=1e-5)
                                np.testing.assert_allclose(raw[..., 2], my, rtol=1e-4, atol=1e-5)
                                found = True
            assert found
    lrs = [lr for _, _, lr in net.steps]
    assert lrs[0] == pytest.approx(1e-3) and all(a > b for a, b in zip(lrs, lrs[1:])) and lrs[-1] > 0


def test_tuning_settings_reject_bad_values(shy):
    lib = shy._capi.lib()
    bad = shy._capi.SHY_ERR_INVALID_ARG
    assert lib.shy_sg_set_conv_path(7) == bad
    assert lib.shy_sg_set_conv_tile(100, 0) == bad and lib.shy_sg_set_conv_tile(128, 9) == bad
    assert lib.shy_sg_set_wgrad_tile(32, 0) == bad and lib.shy_sg_set_wgrad_tile(64, 1) == bad
    assert lib.shy_sg_set_conv_tap_rows(2) == bad
    assert "shy_sg_set_conv_tap_rows" in lib.shy_last_error().decode()
    # valid values are accepted, and the defaults put back
    for call in ((lib.shy_sg_set_conv_tile, (256, 3)), (lib.shy_sg_set_wgrad_tile, (64, 2)),
                 (lib.shy_sg_set_conv_tap_rows, (1,)), (lib.shy_sg_set_conv_path, (2,))):
        assert call[0](*call[1]) == shy._capi.SHY_OK
    assert lib.shy_sg_set_conv_tile(0, 0) == 0 and lib.shy_sg_set_wgrad_tile(0, 0) == 0
    assert lib.shy_sg_set_conv_tap_rows(3) == 0 and lib.shy_sg_set_conv_path(0) == 0
    # a descriptor's own tile is checked per call, before any device work
    import ctypes as C
    d = shy._capi.SgConvDesc(1, 8, 8, 16, 16, 3, 96, 0)
    assert lib.shy_sg_conv_forward(C.byref(d), C.c_void_p(16), 16, C.c_void_p(16), None, C.c_void_p(16), 16, 0,
                                   None, 0, 0, 0, None) == bad
