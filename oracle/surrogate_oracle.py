"""FP64 CPU restatement of the warm-start surrogate (test infrastructure).

The reference has no learned part: its discharge and momentum maps start at
zero and fill through the lrate blend of World::erode (source/world.h:83-85).
This module restates, in numpy float64, every operation the device kernels
of include/shy_surrogate.h perform, and the U-Net that
simplehydrology_gb300/surrogate.py composes from them:

  * convolutions (3x3 and 1x1, zero padding) and their weight and input
    gradients, on NHWC arrays with weights [cout][tap][cin];
  * GELU (the erf form) and its derivative;
  * 2x2 average pooling, nearest 2x upsampling and their adjoints;
  * the input features, the weighted MSE loss, AdamW with decoupled weight
    decay.

With `bf16=True` the network rounds operands where the device stores bf16
(weights, activations, output gradients), so that the device result can be
compared tightly; without it the whole pass is float64, the error reference
for the device's BF16/FP32 arithmetic.  The manual backward pass here is
itself pinned against torch's float64 CPU autograd in tests/.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use this file.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

IN_CH = 16
OUT_CH = 16
# (name, cin, cout, ksize): the network's convolutions in forward order
LAYERS = (
    ("enc0a", 16, 32, 3), ("enc0b", 32, 32, 3),
    ("enc1a", 32, 64, 3), ("enc1b", 64, 64, 3),
    ("enc2a", 64, 128, 3), ("enc2b", 128, 128, 3),
    ("mid", 128, 256, 3),
    ("dec2a", 384, 128, 3), ("dec2b", 128, 128, 3),
    ("dec1a", 192, 64, 3), ("dec1b", 64, 64, 3),
    ("dec0a", 96, 32, 3), ("dec0b", 32, 32, 3),
    ("head", 32, 16, 1),
)


def bf16(x):
    """Round to bfloat16 (nearest, ties to even), returned as float64."""
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _pad(x, k):
    h = k // 2
    return np.pad(x, ((0, 0), (h, h), (h, h), (0, 0))) if h else x


def conv(x, w, b=None):
    """z[b,y,x,o] = sum_{tap,c} w[o,tap,c] x[b,y+dy,x+dx,c] (+ bias); tap = ky*k + kx."""
    cout, taps, cin = w.shape
    k = int(round(taps ** 0.5))
    B, H, W, _ = x.shape
    xp = _pad(x, k)
    z = np.zeros((B, H, W, cout))
    for t in range(taps):
        ky, kx = divmod(t, k)
        z += np.einsum("bhwc,oc->bhwo", xp[:, ky:ky + H, kx:kx + W, :], w[:, t, :], optimize=True)
    if b is not None:
        z += b
    return z


def conv_wgrad(x, dz, k):
    """dw[o,tap,c] = sum_{b,y,x} dz[b,y,x,o] x[b,y+dy,x+dx,c]."""
    B, H, W, cin = x.shape
    xp = _pad(x, k)
    dw = np.zeros((dz.shape[-1], k * k, cin))
    for t in range(k * k):
        ky, kx = divmod(t, k)
        dw[:, t, :] = np.einsum("bhwo,bhwc->oc", dz, xp[:, ky:ky + H, kx:kx + W, :], optimize=True)
    return dw


def flip(w):
    """Weights of the input-gradient convolution: [cin][taps-1-tap][cout]."""
    return np.ascontiguousarray(w[:, ::-1, :].transpose(2, 1, 0))


def conv_dgrad(dz, w):
    """dx = conv(dz, flip(w)): the adjoint of conv with zero padding."""
    return conv(dz, flip(w))


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def pool(x):
    B, H, W, C = x.shape
    return x.reshape(B, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4))


def pool_bwd(dy):
    return 0.25 * np.repeat(np.repeat(dy, 2, axis=1), 2, axis=2)


def up(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def up_bwd(dy):
    B, H, W, C = dy.shape
    return dy.reshape(B, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


def features(h, norm):
    """Network input from heightmaps h[b, H, W]: 16 channels (normalised
    height, central differences along rows and columns -- one-sided at the
    border -- times slope_scale, 13 zeros)."""
    h = np.asarray(h, np.float64)
    B, H, W = h.shape
    gr = np.empty_like(h)
    gc = np.empty_like(h)
    gr[:, 1:-1] = (h[:, 2:] - h[:, :-2]) / 2
    gr[:, 0] = h[:, 1] - h[:, 0]
    gr[:, -1] = h[:, -1] - h[:, -2]
    gc[:, :, 1:-1] = (h[:, :, 2:] - h[:, :, :-2]) / 2
    gc[:, :, 0] = h[:, :, 1] - h[:, :, 0]
    gc[:, :, -1] = h[:, :, -1] - h[:, :, -2]
    x = np.zeros((B, H, W, IN_CH))
    x[..., 0] = (h - norm["height_mean"]) * norm["height_scale"]
    x[..., 1] = gr * norm["slope_scale"]
    x[..., 2] = gc * norm["slope_scale"]
    return x


def loss(zh, target, weights):
    """Weighted MSE over the first three output channels and its gradient
    (zero in the other channels)."""
    e = zh[..., :3] - target
    wv = np.asarray(weights, np.float64)
    n = e.shape[0] * e.shape[1] * e.shape[2]
    L = float((wv * e * e).sum() / (3 * n))
    g = np.zeros_like(zh)
    g[..., :3] = 2 * wv * e / (3 * n)
    return L, g


def adamw(p, g, m, v, lr, b1, b2, eps, wd, t):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return p - lr * (mh / (np.sqrt(vh) + eps) + wd * p), m, v


def init_params(seed):
    """He-normal weights (std sqrt(2 / fan_in)), zero biases; the head uses
    std sqrt(1 / fan_in).  Returns {name: (w[cout][tap][cin], b[cout])}."""
    rng = np.random.default_rng(seed)
    out = {}
    for name, cin, cout, k in LAYERS:
        fan = k * k * cin
        std = np.sqrt((1.0 if name == "head" else 2.0) / fan)
        out[name] = (rng.standard_normal((cout, k * k, cin)) * std, np.zeros(cout))
    return out


class Net:
    """The U-Net of simplehydrology_gb300/surrogate.py in float64.

    forward(x) keeps what backward needs; backward(dzh) returns
    {name: (dw, db)}.  With bf16=True, weights, stored activations and
    output gradients are rounded to bfloat16 where the device stores them.
    """

    def __init__(self, params, bf16_storage=False):
        self.p = params
        self.q = bf16 if bf16_storage else (lambda a: np.asarray(a, np.float64))

    def _w(self, name):
        return self.q(self.p[name][0])

    def _conv(self, name, x, act=True):
        z = conv(x, self._w(name), self.p[name][1])
        return z, (self.q(gelu(z)) if act else None)

    def forward(self, x):
        q = self.q
        s = {"x0": q(x)}
        s["z_e0a"], s["a_e0a"] = self._conv("enc0a", s["x0"])
        s["z_e0b"], s["a_e0b"] = self._conv("enc0b", s["a_e0a"])
        s["p1"] = q(pool(s["a_e0b"]))
        s["z_e1a"], s["a_e1a"] = self._conv("enc1a", s["p1"])
        s["z_e1b"], s["a_e1b"] = self._conv("enc1b", s["a_e1a"])
        s["p2"] = q(pool(s["a_e1b"]))
        s["z_e2a"], s["a_e2a"] = self._conv("enc2a", s["p2"])
        s["z_e2b"], s["a_e2b"] = self._conv("enc2b", s["a_e2a"])
        s["p3"] = q(pool(s["a_e2b"]))
        s["z_mid"], s["a_mid"] = self._conv("mid", s["p3"])
        s["cat2"] = np.concatenate([up(s["a_mid"]), s["a_e2b"]], axis=-1)
        s["z_d2a"], s["a_d2a"] = self._conv("dec2a", s["cat2"])
        s["z_d2b"], s["a_d2b"] = self._conv("dec2b", s["a_d2a"])
        s["cat1"] = np.concatenate([up(s["a_d2b"]), s["a_e1b"]], axis=-1)
        s["z_d1a"], s["a_d1a"] = self._conv("dec1a", s["cat1"])
        s["z_d1b"], s["a_d1b"] = self._conv("dec1b", s["a_d1a"])
        s["cat0"] = np.concatenate([up(s["a_d1b"]), s["a_e0b"]], axis=-1)
        s["z_d0a"], s["a_d0a"] = self._conv("dec0a", s["cat0"])
        s["z_d0b"], s["a_d0b"] = self._conv("dec0b", s["a_d0a"])
        s["z_head"], _ = self._conv("head", s["a_d0b"], act=False)
        self.s = s
        return s["z_head"]

    def backward(self, dzh):
        q, s = self.q, self.s
        g = {}

        def layer(name, x_in, dz, need_dx=True):
            k = 3 if self.p[name][0].shape[1] == 9 else 1
            g[name] = (conv_wgrad(x_in, dz, k), dz.sum(axis=(0, 1, 2)))
            return conv_dgrad(dz, self._w(name)) if need_dx else None

        def act_bwd(da, z):
            return q(da * gelu_grad(z))

        dz = q(dzh)
        da = layer("head", s["a_d0b"], dz)
        da = layer("dec0b", s["a_d0a"], act_bwd(da, s["z_d0b"]))
        dcat0 = layer("dec0a", s["cat0"], act_bwd(da, s["z_d0a"]))
        da = up_bwd(dcat0[..., :64])
        da = layer("dec1b", s["a_d1a"], act_bwd(da, s["z_d1b"]))
        dcat1 = layer("dec1a", s["cat1"], act_bwd(da, s["z_d1a"]))
        da = up_bwd(dcat1[..., :128])
        da = layer("dec2b", s["a_d2a"], act_bwd(da, s["z_d2b"]))
        dcat2 = layer("dec2a", s["cat2"], act_bwd(da, s["z_d2a"]))
        da = up_bwd(dcat2[..., :256])
        dp3 = layer("mid", s["p3"], act_bwd(da, s["z_mid"]))
        da = dcat2[..., 256:] + pool_bwd(dp3)
        da = layer("enc2b", s["a_e2a"], act_bwd(da, s["z_e2b"]))
        dp2 = layer("enc2a", s["p2"], act_bwd(da, s["z_e2a"]))
        da = dcat1[..., 128:] + pool_bwd(dp2)
        da = layer("enc1b", s["a_e1a"], act_bwd(da, s["z_e1b"]))
        dp1 = layer("enc1a", s["p1"], act_bwd(da, s["z_e1a"]))
        da = dcat0[..., 64:] + pool_bwd(dp1)
        da = layer("enc0b", s["a_e0a"], act_bwd(da, s["z_e0b"]))
        layer("enc0a", s["x0"], act_bwd(da, s["z_e0a"]), need_dx=False)
        return g
