"""Learned warm-start of the track maps: a convolutional U-Net that predicts
converged log-discharge and momentum maps from a heightmap.

The reference has no counterpart.  Its discharge and momentum maps start at
zero and fill through World::erode's lrate blend (source/world.h:83-85), so
a fresh terrain needs tens of cycles before they settle.  The surrogate
predicts the settled maps from the heightmap.  `warm_start(world)` writes
them into a World, and plain particle cycles continue from there; the
particle method stays the judge of the result.

Network: 4 levels, channels 32-64-128-256, 3x3 convolutions with GELU, 2x2
average pooling down, nearest 2x upsampling up with the encoder's output
concatenated, and a 1x1 head.  1.36 M parameters.

    level 0 (H x W)    enc0a 16->32, enc0b 32->32       dec0a 96->32, dec0b 32->32, head 32->16 (1x1)
    level 1 (H/2)      enc1a 32->64, enc1b 64->64       dec1a 192->64, dec1b 64->64
    level 2 (H/4)      enc2a 64->128, enc2b 128->128    dec2a 384->128, dec2b 128->128
    level 3 (H/8)      mid 128->256

Input: 16 channels (normalised height, its central differences, 13 zeros).
Output: head channels 0-2, the normalised log1p(discharge), momentum x and
momentum y; channels 3-15 pad the head to the tensor cores' minimum N.

Every convolution, forward and backward, runs on the library's BF16
tensor-core kernels (include/shy_surrogate.h) with FP32 accumulation.
Weights are kept in FP32 and trained with AdamW.  Activations are NHWC
bf16; each convolution's pre-activation is kept in f32 for the backward
pass.  The network is fully convolutional, so a 1024 x 1024 map runs in one
pass, with no tiling.  torch supplies device memory and the stream only.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from ._capi import SgAdamw, SgConvDesc, SgNorm, check, lib

IN_CH = 16
OUT_CH = 16
# (name, cin, cout, ksize) in forward order
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
CHANNELS = (32, 64, 128, 256)
ACT_NONE, ACT_GELU = 0, 1
LEVEL = {"enc0a": 0, "enc0b": 0, "enc1a": 1, "enc1b": 1, "enc2a": 2, "enc2b": 2, "mid": 3,
         "dec2a": 2, "dec2b": 2, "dec1a": 1, "dec1b": 1, "dec0a": 0, "dec0b": 0, "head": 0}
# TMA pipeline candidates the autotuner times: (pixels per tile, stages,
# taps per stage) for forward and input-gradient convolutions (taps per
# stage 3 applies to 3x3 kernels), (pixels per stage, stages) for weight
# gradients
CONV_TILES = tuple((px, st, rows) for rows in (1, 3) for px in (128, 256, 512) for st in (2, 3))
WGRAD_TILES = ((64, 2), (64, 3), (128, 2), (128, 3))


def _torch():
    import torch
    return torch


def param_count():
    return sum(k * k * ci * co + co for _, ci, co, k in LAYERS)


def flops_per_pixel(training: bool):
    """2 x multiply-adds of the convolutions per level-0 pixel; a training
    step adds the input-gradient (all but the first layer) and
    weight-gradient convolutions."""
    level = {"enc0": 0, "dec0": 0, "head": 0, "enc1": 1, "dec1": 1, "enc2": 2, "dec2": 2, "mid": 3}
    f = 0.0
    for name, ci, co, k in LAYERS:
        macs = k * k * ci * co / 4 ** level[name[:4] if name != "mid" else "mid"]
        f += 2 * macs * ((3 if name != "enc0a" else 2) if training else 1)
    return f


class Norm:
    """Input and output scaling (shy_sg_norm)."""

    def __init__(self, height_mean=0.5, height_scale=4.0, slope_scale=100.0,
                 out_mean=(0.0, 0.0, 0.0), out_scale=(1.0, 1.0, 1.0)):
        self.height_mean, self.height_scale, self.slope_scale = height_mean, height_scale, slope_scale
        self.out_mean, self.out_scale = tuple(out_mean), tuple(out_scale)

    @classmethod
    def fit(cls, heights, discharge, momx, momy):
        """Scaling from training data: standardise the height, unit-scale the
        slope channels and each output channel."""
        h = np.asarray(heights, np.float64)
        g = np.abs(np.diff(h, axis=-1)).mean() + 1e-12
        ld = np.log1p(np.asarray(discharge, np.float64))
        mx, my = np.asarray(momx, np.float64), np.asarray(momy, np.float64)
        return cls(float(h.mean()), float(1.0 / (h.std() + 1e-12)), float(1.0 / g),
                   (float(ld.mean()), float(mx.mean()), float(my.mean())),
                   (float(ld.std() + 1e-12), float(mx.std() + 1e-12), float(my.std() + 1e-12)))

    def c(self):
        n = SgNorm()
        n.height_mean, n.height_scale, n.slope_scale = self.height_mean, self.height_scale, self.slope_scale
        for i in range(3):
            n.out_mean[i] = self.out_mean[i]
            n.out_scale[i] = self.out_scale[i]
        return n

    def as_dict(self):
        return {"height_mean": self.height_mean, "height_scale": self.height_scale,
                "slope_scale": self.slope_scale, "out_mean": list(self.out_mean),
                "out_scale": list(self.out_scale)}

    def targets(self, discharge, momx, momy):
        """Normalised training targets [..., 3] (float32)."""
        t = np.stack([np.log1p(np.asarray(discharge, np.float64)), np.asarray(momx, np.float64),
                      np.asarray(momy, np.float64)], axis=-1)
        return ((t - np.asarray(self.out_mean)) / np.asarray(self.out_scale)).astype(np.float32)


class _Workspace:
    """Device buffers of one (batch, height, width) shape."""

    def __init__(self, torch, dev, B, H, W, training):
        bf, f32 = torch.bfloat16, torch.float32
        self.shape = (B, H, W)
        self.training = training
        P = [B * (H >> l) * (W >> l) for l in range(4)]
        self.P = P

        def t(n, c, dt):
            return torch.empty((n, c), dtype=dt, device=dev)

        c0, c1, c2, c3 = CHANNELS
        self.x0 = t(P[0], IN_CH, bf)
        # bf16 activations (kept for the weight gradients)
        self.a = {"enc0a": t(P[0], c0, bf), "enc1a": t(P[1], c1, bf), "enc2a": t(P[2], c2, bf),
                  "mid": t(P[3], c3, bf), "dec2a": t(P[2], c2, bf), "dec2b": t(P[2], c2, bf),
                  "dec1a": t(P[1], c1, bf), "dec1b": t(P[1], c1, bf), "dec0a": t(P[0], c0, bf),
                  "dec0b": t(P[0], c0, bf)}
        self.cat = [t(P[0], 3 * c0, bf), t(P[1], 3 * c1, bf), t(P[2], 3 * c2, bf)]
        self.pool = [None, t(P[1], c0, bf), t(P[2], c1, bf), t(P[3], c2, bf)]
        self.zh = t(P[0], OUT_CH, f32)
        if training:
            lvl = {"enc0a": 0, "enc0b": 0, "enc1a": 1, "enc1b": 1, "enc2a": 2, "enc2b": 2, "mid": 3,
                   "dec2a": 2, "dec2b": 2, "dec1a": 1, "dec1b": 1, "dec0a": 0, "dec0b": 0}
            self.z = {n: t(P[lvl[n]], co, f32) for n, _, co, _ in LAYERS if n != "head"}
            self.da = [t(P[l], CHANNELS[l], f32) for l in range(4)]
            self.dz = [t(P[l], CHANNELS[l], bf) for l in range(4)]
            self.dcat = [t(P[l], 3 * CHANNELS[l], f32) for l in range(3)]
            self.dpool = [None, t(P[1], c0, f32), t(P[2], c1, f32), t(P[3], c2, f32)]
            self.dzh = t(P[0], OUT_CH, bf)
            self.target = t(P[0], 3, f32)
            self.loss = torch.zeros(1, dtype=torch.float64, device=dev)
        else:
            self.z = {}


class Surrogate:
    """The U-Net with FP32 master weights, bf16 working copies and AdamW
    state, on one CUDA device."""

    def __init__(self, seed: int = 0, device: int = 0, norm: Norm | None = None, init=None):
        torch = _torch()
        self.torch = torch
        self.dev = torch.device("cuda", device)
        self.norm = norm or Norm()
        self.layers = {}
        off = 0
        for name, ci, co, k in LAYERS:
            nw = co * k * k * ci
            self.layers[name] = dict(cin=ci, cout=co, k=k, w=off, b=off + nw, nw=nw)
            off += nw + co
        self.nparams = off
        host = np.zeros(off, np.float32)
        rng = np.random.default_rng(seed)
        for name, ci, co, k in LAYERS:
            L = self.layers[name]
            if init is not None:
                w, b = init[name]
            else:
                std = math.sqrt((1.0 if name == "head" else 2.0) / (k * k * ci))
                w, b = rng.standard_normal((co, k * k, ci)) * std, np.zeros(co)
            host[L["w"]:L["w"] + L["nw"]] = np.asarray(w, np.float32).ravel()
            host[L["b"]:L["b"] + co] = np.asarray(b, np.float32)
        self.params = torch.from_numpy(host).to(self.dev)
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.t = 0
        for name, L in self.layers.items():
            L["wb"] = torch.empty(L["nw"], dtype=torch.bfloat16, device=self.dev)
            L["wf"] = torch.empty(L["nw"], dtype=torch.bfloat16, device=self.dev)
        self._ws = {}
        self._prepped = False
        self.launches = 0
        self.tune = {}  # (layer, "fwd" | "dgrad" | "wgrad") -> a CONV_TILES or WGRAD_TILES entry

    # -- plumbing ---------------------------------------------------------
    def _stream(self):
        return C.c_void_p(self.torch.cuda.current_stream(self.dev).cuda_stream)

    @staticmethod
    def _p(t, off=0):
        return C.c_void_p(t.data_ptr() + off * t.element_size()) if t is not None else None

    def _call(self, fn, *args):
        check(getattr(lib(), fn)(*args, self._stream()))
        self.launches += 1

    def workspace(self, B, H, W, training):
        if H % 8 or W % 8:
            raise ValueError("map sides must be multiples of 8")
        key = (B, H, W, training)
        ws = self._ws.get(key)
        if ws is None:
            ws = _Workspace(self.torch, self.dev, B, H, W, training)
            self._ws[key] = ws
        return ws

    def prep_weights(self):
        for name, L in self.layers.items():
            self._call("shy_sg_weight_prep", L["cout"], L["k"], L["cin"], self._p(self.params, L["w"]),
                       self._p(L["wb"]), self._p(L["wf"]))
        self._prepped = True

    def _desc(self, ws, name, kind):
        """Convolution descriptor of one layer's forward ("fwd"), input
        gradient ("dgrad", channels swapped) or weight gradient ("wgrad"),
        with the autotuned tile if there is one."""
        L = self.layers[name]
        B, H, W = ws.shape
        lv = LEVEL[name]
        ci, co = (L["cout"], L["cin"]) if kind == "dgrad" else (L["cin"], L["cout"])
        tile, stages, rows = (tuple(self.tune.get((name, kind), ())) + (0, 0, 0))[:3]
        return SgConvDesc(B, H >> lv, W >> lv, ci, co, L["k"], tile, stages, rows)

    def _conv(self, ws, name, x, xs, z, zs, zo, a, as_, ao, act):
        L = self.layers[name]
        d = self._desc(ws, name, "fwd")
        self._call("shy_sg_conv_forward", C.byref(d), self._p(x), xs, self._p(L["wb"]),
                   self._p(self.params, L["b"]), self._p(z), zs, zo, self._p(a), as_, ao, act)

    # -- forward ------------------------------------------------------------
    def features(self, ws, heights):
        B, H, W = ws.shape
        n = self.norm.c()
        self._call("shy_sg_features", B, H, W, self._p(heights), C.byref(n), self._p(ws.x0))

    def forward(self, ws):
        """Forward pass from ws.x0 to ws.zh (f32, 16 channels)."""
        if not self._prepped:
            self.prep_weights()
        B, H, W = ws.shape
        c0, c1, c2, c3 = CHANNELS
        z = ws.z.get
        G = ACT_GELU
        self._conv(ws, "enc0a", ws.x0, IN_CH, z("enc0a"), c0, 0, ws.a["enc0a"], c0, 0, G)
        self._conv(ws, "enc0b", ws.a["enc0a"], c0, z("enc0b"), c0, 0, ws.cat[0], 3 * c0, 2 * c0, G)
        self._call("shy_sg_pool_forward", B, H, W, c0, self._p(ws.cat[0]), 3 * c0, 2 * c0,
                   self._p(ws.pool[1]), c0, 0)
        self._conv(ws, "enc1a", ws.pool[1], c0, z("enc1a"), c1, 0, ws.a["enc1a"], c1, 0, G)
        self._conv(ws, "enc1b", ws.a["enc1a"], c1, z("enc1b"), c1, 0, ws.cat[1], 3 * c1, 2 * c1, G)
        self._call("shy_sg_pool_forward", B, H >> 1, W >> 1, c1, self._p(ws.cat[1]), 3 * c1, 2 * c1,
                   self._p(ws.pool[2]), c1, 0)
        self._conv(ws, "enc2a", ws.pool[2], c1, z("enc2a"), c2, 0, ws.a["enc2a"], c2, 0, G)
        self._conv(ws, "enc2b", ws.a["enc2a"], c2, z("enc2b"), c2, 0, ws.cat[2], 3 * c2, 2 * c2, G)
        self._call("shy_sg_pool_forward", B, H >> 2, W >> 2, c2, self._p(ws.cat[2]), 3 * c2, 2 * c2,
                   self._p(ws.pool[3]), c2, 0)
        self._conv(ws, "mid", ws.pool[3], c2, z("mid"), c3, 0, ws.a["mid"], c3, 0, G)
        self._call("shy_sg_upsample_forward", B, H >> 3, W >> 3, c3, self._p(ws.a["mid"]), c3, 0,
                   self._p(ws.cat[2]), 3 * c2, 0)
        self._conv(ws, "dec2a", ws.cat[2], 3 * c2, z("dec2a"), c2, 0, ws.a["dec2a"], c2, 0, G)
        self._conv(ws, "dec2b", ws.a["dec2a"], c2, z("dec2b"), c2, 0, ws.a["dec2b"], c2, 0, G)
        self._call("shy_sg_upsample_forward", B, H >> 2, W >> 2, c2, self._p(ws.a["dec2b"]), c2, 0,
                   self._p(ws.cat[1]), 3 * c1, 0)
        self._conv(ws, "dec1a", ws.cat[1], 3 * c1, z("dec1a"), c1, 0, ws.a["dec1a"], c1, 0, G)
        self._conv(ws, "dec1b", ws.a["dec1a"], c1, z("dec1b"), c1, 0, ws.a["dec1b"], c1, 0, G)
        self._call("shy_sg_upsample_forward", B, H >> 1, W >> 1, c1, self._p(ws.a["dec1b"]), c1, 0,
                   self._p(ws.cat[0]), 3 * c0, 0)
        self._conv(ws, "dec0a", ws.cat[0], 3 * c0, z("dec0a"), c0, 0, ws.a["dec0a"], c0, 0, G)
        self._conv(ws, "dec0b", ws.a["dec0a"], c0, z("dec0b"), c0, 0, ws.a["dec0b"], c0, 0, G)
        self._conv(ws, "head", ws.a["dec0b"], c0, ws.zh, OUT_CH, 0, None, 0, 0, ACT_NONE)

    # -- backward -----------------------------------------------------------
    def _layer_bwd(self, ws, name, x_in, xs, dz, dx, dxs, bias=False):
        """Weight gradient of one convolution from its output gradient dz
        (bf16, contiguous), and its bias gradient if `bias` (the GELU
        backward that made dz adds it otherwise); its input gradient into dx
        (f32, pixel stride dxs) unless dx is None."""
        L = self.layers[name]
        d = self._desc(ws, name, "wgrad")
        self._call("shy_sg_conv_wgrad", C.byref(d), self._p(x_in), xs, self._p(dz), L["cout"],
                   self._p(self.grads, L["w"]))
        if bias:
            self._call("shy_sg_bias_grad", d.batch * d.height * d.width, L["cout"], self._p(dz), L["cout"],
                       self._p(self.grads, L["b"]))
        if dx is not None:
            dd = self._desc(ws, name, "dgrad")
            self._call("shy_sg_conv_forward", C.byref(dd), self._p(dz), L["cout"], self._p(L["wf"]), None,
                       self._p(dx), dxs, 0, None, 0, 0, ACT_NONE)

    def _gelu_bwd(self, ws, level, c, da, das, dao, name):
        """Output gradient of layer `name` (bf16 into ws.dz[level]) and its
        bias gradient."""
        self._call("shy_sg_gelu_backward", ws.P[level], c, self._p(da), das, dao, self._p(ws.z[name]), c, 0,
                   self._p(ws.dz[level]), self._p(self.grads, self.layers[name]["b"]))

    def backward(self, ws):
        """Gradients of the loss (ws.dzh holds its output gradient) into
        self.grads, which must be zero on entry."""
        B, H, W = ws.shape
        c0, c1, c2, c3 = CHANNELS
        da, dz, dcat, dp = ws.da, ws.dz, ws.dcat, ws.dpool
        self._layer_bwd(ws, "head", ws.a["dec0b"], c0, ws.dzh, da[0], c0, bias=True)
        self._gelu_bwd(ws, 0, c0, da[0], c0, 0, "dec0b")
        self._layer_bwd(ws, "dec0b", ws.a["dec0a"], c0, dz[0], da[0], c0)
        self._gelu_bwd(ws, 0, c0, da[0], c0, 0, "dec0a")
        self._layer_bwd(ws, "dec0a", ws.cat[0], 3 * c0, dz[0], dcat[0], 3 * c0)
        da[1].zero_()
        self._call("shy_sg_upsample_backward", B, H >> 1, W >> 1, c1, self._p(dcat[0]), 3 * c0, 0,
                   self._p(da[1]), c1, 0)
        self._gelu_bwd(ws, 1, c1, da[1], c1, 0, "dec1b")
        self._layer_bwd(ws, "dec1b", ws.a["dec1a"], c1, dz[1], da[1], c1)
        self._gelu_bwd(ws, 1, c1, da[1], c1, 0, "dec1a")
        self._layer_bwd(ws, "dec1a", ws.cat[1], 3 * c1, dz[1], dcat[1], 3 * c1)
        da[2].zero_()
        self._call("shy_sg_upsample_backward", B, H >> 2, W >> 2, c2, self._p(dcat[1]), 3 * c1, 0,
                   self._p(da[2]), c2, 0)
        self._gelu_bwd(ws, 2, c2, da[2], c2, 0, "dec2b")
        self._layer_bwd(ws, "dec2b", ws.a["dec2a"], c2, dz[2], da[2], c2)
        self._gelu_bwd(ws, 2, c2, da[2], c2, 0, "dec2a")
        self._layer_bwd(ws, "dec2a", ws.cat[2], 3 * c2, dz[2], dcat[2], 3 * c2)
        da[3].zero_()
        self._call("shy_sg_upsample_backward", B, H >> 3, W >> 3, c3, self._p(dcat[2]), 3 * c2, 0,
                   self._p(da[3]), c3, 0)
        self._gelu_bwd(ws, 3, c3, da[3], c3, 0, "mid")
        self._layer_bwd(ws, "mid", ws.pool[3], c2, dz[3], dp[3], c2)
        # level 2 encoder: skip gradient from dec2a plus the pooled path
        self._call("shy_sg_pool_backward", B, H >> 2, W >> 2, c2, self._p(dp[3]), c2, 0, self._p(dcat[2]),
                   3 * c2, 2 * c2)
        self._gelu_bwd(ws, 2, c2, dcat[2], 3 * c2, 2 * c2, "enc2b")
        self._layer_bwd(ws, "enc2b", ws.a["enc2a"], c2, dz[2], da[2], c2)
        self._gelu_bwd(ws, 2, c2, da[2], c2, 0, "enc2a")
        self._layer_bwd(ws, "enc2a", ws.pool[2], c1, dz[2], dp[2], c1)
        self._call("shy_sg_pool_backward", B, H >> 1, W >> 1, c1, self._p(dp[2]), c1, 0, self._p(dcat[1]),
                   3 * c1, 2 * c1)
        self._gelu_bwd(ws, 1, c1, dcat[1], 3 * c1, 2 * c1, "enc1b")
        self._layer_bwd(ws, "enc1b", ws.a["enc1a"], c1, dz[1], da[1], c1)
        self._gelu_bwd(ws, 1, c1, da[1], c1, 0, "enc1a")
        self._layer_bwd(ws, "enc1a", ws.pool[1], c0, dz[1], dp[1], c0)
        self._call("shy_sg_pool_backward", B, H, W, c0, self._p(dp[1]), c0, 0, self._p(dcat[0]), 3 * c0,
                   2 * c0)
        self._gelu_bwd(ws, 0, c0, dcat[0], 3 * c0, 2 * c0, "enc0b")
        self._layer_bwd(ws, "enc0b", ws.a["enc0a"], c0, dz[0], da[0], c0)
        self._gelu_bwd(ws, 0, c0, da[0], c0, 0, "enc0a")
        self._layer_bwd(ws, "enc0a", ws.x0, IN_CH, dz[0], None, 0)

    # -- autotuning ---------------------------------------------------------
    def _layer_inputs(self, ws):
        """Each convolution's input tensor in the workspace and its pixel stride."""
        c0, c1, c2, c3 = CHANNELS
        return {"enc0a": (ws.x0, IN_CH), "enc0b": (ws.a["enc0a"], c0), "enc1a": (ws.pool[1], c0),
                "enc1b": (ws.a["enc1a"], c1), "enc2a": (ws.pool[2], c1), "enc2b": (ws.a["enc2a"], c2),
                "mid": (ws.pool[3], c2), "dec2a": (ws.cat[2], 3 * c2), "dec2b": (ws.a["dec2a"], c2),
                "dec1a": (ws.cat[1], 3 * c1), "dec1b": (ws.a["dec1a"], c1), "dec0a": (ws.cat[0], 3 * c0),
                "dec0b": (ws.a["dec0a"], c0), "head": (ws.a["dec0b"], c0)}

    def autotune(self, B, H, W, reps=5):
        """Time every TMA tile candidate for each layer's forward, input- and
        weight-gradient convolution at this batch shape (CUDA events, scratch
        outputs) and keep the fastest for later calls.  Returns
        {(layer, kind): (candidate, ms)}."""
        torch = self.torch
        if not self._prepped:
            self.prep_weights()
        ws = self.workspace(B, H, W, True)
        ins = self._layer_inputs(ws)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        stream = torch.cuda.current_stream(self.dev)
        out = {}
        for name, ci, co, k in LAYERS:
            P = ws.P[LEVEL[name]]
            L = self.layers[name]
            x, xs = ins[name]
            dz = torch.zeros((P, co), dtype=torch.bfloat16, device=self.dev)
            zf = torch.empty((P, max(ci, co)), dtype=torch.float32, device=self.dev)
            gw = torch.zeros(L["nw"], dtype=torch.float32, device=self.dev)
            kinds = ("fwd", "wgrad") if name == "enc0a" else ("fwd", "dgrad", "wgrad")
            for kind in kinds:
                best = None
                cands = WGRAD_TILES if kind == "wgrad" else [c for c in CONV_TILES if k == 3 or c[2] == 1]
                for cand in cands:
                    self.tune[(name, kind)] = cand
                    d = self._desc(ws, name, kind)
                    if kind == "fwd":
                        fn = lambda: self._call("shy_sg_conv_forward", C.byref(d), self._p(x), xs,  # noqa: E731
                                                self._p(L["wb"]), None, self._p(zf), co, 0, None, 0, 0, ACT_NONE)
                    elif kind == "dgrad":
                        fn = lambda: self._call("shy_sg_conv_forward", C.byref(d), self._p(dz), co,  # noqa: E731
                                                self._p(L["wf"]), None, self._p(zf), ci, 0, None, 0, 0, ACT_NONE)
                    else:
                        fn = lambda: self._call("shy_sg_conv_wgrad", C.byref(d), self._p(x), xs,  # noqa: E731
                                                self._p(dz), co, self._p(gw))
                    fn()
                    ev[0].record(stream)
                    for _ in range(reps):
                        fn()
                    ev[1].record(stream)
                    ev[1].synchronize()
                    ms = ev[0].elapsed_time(ev[1]) / reps
                    if best is None or ms < best[1]:
                        best = (cand, ms)
                self.tune[(name, kind)] = best[0]
                out[(name, kind)] = best
        self.status()
        return out

    # -- training -----------------------------------------------------------
    def loss_and_grads(self, ws, weights=(1.0, 1.0, 1.0)):
        """Forward, loss against ws.target, backward; gradients in self.grads."""
        self.forward(ws)
        ws.loss.zero_()
        w = (C.c_float * 3)(*weights)
        self._call("shy_sg_loss", ws.P[0], self._p(ws.zh), OUT_CH, self._p(ws.target), w, self._p(ws.dzh),
                   self._p(ws.loss))
        self.grads.zero_()
        self.backward(ws)

    def adamw_step(self, lr, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=1e-4):
        self.t += 1
        a = SgAdamw(lr, beta1, beta2, eps, weight_decay, 1.0 - beta1 ** self.t, 1.0 - beta2 ** self.t)
        self._call("shy_sg_adamw", self.nparams, self._p(self.params), self._p(self.grads), self._p(self.m),
                   self._p(self.v), C.byref(a))
        self.prep_weights()

    def train_step(self, heights, targets, lr, weights=(1.0, 1.0, 1.0)):
        """One AdamW step on a batch: heights (B, H, W) and normalised
        targets (B, H, W, 3), device float32 tensors.  Returns the loss as a
        device tensor (read it when convenient)."""
        B, H, W = heights.shape
        ws = self.workspace(B, H, W, True)
        self.features(ws, heights)
        ws.target.view(B, H, W, 3).copy_(targets)
        self.loss_and_grads(ws, weights)
        self.adamw_step(lr)
        return ws.loss

    # -- inference ----------------------------------------------------------
    def predict(self, heights):
        """Maps from heightmaps (B, H, W) device float32: returns device
        tensors (discharge, momentum x, momentum y), each (B, H, W)."""
        torch = self.torch
        B, H, W = heights.shape
        ws = self.workspace(B, H, W, False)
        self.features(ws, heights)
        self.forward(ws)
        out = [torch.empty((B, H, W), dtype=torch.float32, device=self.dev) for _ in range(3)]
        n = self.norm.c()
        self._call("shy_sg_decode", ws.P[0], self._p(ws.zh), OUT_CH, C.byref(n), self._p(out[0]),
                   self._p(out[1]), self._p(out[2]))
        return tuple(out)

    def warm_start(self, world, terrain: int = 0, scale: float = 1.0):
        """Write the predicted discharge and momentum maps of a terrain into a
        World or Batch (its current heightmap is the input), times `scale`.
        The plain method's maps after k cycles from zero are about
        (1 - (1 - lrate)^k) of their settled values (the lrate blend,
        source/world.h:83-85), so a scale below 1 starts the world where a
        plain run stands after that many cycles.  Device to device: the
        heights come out and the maps go in through
        shy_terrain_get/set_state_device, never through host memory."""
        torch = self.torch
        h = world.get_state_device(terrain)["height"]
        d, mx, my = self.predict(h[None])
        if scale != 1.0:
            d, mx, my = d * scale, mx * scale, my * scale
        torch.cuda.current_stream(self.dev).synchronize()
        world.set_state_device(terrain, discharge=d[0].contiguous(), momentum_x=mx[0].contiguous(),
                               momentum_y=my[0].contiguous())

    def warm_start_judged(self, world, drops: int, probe_cycles: int = 5, threshold: float = 0.05,
                          terrain: int = 0):
        """Warm start with the plain particle method as judge and fallback.

        The world's state (heights, maps, spawn-stream cycle) is kept on the
        device; the prediction is written into the world and `probe_cycles`
        plain cycles of `drops` drops run from it.  The judge is the log-L2
        distance between the mean discharge of those cycles and the
        prediction: the particle method, started from a right prediction,
        keeps it.  At or below `threshold` the warm start is kept and the
        world continues from the probe's end.  Above it the warm start is
        discarded: the kept state is restored and the same cycles run plain,
        so the world ends where it would have without the surrogate (bit for
        bit when its fixed-point heights were last derived from its float
        heights, as after set_field or generate: the restore goes through
        the float heights).  Returns {"accepted", "log_l2", "probe_cycles"}.
        A single-terrain World only (the probe runs shy_erode)."""
        torch = self.torch
        saved = world.get_state_device(terrain)
        cycle = world.cycle()
        d, mx, my = self.predict(saved["height"][None])
        torch.cuda.current_stream(self.dev).synchronize()
        pred = d[0].clone()
        world.set_state_device(terrain, discharge=d[0], momentum_x=mx[0], momentum_y=my[0])
        acc = torch.zeros_like(pred)
        probe = {"discharge": torch.empty_like(pred)}
        for _ in range(probe_cycles):
            world.erode(drops, 1)
            world.get_state_device(terrain, out=probe)
            acc += probe["discharge"]
        acc /= max(1, probe_cycles)
        a, b = torch.log1p(acc.double()), torch.log1p(pred.double())
        nb = float(torch.linalg.vector_norm(b))
        dist = float(torch.linalg.vector_norm(a - b)) / nb if nb > 0 else float("inf")
        accepted = dist <= threshold
        if not accepted:  # the fallback: the plain method from the kept state
            world.set_state_device(terrain, **saved)
            world.set_cycle(cycle)
            world.erode(drops, probe_cycles)
        return {"accepted": accepted, "log_l2": dist, "probe_cycles": probe_cycles}

    def status(self):
        check(lib().shy_sg_status())

    # -- state --------------------------------------------------------------
    def state_dict(self):
        return {"params": self.params.cpu().numpy(), "norm": self.norm.as_dict(), "t": self.t}

    def load_state_dict(self, s):
        self.params.copy_(self.torch.from_numpy(np.asarray(s["params"], np.float32)))
        n = s["norm"]
        self.norm = Norm(n["height_mean"], n["height_scale"], n["slope_scale"], n["out_mean"], n["out_scale"])
        self._prepped = False

    def weights_of(self, name):
        """(w[cout][tap][cin], b[cout]) of one layer as numpy float32."""
        L = self.layers[name]
        p = self.params.cpu().numpy()
        w = p[L["w"]:L["w"] + L["nw"]].reshape(L["cout"], L["k"] ** 2, L["cin"])
        return w, p[L["b"]:L["b"] + L["cout"]]

    def grads_of(self, name):
        L = self.layers[name]
        g = self.grads.cpu().numpy()
        return (g[L["w"]:L["w"] + L["nw"]].reshape(L["cout"], L["k"] ** 2, L["cin"]),
                g[L["b"]:L["b"] + L["cout"]])


SPAWN_STRIDE = 7919  # spawn seed of run r of a terrain: its seed + SPAWN_STRIDE * r


def make_pairs(n, size=256, drops=None, cycles=50, seed0=10000, per_launch=64, params=None, spawn_runs=1):
    """Training pairs from the batched GPU particle method.  Terrain i is
    the value-noise heightmap of seed seed0 + i.  Its input is the heightmap
    before erosion.  Its targets are the discharge and momentum maps after
    `cycles` plain cycles from zero maps, at `drops` drops per cycle (by
    default size^2 / 16, the density of 65,536 drops on 1024 x 1024),
    averaged over `spawn_runs` runs whose spawns differ (spawn seeds
    seed0 + i + SPAWN_STRIDE * r): a target that depends on the terrain, not
    on one run's spawn order.  Terrains run `per_launch` at a time (times
    the runs) in one Batch.  Returns float32 arrays (heights, discharge,
    momentum x, momentum y), each (n, size, size)."""
    from . import Batch
    drops = drops or max(1, size * size // 16)
    runs = max(1, int(spawn_runs))
    out = [np.empty((n, size, size), np.float32) for _ in range(4)]
    tmp = np.empty((size, size), np.float32)
    for s in range(0, n, per_launch):
        k = min(per_launch, n - s)
        seeds = [seed0 + s + i + SPAWN_STRIDE * r for r in range(runs) for i in range(k)]
        b = Batch([(size, size)] * (k * runs), [drops] * (k * runs), seeds, params)
        try:
            for r in range(runs):
                for i in range(k):
                    b.generate(r * k + i, seed0 + s + i, 8)
            for i in range(k):
                b.get_field(i, "height", out=out[0][s + i])
            b.erode(cycles)
            for j, f in enumerate(("discharge", "momentum_x", "momentum_y")):
                for i in range(k):
                    acc = np.zeros((size, size), np.float64)
                    for r in range(runs):
                        acc += b.get_field(r * k + i, f, out=tmp)
                    out[j + 1][s + i] = (acc / runs).astype(np.float32)
        finally:
            b.close()
    return tuple(out)


def train(net, heights, discharge, momx, momy, epochs, batch=16, lr=2e-3, seed=0, augment=True, crop=None,
          steps_per_epoch=None):
    """AdamW over the pairs with a cosine learning-rate schedule.  With
    `augment`, each batch is flipped along either axis at random (discharge
    is unchanged and the momentum component along a flipped axis changes
    sign; a world's x-major map is an image with rows = x).  With `crop`,
    each sample is a random crop x crop window of its map (offsets multiples
    of 8), and an epoch is `steps_per_epoch` batches.  Returns the mean loss
    of each epoch."""
    torch = net.torch
    H = torch.from_numpy(np.ascontiguousarray(heights, np.float32)).to(net.dev)
    T = torch.from_numpy(net.norm.targets(discharge, momx, momy)).to(net.dev)
    sign = torch.tensor(net.norm.out_mean, dtype=torch.float32, device=net.dev)
    scale = torch.tensor(net.norm.out_scale, dtype=torch.float32, device=net.dev)
    n, side = H.shape[0], H.shape[-1]
    per_epoch = steps_per_epoch or max(1, n // batch)
    total = epochs * per_epoch
    rng = np.random.default_rng(seed)
    losses, step = [], 0
    for _ in range(epochs):
        # one upload per epoch: a per-step host-to-device copy would make the
        # host wait for the device every step
        order = np.concatenate([rng.permutation(n) for _ in range((per_epoch * batch + n - 1) // n)])
        perm = torch.from_numpy(order).to(net.dev)
        acc = torch.zeros(1, dtype=torch.float64, device=net.dev)
        for j in range(per_epoch):
            idx = perm[j * batch:(j + 1) * batch]
            if crop and crop < side:
                offs = rng.integers(0, (side - crop) // 8 + 1, size=(batch, 2)) * 8
                h = torch.stack([H[int(order[j * batch + i])][oy:oy + crop, ox:ox + crop]
                                 for i, (oy, ox) in enumerate(offs)])
                t = torch.stack([T[int(order[j * batch + i])][oy:oy + crop, ox:ox + crop]
                                 for i, (oy, ox) in enumerate(offs)])
            else:
                h, t = H[idx], T[idx]
            if augment:
                for axis, comp in ((1, 1), (2, 2)):
                    if rng.random() < 0.5:
                        h, t = h.flip(axis), t.flip(axis)
                        # momentum along the flipped axis: raw -> -raw in normalised units
                        t[..., comp] = -t[..., comp] - 2.0 * sign[comp] / scale[comp]
                h, t = h.contiguous(), t.contiguous()
            lr_t = lr * 0.5 * (1.0 + math.cos(math.pi * step / total))
            acc += net.train_step(h, t, lr_t)
            step += 1
        losses.append(float(acc.item()) / per_epoch)
    return losses


def log_l2(d, ref):
    """||log1p(d) - log1p(ref)|| / ||log1p(ref)||, the discharge distance."""
    a = np.log1p(np.asarray(d, np.float64))
    b = np.log1p(np.asarray(ref, np.float64))
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


__all__ = ["Surrogate", "Norm", "LAYERS", "param_count", "flops_per_pixel", "make_pairs", "train", "log_l2",
           "SPAWN_STRIDE"]
