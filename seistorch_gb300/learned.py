"""Learned gradient preconditioner: a 4-level convolutional network that maps
the raw FWI gradient and the source illumination to a model update.

There is no counterpart in the reference, which preconditions the gradient
by the illumination only (process.py:115-118, rnn.py:127-128); that plain
illumination-compensated gradient stays the fallback of the FWI loop
(``seistorch_gb300.fwi``).

Network (about 1.16 M parameters, bf16 weights and activations, fp32
accumulation and master weights), input 2 x H x W (H, W multiples of 8,
W >= 512):

    level 1 (H x W)      : in 2->32 (SIMT), e1b 32->32            skip1 (32)
    level 2 (H/2 x W/2)  : pool, e2a 32->64, e2b 64->64           skip2 (64)
    level 3 (H/4 x W/4)  : pool, e3a 64->128, e3b 128->128        skip3 (128)
    level 4 (H/8 x W/8)  : pool, b4 128->256
    decoder              : up, [b4 | skip3] 384->128 (d3), up, [d3 | skip2]
                           192->64 (d2), up, [d2 | skip1] 96->32 (d1),
                           out 32->1 (SIMT, linear)

All 3x3 convolutions except the first and last run on the tcgen05 tensor
cores (``sgb_nn_conv3x3``: forward and data gradient;
``sgb_nn_conv3x3_wgrad``: weight gradient); ReLU after every hidden layer;
2x2 average pooling, nearest upsampling, skip concatenation by writing into
channel slices.  Adam on fp32 master weights; the bf16 copies are repacked
after every step.
"""
import ctypes
import math

import numpy as np
import torch

from . import _native as N

# name, cin, cout, kind ("in": SIMT 2-channel input, "tc": tensor cores, "out": SIMT 1-channel output)
LAYERS = [("e1a", 2, 32, "in"), ("e1b", 32, 32, "tc"), ("e2a", 32, 64, "tc"), ("e2b", 64, 64, "tc"),
          ("e3a", 64, 128, "tc"), ("e3b", 128, 128, "tc"), ("b4", 128, 256, "tc"), ("d3", 384, 128, "tc"),
          ("d2", 192, 64, "tc"), ("d1", 96, 32, "tc"), ("out", 32, 1, "out")]
BF16 = torch.bfloat16


def n_params():
    return sum(ci * co * 9 + co for _, ci, co, _ in LAYERS)


class PrecondNet:
    """The network's parameters, optimiser state and activation buffers on
    one GPU, driven through the C ABI on the current torch stream."""

    def __init__(self, device=None, seed=0):
        self.device = torch.device(device or "cuda")
        N.load()
        total = n_params()
        self.params = torch.zeros(total, dtype=torch.float32, device=self.device)
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step_count = 0
        self.W, self.b, self.gW, self.gb = {}, {}, {}, {}
        self.wt, self.wflip = {}, {}
        rng = np.random.default_rng(seed)
        off = 0
        init = np.zeros(total, np.float32)
        for name, ci, co, kind in LAYERS:
            nw = ci * co * 9
            std = math.sqrt(2.0 / (ci * 9)) if kind != "out" else math.sqrt(1.0 / (ci * 9)) * 0.1
            init[off:off + nw] = rng.standard_normal(nw) * std
            self.W[name] = self.params[off:off + nw].view(co, ci, 3, 3)
            self.gW[name] = self.grads[off:off + nw].view(co, ci, 3, 3)
            off += nw
            self.b[name] = self.params[off:off + co]
            self.gb[name] = self.grads[off:off + co]
            off += co
            if kind == "tc":
                self.wt[name] = torch.empty(co, 9, ci, dtype=BF16, device=self.device)
                self.wflip[name] = torch.empty(ci, 9, co, dtype=BF16, device=self.device)
        self.params.copy_(torch.from_numpy(init).to(self.device))
        self._bufs = None
        self._shape = None
        self.pack()

    # -- parameters
    def pack(self):
        """Repack the bf16 weight copies from the fp32 master weights."""
        s = N.stream_handle()
        for name, ci, co, kind in LAYERS:
            if kind == "tc":
                N.call("sgb_nn_pack_weights", co, ci, N.ptr(self.W[name]), N.ptr(self.wt[name]),
                       N.ptr(self.wflip[name]), s)

    def state_dict(self):
        return {"params": self.params.detach().cpu().numpy().copy(), "step": self.step_count}

    def load_state_dict(self, sd):
        self.params.copy_(torch.as_tensor(sd["params"], device=self.device))
        self.step_count = int(sd.get("step", 0))
        self.pack()

    # -- buffers
    def _alloc(self, B, H, W):
        if self._shape == (B, H, W):
            return self._bufs
        if H % 8 or W % 8 or W < 512:
            raise ValueError("the network needs H, W multiples of 8 and W >= 512")
        d = self.device
        L = [(H, W), (H // 2, W // 2), (H // 4, W // 4), (H // 8, W // 8)]
        bf = lambda h, w, c: torch.zeros(B, h, w, c, dtype=BF16, device=d)
        f32 = lambda h, w, c: torch.zeros(B, h, w, c, dtype=torch.float32, device=d)
        (h1, w1), (h2, w2), (h3, w3), (h4, w4) = L
        b = dict(
            a1a=bf(h1, w1, 32), cat1=bf(h1, w1, 96), p1=bf(h2, w2, 32), a2a=bf(h2, w2, 64), cat2=bf(h2, w2, 192),
            p2=bf(h3, w3, 64), a3a=bf(h3, w3, 128), cat3=bf(h3, w3, 384), p3=bf(h4, w4, 128), a4=bf(h4, w4, 256),
            ad3=bf(h3, w3, 128), ad2=bf(h2, w2, 64), ad1=bf(h1, w1, 32),
            pred=torch.zeros(B, h1, w1, dtype=torch.float32, device=d),
            # backward
            g1=bf(h1, w1, 32), g1b=bf(h1, w1, 32), dcat1=f32(h1, w1, 96), g2=bf(h2, w2, 64), g2b=bf(h2, w2, 64),
            dcat2=f32(h2, w2, 192), g3=bf(h3, w3, 128), g3b=bf(h3, w3, 128), dcat3=f32(h3, w3, 384),
            g4=bf(h4, w4, 256), dp3=f32(h4, w4, 128), dp2=f32(h3, w3, 64), dp1=f32(h2, w2, 32),
            chw_dy=torch.zeros(B * h1 * w1 * 64, dtype=BF16, device=d),
            chw_x=torch.zeros(3 * B * h1 * w1 * 96, dtype=BF16, device=d),
            dpred=torch.zeros(B, h1, w1, dtype=torch.float32, device=d),
            loss=torch.zeros(1, dtype=torch.float32, device=d))
        self._bufs, self._shape, self._levels = b, (B, H, W), L
        return b

    # -- layers
    def _tc(self, name, x, h, w, out, cstride, coff, relu=True, bias=True):
        _, ci, co, _ = next(l for l in LAYERS if l[0] == name)
        B = self._shape[0]
        c = N.NnConv(B, h, w, ci, co, N.ptr(x), N.ptr(self.wt[name]), N.ptr(self.b[name]) if bias else None,
                     int(relu), None, 0, N.ptr(out), None, cstride, coff)
        N.call("sgb_nn_conv3x3", ctypes.byref(c), N.stream_handle())

    def _tc_dgrad(self, name, dy, h, w, out_f32=None, out_bf16=None, mask=None):
        _, ci, co, _ = next(l for l in LAYERS if l[0] == name)
        B = self._shape[0]
        c = N.NnConv(B, h, w, co, ci, N.ptr(dy), N.ptr(self.wflip[name]), None, 0, N.ptr(mask),
                     ci if mask is not None else 0, N.ptr(out_bf16), N.ptr(out_f32), ci, 0)
        N.call("sgb_nn_conv3x3", ctypes.byref(c), N.stream_handle())

    def _tc_wgrad(self, name, dy, x, h, w):
        _, ci, co, _ = next(l for l in LAYERS if l[0] == name)
        b = self._bufs
        B = self._shape[0]
        s = N.stream_handle()
        n_dy = B * co * h * w
        n_x = B * ci * h * w
        dy_chw = b["chw_dy"][:n_dy] if n_dy <= b["chw_dy"].numel() else torch.empty(n_dy, dtype=BF16,
                                                                                     device=self.device)
        x_chw = b["chw_x"][:3 * n_x] if 3 * n_x <= b["chw_x"].numel() else torch.empty(3 * n_x, dtype=BF16,
                                                                                        device=self.device)
        N.call("sgb_nn_to_chw", B, h, w, co, co, 0, N.ptr(dy), 1, N.ptr(dy_chw), s)
        N.call("sgb_nn_to_chw", B, h, w, ci, ci, 0, N.ptr(x), 3, N.ptr(x_chw), s)
        p = N.NnWgrad(B, h, w, ci, co, N.ptr(dy_chw),
                      N.PTR3(*[x_chw.data_ptr() + 2 * k * n_x for k in range(3)]), N.ptr(self.gW[name]))
        N.call("sgb_nn_conv3x3_wgrad", ctypes.byref(p), s)
        N.call("sgb_nn_bias_grad", B, h * w, co, N.ptr(dy_chw), N.ptr(self.gb[name]), s)

    # -- forward / backward
    def forward(self, x):
        """x: fp32 (B, 2, H, W) on the device -> prediction fp32 (B, H, W)."""
        B, C, H, W = x.shape
        if C != 2:
            raise ValueError("the network takes 2 input channels (gradient, illumination)")
        b = self._alloc(B, H, W)
        self._x = x.contiguous().to(torch.float32)
        (h1, w1), (h2, w2), (h3, w3), (h4, w4) = self._levels
        s = N.stream_handle()
        N.call("sgb_nn_conv_in", B, h1, w1, 32, N.ptr(self._x), N.ptr(self.W["e1a"]), N.ptr(self.b["e1a"]),
               N.ptr(b["a1a"]), 32, 0, s)
        self._tc("e1b", b["a1a"], h1, w1, b["cat1"], 96, 64)
        N.call("sgb_nn_pool2", B, h1, w1, 32, N.ptr(b["cat1"]), 96, 64, N.ptr(b["p1"]), s)
        self._tc("e2a", b["p1"], h2, w2, b["a2a"], 64, 0)
        self._tc("e2b", b["a2a"], h2, w2, b["cat2"], 192, 128)
        N.call("sgb_nn_pool2", B, h2, w2, 64, N.ptr(b["cat2"]), 192, 128, N.ptr(b["p2"]), s)
        self._tc("e3a", b["p2"], h3, w3, b["a3a"], 128, 0)
        self._tc("e3b", b["a3a"], h3, w3, b["cat3"], 384, 256)
        N.call("sgb_nn_pool2", B, h3, w3, 128, N.ptr(b["cat3"]), 384, 256, N.ptr(b["p3"]), s)
        self._tc("b4", b["p3"], h4, w4, b["a4"], 256, 0)
        N.call("sgb_nn_up2", B, h3, w3, 256, N.ptr(b["a4"]), N.ptr(b["cat3"]), 384, 0, s)
        self._tc("d3", b["cat3"], h3, w3, b["ad3"], 128, 0)
        N.call("sgb_nn_up2", B, h2, w2, 128, N.ptr(b["ad3"]), N.ptr(b["cat2"]), 192, 0, s)
        self._tc("d2", b["cat2"], h2, w2, b["ad2"], 64, 0)
        N.call("sgb_nn_up2", B, h1, w1, 64, N.ptr(b["ad2"]), N.ptr(b["cat1"]), 96, 0, s)
        self._tc("d1", b["cat1"], h1, w1, b["ad1"], 32, 0)
        N.call("sgb_nn_conv_out", B, h1, w1, 32, N.ptr(b["ad1"]), 32, N.ptr(self.W["out"]), N.ptr(self.b["out"]),
               N.ptr(b["pred"]), s)
        return b["pred"]

    def backward(self, dpred):
        """Accumulate parameter gradients of sum(pred * dpred) into self.grads."""
        b = self._bufs
        B = self._shape[0]
        (h1, w1), (h2, w2), (h3, w3), (h4, w4) = self._levels
        s = N.stream_handle()
        dpred = dpred.contiguous().to(torch.float32)
        N.call("sgb_nn_conv_out_bwd", B, h1, w1, 32, N.ptr(dpred), N.ptr(self.W["out"]), N.ptr(b["ad1"]), 32,
               N.ptr(b["g1"]), N.ptr(self.gW["out"]), N.ptr(self.gb["out"]), s)
        # decoder level 1
        self._tc_wgrad("d1", b["g1"], b["cat1"], h1, w1)
        self._tc_dgrad("d1", b["g1"], h1, w1, out_f32=b["dcat1"])
        N.call("sgb_nn_up2_bwd", B, h1, w1, 64, N.ptr(b["dcat1"]), 96, 0, N.ptr(b["ad2"]), N.ptr(b["g2"]), s)
        # decoder level 2
        self._tc_wgrad("d2", b["g2"], b["cat2"], h2, w2)
        self._tc_dgrad("d2", b["g2"], h2, w2, out_f32=b["dcat2"])
        N.call("sgb_nn_up2_bwd", B, h2, w2, 128, N.ptr(b["dcat2"]), 192, 0, N.ptr(b["ad3"]), N.ptr(b["g3"]), s)
        # decoder level 3
        self._tc_wgrad("d3", b["g3"], b["cat3"], h3, w3)
        self._tc_dgrad("d3", b["g3"], h3, w3, out_f32=b["dcat3"])
        N.call("sgb_nn_up2_bwd", B, h3, w3, 256, N.ptr(b["dcat3"]), 384, 0, N.ptr(b["a4"]), N.ptr(b["g4"]), s)
        # bottleneck
        self._tc_wgrad("b4", b["g4"], b["p3"], h4, w4)
        self._tc_dgrad("b4", b["g4"], h4, w4, out_f32=b["dp3"])
        N.call("sgb_nn_pool2_bwd", B, h3, w3, 128, N.ptr(b["dp3"]), N.ptr(b["dcat3"]), 384, 256, N.ptr(b["cat3"]),
               384, 256, N.ptr(b["g3b"]), s)
        # encoder level 3
        self._tc_wgrad("e3b", b["g3b"], b["a3a"], h3, w3)
        self._tc_dgrad("e3b", b["g3b"], h3, w3, out_bf16=b["g3"], mask=b["a3a"])
        self._tc_wgrad("e3a", b["g3"], b["p2"], h3, w3)
        self._tc_dgrad("e3a", b["g3"], h3, w3, out_f32=b["dp2"])
        N.call("sgb_nn_pool2_bwd", B, h2, w2, 64, N.ptr(b["dp2"]), N.ptr(b["dcat2"]), 192, 128, N.ptr(b["cat2"]),
               192, 128, N.ptr(b["g2b"]), s)
        # encoder level 2
        self._tc_wgrad("e2b", b["g2b"], b["a2a"], h2, w2)
        self._tc_dgrad("e2b", b["g2b"], h2, w2, out_bf16=b["g2"], mask=b["a2a"])
        self._tc_wgrad("e2a", b["g2"], b["p1"], h2, w2)
        self._tc_dgrad("e2a", b["g2"], h2, w2, out_f32=b["dp1"])
        N.call("sgb_nn_pool2_bwd", B, h1, w1, 32, N.ptr(b["dp1"]), N.ptr(b["dcat1"]), 96, 64, N.ptr(b["cat1"]),
               96, 64, N.ptr(b["g1b"]), s)
        # encoder level 1
        self._tc_wgrad("e1b", b["g1b"], b["a1a"], h1, w1)
        self._tc_dgrad("e1b", b["g1b"], h1, w1, out_bf16=b["g1"], mask=b["a1a"])
        N.call("sgb_nn_conv_in_wgrad", B, h1, w1, 32, N.ptr(self._x), N.ptr(b["g1"]), 32, N.ptr(self.gW["e1a"]),
               N.ptr(self.gb["e1a"]), s)

    def zero_grad(self):
        self.grads.zero_()

    def adam_step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, wd=0.0):
        self.step_count += 1
        N.call("sgb_nn_adam", self.params.numel(), N.ptr(self.params), N.ptr(self.grads), N.ptr(self.m),
               N.ptr(self.v), lr, b1, b2, eps, self.step_count, wd, N.stream_handle())
        self.pack()

    def train_batch(self, x, target, lr=1e-3):
        """One Adam step on the mean squared error; returns the loss (device scalar)."""
        pred = self.forward(x)
        b = self._bufs
        b["loss"].zero_()
        N.call("sgb_nn_mse", pred.numel(), N.ptr(pred), N.ptr(target.contiguous()), N.ptr(b["dpred"]),
               N.ptr(b["loss"]), N.stream_handle())
        self.zero_grad()
        self.backward(b["dpred"])
        self.adam_step(lr)
        return b["loss"]

    def predict(self, x):
        return self.forward(x).clone()
