"""Level-3 surrogate: a 3-D convolutional U-Net (3 levels, 32 / 64 / 128
channels, BF16 weights and activations, FP32 accumulation) that predicts the
Level-3 field at the end of one Level-2 step, trained and run with the BF16
tensor-core kernels of libgomelt (``gm_unet_*``).  No counterpart in the
reference.

Network (grid G1 = B x X x Y x Z voxels = Level-3 nodes ix < X, iy < Y,
1 <= iz <= Z; G2 = G1 / 2, G3 = G1 / 4; every convolution 3x3x3 + ReLU):

    x(16) -c1-> 32 -c2-> e1 (32) --pool--> 32 -c3-> 64 -c4-> e2 (64) --pool-->
    64 -c5-> 128 -c6-> 128 --up--> [128 | e2] -c7-> 64 -c8-> 64 --up-->
    [64 | e1] -c9-> 32 -c10-> 32 -head (1x1)-> y

Input channels (``gm_surrogate_pack``): the Level-2 field at the end of the
step prolongated to Level 3, the Level-3 field at its start, the node offset
from the mid-step laser position, power and speed.  Output: the fine
correction (T3_end - I(T2)) / S.  A prediction is accepted when the energy
balance of the window over the step (``diagnostics.Diagnostics``) closes to
1 % of the absorbed laser energy; otherwise the plain Level-3 steps run.
"""

from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

import _native as N
import kern

# (name, cin, cout, level)
LAYERS = [("c1", 16, 32, 0), ("c2", 32, 32, 0), ("c3", 32, 64, 1), ("c4", 64, 64, 1), ("c5", 64, 128, 2),
          ("c6", 128, 128, 2), ("c7", 192, 64, 1), ("c8", 64, 64, 1), ("c9", 96, 32, 0), ("c10", 32, 32, 0)]
HEAD_C = 32
T_SCALE = 1000.0  # K per unit of the network's temperature channels
P_SCALE, V_SCALE = 400.0, 1500.0  # W, mm/s


def _i4(v):
    return (C.c_int * 4)(*[int(x) for x in v])


def _ptr(t):
    return None if t is None else t.data_ptr()


class UNet:
    def __init__(self, device="cuda", seed=0, stream=None):
        self.dev = torch.device(device)
        self.stream = stream
        g = torch.Generator(device="cpu").manual_seed(seed)
        self.p = {}
        for name, cin, cout, _ in LAYERS:
            fan = 27 * cin if name != "c1" else 27 * 6  # six live input channels
            W = torch.randn(27, cout, cin, generator=g) * math.sqrt(2.0 / fan)
            if name == "c1":
                W[:, :, 6:] = 0
            self.p[name] = self._param(W)
            self.p[name + "b"] = self._param(torch.zeros(cout), bf16=False)
        self.p["head"] = self._param(torch.randn(HEAD_C, generator=g) * 0.01, bf16=False)
        self.t = 0
        self._bufs = {}

    def _param(self, w, bf16=True):
        d = dict(w=w.to(self.dev, torch.float32).contiguous())
        d["g"] = torch.zeros_like(d["w"])
        d["m"] = torch.zeros_like(d["w"])
        d["v"] = torch.zeros_like(d["w"])
        if bf16:
            d["wb"] = d["w"].to(torch.bfloat16).contiguous()
            d["wt"] = d["w"].permute(0, 2, 1).contiguous().to(torch.bfloat16)
        return d

    # ------------------------------------------------------------------
    def _call(self, name, *args, kernels=None):
        N.call(name, *args, kern.stream_ptr(self.stream), kernels=kernels)

    def _conv(self, grid, cin, cout, inp, W, out, *, bias=None, relu=1, mask=None, mirror=0):
        a = N.gm_conv_args()
        a.grid[:] = [int(x) for x in grid]
        a.cin, a.cout = cin, cout
        a.in_, a.in_stride, a.in_off = inp[0].data_ptr(), inp[1], inp[2]
        a.w = W.data_ptr()
        a.bias = _ptr(bias)
        a.relu = relu
        if mask is not None:
            a.mask, a.mask_stride, a.mask_off = mask[0].data_ptr(), mask[1], mask[2]
        a.mirror = mirror
        a.out, a.out_stride, a.out_off = out[0].data_ptr(), out[1], out[2]
        # work of the tensor-core form: the weights in its tile layout (one buffer, calls in stream order)
        a.wpack = self._buf("wpack", (27 * cin * cout,), torch.bfloat16, grow=True).data_ptr()
        kernels = 2 if N.lib().gm_unet_conv3_tc_eligible(C.byref(a)) else 1
        self._call("gm_unet_conv3", C.byref(a), kernels=kernels)

    def _wgrad(self, grid, cin, cout, inp, dy, dw):
        need = int(N.lib().gm_unet_wgrad_scratch(_i4(grid), cin, cout))
        scr = self._buf("wscr", (need,), torch.float32, grow=True)
        a = N.gm_wgrad_args()
        a.grid[:] = [int(x) for x in grid]
        a.cin, a.cout = cin, cout
        a.in_, a.in_stride, a.in_off = inp[0].data_ptr(), inp[1], inp[2]
        a.dy, a.dy_stride, a.dy_off = dy[0].data_ptr(), dy[1], dy[2]
        a.dw = dw.data_ptr()
        a.scratch, a.scratch_cap = scr.data_ptr(), scr.numel()
        self._call("gm_unet_wgrad", C.byref(a))

    def _bias_grad(self, grid, Cn, dy, db):
        V = int(np.prod(grid))
        nb = min(1024, (V + 4095) // 4096)
        scr = self._buf("bscr", (max(nb * Cn, 1),), torch.float32, grow=True)
        self._call("gm_unet_bias_grad", _i4(grid), Cn, dy[0].data_ptr(), dy[1], dy[2], scr.data_ptr(), scr.numel(),
                   db.data_ptr())

    def _buf(self, key, shape, dtype, grow=False):
        t = self._bufs.get(key)
        n = int(np.prod(shape))
        if t is None or t.dtype != dtype or (t.numel() < n if grow else t.shape != torch.Size(shape)):
            t = torch.empty(shape, dtype=dtype, device=self.dev)
            self._bufs[key] = t
        return t

    def _acts(self, B, X, Y, Z):
        V = [B * X * Y * Z, B * (X // 2) * (Y // 2) * (Z // 2), B * (X // 4) * (Y // 4) * (Z // 4)]
        bf = torch.bfloat16
        spec = {"a1": (0, 32), "d1cat": (0, 96), "a9": (0, 32), "a10": (0, 32), "p1": (1, 32), "a3": (1, 64),
                "d2cat": (1, 192), "a7": (1, 64), "a8": (1, 64), "p2": (2, 64), "a5": (2, 128), "a6": (2, 128)}
        A = {k: self._buf("act_" + k, (V[lv], c), bf) for k, (lv, c) in spec.items()}
        Gd = {k: self._buf("grd_" + k, (V[lv], c), bf) for k, (lv, c) in spec.items()}
        Gd["tmp1"] = self._buf("grd_tmp1", (V[0], 32), bf)
        Gd["tmp2"] = self._buf("grd_tmp2", (V[1], 64), bf)
        return V, A, Gd

    # ------------------------------------------------------------------
    def forward(self, x, grid):
        """x: BF16 [V, 16] (network grid {B, X, Y, Z}); returns FP32 [V]."""
        B, X, Y, Z = (int(v) for v in grid)
        if X % 4 or Y % 4 or Z % 4:
            raise N.GomeltError("network grid must be divisible by 4 along X, Y, Z")
        G1, G2, G3 = (B, X, Y, Z), (B, X // 2, Y // 2, Z // 2), (B, X // 4, Y // 4, Z // 4)
        V, A, _ = self._acts(B, X, Y, Z)
        P = self.p
        self.grid, self.x = grid, x
        cv = self._conv
        cv(G1, 16, 32, (x, 16, 0), P["c1"]["wb"], (A["a1"], 32, 0), bias=P["c1b"]["w"])
        cv(G1, 32, 32, (A["a1"], 32, 0), P["c2"]["wb"], (A["d1cat"], 96, 64), bias=P["c2b"]["w"])
        self._call("gm_unet_pool2", _i4(G1), 32, A["d1cat"].data_ptr(), 96, 64, A["p1"].data_ptr(), 32, 0, 0)
        cv(G2, 32, 64, (A["p1"], 32, 0), P["c3"]["wb"], (A["a3"], 64, 0), bias=P["c3b"]["w"])
        cv(G2, 64, 64, (A["a3"], 64, 0), P["c4"]["wb"], (A["d2cat"], 192, 128), bias=P["c4b"]["w"])
        self._call("gm_unet_pool2", _i4(G2), 64, A["d2cat"].data_ptr(), 192, 128, A["p2"].data_ptr(), 64, 0, 0)
        cv(G3, 64, 128, (A["p2"], 64, 0), P["c5"]["wb"], (A["a5"], 128, 0), bias=P["c5b"]["w"])
        cv(G3, 128, 128, (A["a5"], 128, 0), P["c6"]["wb"], (A["a6"], 128, 0), bias=P["c6b"]["w"])
        self._call("gm_unet_up2", _i4(G2), 128, A["a6"].data_ptr(), 128, 0, A["d2cat"].data_ptr(), 192, 0, 0)
        cv(G2, 192, 64, (A["d2cat"], 192, 0), P["c7"]["wb"], (A["a7"], 64, 0), bias=P["c7b"]["w"])
        cv(G2, 64, 64, (A["a7"], 64, 0), P["c8"]["wb"], (A["a8"], 64, 0), bias=P["c8b"]["w"])
        self._call("gm_unet_up2", _i4(G1), 64, A["a8"].data_ptr(), 64, 0, A["d1cat"].data_ptr(), 96, 0, 0)
        cv(G1, 96, 32, (A["d1cat"], 96, 0), P["c9"]["wb"], (A["a9"], 32, 0), bias=P["c9b"]["w"])
        cv(G1, 32, 32, (A["a9"], 32, 0), P["c10"]["wb"], (A["a10"], 32, 0), bias=P["c10b"]["w"])
        pred = self._buf("pred", (V[0],), torch.float32)
        self._call("gm_unet_head", V[0], HEAD_C, A["a10"].data_ptr(), 32, 0, P["head"]["w"].data_ptr(),
                   C.c_float(0.0), pred.data_ptr())
        return pred

    def backward(self, target, lmask, inv_count):
        """Gradients of mean_masked (pred - target)^2 for the last forward;
        returns the loss as a device scalar."""
        B, X, Y, Z = (int(v) for v in self.grid)
        G1, G2, G3 = (B, X, Y, Z), (B, X // 2, Y // 2, Z // 2), (B, X // 4, Y // 4, Z // 4)
        V, A, Gd = self._acts(B, X, Y, Z)
        P = self.p
        pred = self._bufs["pred"]
        hs = int(N.lib().gm_unet_head_scratch(V[0], HEAD_C))
        hscr = self._buf("hscr", (hs,), torch.float32, grow=True)
        dwb = self._buf("dwb", (HEAD_C + 2,), torch.float32)
        self._call("gm_unet_head_bwd", V[0], HEAD_C, A["a10"].data_ptr(), 32, 0, P["head"]["w"].data_ptr(),
                   pred.data_ptr(), target.data_ptr(), _ptr(lmask), C.c_float(inv_count), Gd["a10"].data_ptr(), 32,
                   0, hscr.data_ptr(), hscr.numel(), dwb.data_ptr())
        P["head"]["g"].copy_(dwb[:HEAD_C])

        def layer(name, grid, cin, cout, inp, dy, dx=None, mask=None):
            self._wgrad(grid, cin, cout, inp, dy, P[name]["g"])
            self._bias_grad(grid, cout, dy, P[name + "b"]["g"])
            if dx is not None:
                self._conv(grid, cout, cin, dy, P[name]["wt"], dx, relu=0, mask=mask, mirror=1)

        layer("c10", G1, 32, 32, (A["a9"], 32, 0), (Gd["a10"], 32, 0), (Gd["a9"], 32, 0), (A["a9"], 32, 0))
        layer("c9", G1, 96, 32, (A["d1cat"], 96, 0), (Gd["a9"], 32, 0), (Gd["d1cat"], 96, 0), (A["d1cat"], 96, 0))
        self._call("gm_unet_up2", _i4(G1), 64, Gd["d1cat"].data_ptr(), 96, 0, Gd["a8"].data_ptr(), 64, 0, 1)
        layer("c8", G2, 64, 64, (A["a7"], 64, 0), (Gd["a8"], 64, 0), (Gd["a7"], 64, 0), (A["a7"], 64, 0))
        layer("c7", G2, 192, 64, (A["d2cat"], 192, 0), (Gd["a7"], 64, 0), (Gd["d2cat"], 192, 0), (A["d2cat"], 192, 0))
        self._call("gm_unet_up2", _i4(G2), 128, Gd["d2cat"].data_ptr(), 192, 0, Gd["a6"].data_ptr(), 128, 0, 1)
        layer("c6", G3, 128, 128, (A["a5"], 128, 0), (Gd["a6"], 128, 0), (Gd["a5"], 128, 0), (A["a5"], 128, 0))
        layer("c5", G3, 64, 128, (A["p2"], 64, 0), (Gd["a5"], 128, 0), (Gd["p2"], 64, 0), None)
        self._call("gm_unet_pool2", _i4(G2), 64, Gd["p2"].data_ptr(), 64, 0, Gd["tmp2"].data_ptr(), 64, 0, 1)
        self._call("gm_unet_add_slice", V[1], 64, Gd["tmp2"].data_ptr(), 64, 0, Gd["d2cat"].data_ptr(), 192, 128,
                   A["d2cat"].data_ptr(), 192, 128)
        layer("c4", G2, 64, 64, (A["a3"], 64, 0), (Gd["d2cat"], 192, 128), (Gd["a3"], 64, 0), (A["a3"], 64, 0))
        layer("c3", G2, 32, 64, (A["p1"], 32, 0), (Gd["a3"], 64, 0), (Gd["p1"], 32, 0), None)
        self._call("gm_unet_pool2", _i4(G1), 32, Gd["p1"].data_ptr(), 32, 0, Gd["tmp1"].data_ptr(), 32, 0, 1)
        self._call("gm_unet_add_slice", V[0], 32, Gd["tmp1"].data_ptr(), 32, 0, Gd["d1cat"].data_ptr(), 96, 64,
                   A["d1cat"].data_ptr(), 96, 64)
        layer("c2", G1, 32, 32, (A["a1"], 32, 0), (Gd["d1cat"], 96, 64), (Gd["a1"], 32, 0), (A["a1"], 32, 0))
        layer("c1", G1, 16, 32, (self.x, 16, 0), (Gd["a1"], 32, 0))
        return dwb[HEAD_C + 1]

    def step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, wd=0.0):
        self.t += 1
        c1, c2 = 1.0 - beta1 ** self.t, 1.0 - beta2 ** self.t
        for name, cin, cout, _ in LAYERS:
            for key, bf in ((name, True), (name + "b", False)):
                d = self.p[key]
                a = N.gm_adam_args()
                a.n = d["w"].numel()
                a.w, a.grad, a.m, a.v = d["w"].data_ptr(), d["g"].data_ptr(), d["m"].data_ptr(), d["v"].data_ptr()
                a.lr, a.beta1, a.beta2, a.eps, a.c1, a.c2, a.wd = lr, beta1, beta2, eps, c1, c2, wd
                if bf:
                    a.wb, a.wt, a.cout, a.cin = d["wb"].data_ptr(), d["wt"].data_ptr(), cout, cin
                self._call("gm_unet_adam", C.byref(a))
        d = self.p["head"]
        a = N.gm_adam_args()
        a.n = d["w"].numel()
        a.w, a.grad, a.m, a.v = d["w"].data_ptr(), d["g"].data_ptr(), d["m"].data_ptr(), d["v"].data_ptr()
        a.lr, a.beta1, a.beta2, a.eps, a.c1, a.c2, a.wd = lr, beta1, beta2, eps, c1, c2, wd
        self._call("gm_unet_adam", C.byref(a))

    def flops(self, grid):
        """Multiply-add FLOPs (x2) of one forward on grid {B, X, Y, Z}."""
        B, X, Y, Z = (int(v) for v in grid)
        V = [B * X * Y * Z, B * X * Y * Z // 8, B * X * Y * Z // 64]
        f = sum(2 * 27 * cin * cout * V[lv] for _, cin, cout, lv in LAYERS)
        return f + 2 * HEAD_C * V[0]

    def state(self):
        return {k: v["w"].detach().cpu().numpy() for k, v in self.p.items()}

    def load(self, st):
        for k, w in st.items():
            d = self.p[k]
            d["w"].copy_(torch.as_tensor(w, device=self.dev))
            if "wb" in d:
                d["wb"].copy_(d["w"].to(torch.bfloat16))
                d["wt"].copy_(d["w"].permute(0, 2, 1).to(torch.bfloat16))


def pack(*, grid, nodes, T2i, T3o, par, T_amb, x, T3n=None, target=None, lmask=None, stream=None):
    """Network input (and target / loss mask) of B windows; see
    gm_surrogate_pack."""
    a = N.gm_surr_args()
    a.grid[:] = [int(v) for v in grid]
    a.nodes[:] = [int(v) for v in nodes]
    a.T2i, a.T3o, a.T3n, a.par = T2i.data_ptr(), T3o.data_ptr(), _ptr(T3n), par.data_ptr()
    a.T_amb, a.scale = float(T_amb), T_SCALE
    a.x, a.target, a.lmask = x.data_ptr(), _ptr(target), _ptr(lmask)
    N.call("gm_surrogate_pack", C.byref(a), kern.stream_ptr(stream))
    return a


def unpack(a, pred, T3, stream=None):
    N.call("gm_surrogate_unpack", C.byref(a), pred.data_ptr(), T3.data_ptr(), kern.stream_ptr(stream))


def window_params(origin, h, laser_xy, radius, power, speed):
    """The 8 per-sample doubles of gm_surrogate_pack."""
    return [origin[0], origin[1], h, laser_xy[0], laser_xy[1], 1.0 / radius, power / P_SCALE, speed / V_SCALE]
