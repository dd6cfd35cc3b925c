"""Learned preconditioner for the Poisson CG: a 3-level 3-D U-Net (16/32/64
channels, 3x3x3 kernels, BF16 weights and activations, FP32 accumulation),
applied as z = M(r) inside flexible CG, with Jacobi-PCG as the fallback.

Forward and backward passes run on the project's tensor-core kernels
(ngb_conv3d, ngb_conv3d_bwd_weight, ngb_pool2, ngb_up2, ngb_relu_bwd,
ngb_adam); torch provides device buffers and elementwise glue. The network is
bias-free with ReLU activations, so M(a r) = a M(r) for a > 0; the input is
scaled by its RMS and the output scaled back.

Layer graph (level l has grid n / 2^l; "cat" buffers hold a skip connection
next to the upsampled coarse features, so concatenation costs nothing):

    in0(16) -c0a-> a0(16) -c0b-> cat0[32:48] -pool-> p0(16) -c1a-> a1(32) -c1b-> cat1[64:96]
    -pool-> p1(32) -c2a-> a2(64) -c2b-> b2(64) -up-> cat1[0:64]
    cat1(96) -c1c-> d1a(32) -c1d-> d1b(32) -up-> cat0[0:32]
    cat0(48) -c0c-> d0a(16) -c0d-> out(16, channel 0 = M(r))
"""
import ctypes
import math

import torch

from . import STORE_F32, STORE_F64, _ptr, check, lib

LAYERS = [("c0a", 16, 16), ("c0b", 16, 16), ("c1a", 16, 32), ("c1b", 32, 32), ("c2a", 32, 64), ("c2b", 64, 64),
          ("c1c", 96, 32), ("c1d", 32, 32), ("c0c", 48, 16), ("c0d", 16, 16)]


def _p(t, off=0):
    """Pointer to channel `off` of a [V, C] tensor."""
    return ctypes.c_void_p(t.data_ptr() + off * t.element_size())


class UNet:
    def __init__(self, seed=0, device="cuda"):
        self.dev = torch.device(device)
        g = torch.Generator().manual_seed(seed)
        self.w = {}  # FP32 master weights [cout, 27, cin]
        for name, cin, cout in LAYERS:
            std = math.sqrt(2.0 / (27 * cin))
            w = torch.randn(cout, 27, cin, generator=g) * std
            if name == "c0d":
                w.zero_()
                w[0] = torch.randn(27, cin, generator=g) * (0.1 * std)
            self.w[name] = w.to(self.dev).contiguous()
        self.wb, self.wt, self.g, self.m, self.s = {}, {}, {}, {}, {}
        for name, cin, cout in LAYERS:
            self.wb[name] = self.w[name].to(torch.bfloat16).contiguous()
            self.wt[name] = torch.empty(cin, 27, cout, dtype=torch.bfloat16, device=self.dev)
            self.g[name] = torch.zeros_like(self.w[name])
            self.m[name] = torch.zeros_like(self.w[name])
            self.s[name] = torch.zeros_like(self.w[name])
        self.step_count = 0
        self.shape = None
        # tcgen05 convolutions where the grid shape allows (ngb_conv3d_tc),
        # the mma.sync kernel elsewhere
        self.tensor_cores = True
        self._pk = {}
        self._refresh_flipped()

    # ------------------------------------------------------------------ buffers
    def _alloc(self, n):
        if self.shape == n:
            return
        if n % 4:
            raise ValueError("grid size must be a multiple of 4 (two poolings)")
        self.shape = n
        V0, V1, V2 = n ** 3, (n // 2) ** 3, (n // 4) ** 3
        bf, f = torch.bfloat16, torch.float32
        E = lambda V, C, dt: torch.zeros(V, C, dtype=dt, device=self.dev)
        self.in0, self.a0, self.cat0, self.d0a = E(V0, 16, bf), E(V0, 16, bf), E(V0, 48, bf), E(V0, 16, bf)
        self.out = E(V0, 16, f)
        self.p0, self.a1, self.cat1, self.d1a, self.d1b = E(V1, 16, bf), E(V1, 32, bf), E(V1, 96, bf), E(V1, 32, bf), E(V1, 32, bf)
        self.p1, self.a2, self.b2 = E(V2, 32, bf), E(V2, 64, bf), E(V2, 64, bf)
        self.grads = None

    def _alloc_grads(self):
        if self.grads is not None:
            return
        n = self.shape
        V0, V1, V2 = n ** 3, (n // 2) ** 3, (n // 4) ** 3
        bf, f = torch.bfloat16, torch.float32
        E = lambda V, C, dt: torch.zeros(V, C, dtype=dt, device=self.dev)
        self.grads = dict(gout=E(V0, 16, f), g16=E(V0, 16, f), gcat0=E(V0, 48, f), dyb0=E(V0, 16, bf),
                          g1=E(V1, 32, f), gcat1=E(V1, 96, f), gp0=E(V1, 16, f), dyb1=E(V1, 32, bf),
                          g2=E(V2, 64, f), gp1=E(V2, 32, f), dyb2=E(V2, 64, bf))

    def _refresh_flipped(self):
        self._pk = {}
        for name, cin, cout in LAYERS:
            check(lib().ngb_flip_weights(cout, cin, _ptr(self.w[name]), _ptr(self.wt[name]), None))

    def _packed(self, w):
        """Tensor-core operand image of BF16 weights [cout, 27, cin] (cached until the weights change)."""
        key = (w.data_ptr(), tuple(w.shape))
        pk = self._pk.get(key)
        if pk is None:
            pk = torch.empty_like(w)
            check(lib().ngb_conv3d_pack(w.shape[0], w.shape[2], _ptr(w), _ptr(pk), None))
            self._pk[key] = pk
        return pk

    # ------------------------------------------------------------------ primitives
    def _conv(self, lvl, x, xoff, cin, w, y, yoff, cout, out_f32=False, relu=False, acc=False):
        n = self.shape >> lvl
        L = lib()
        if self.tensor_cores and L.ngb_conv3d_tc_supported(n, n, n, x.shape[1], cin, y.shape[1], cout):
            check(L.ngb_conv3d_tc(n, n, n, _p(x, xoff), x.shape[1], cin, _ptr(self._packed(w)), None, _p(y, yoff), y.shape[1],
                                  cout, int(out_f32), int(relu), int(acc), None))
            self._tc_used = True
            return
        for lo in range(0, cout, 64):  # the mma.sync kernel takes at most 64 output channels
            hi = min(cout, lo + 64)
            check(L.ngb_conv3d(n, n, n, _p(x, xoff), x.shape[1], cin, _ptr(w[lo:hi]), None, _p(y, yoff + lo), y.shape[1],
                               hi - lo, int(out_f32), int(relu), int(acc), None))

    def _tc_check(self):
        """Raise if a tensor-core convolution of the last pass reported a pipeline time-out (synchronises)."""
        if getattr(self, "_tc_used", False):
            self._tc_used = False
            check(lib().ngb_conv3d_tc_check(None))

    def _bwdw(self, lvl, x, xoff, cin, dy, cout, dw):
        n = self.shape >> lvl
        check(lib().ngb_conv3d_bwd_weight(n, n, n, _p(x, xoff), x.shape[1], cin, _p(dy), dy.shape[1], cout, _ptr(dw), None))

    def _relu_bwd(self, g, goff, C, y, yoff, out):
        V = g.shape[0]
        check(lib().ngb_relu_bwd(V, C, _p(g, goff), g.shape[1], _p(y, yoff) if y is not None else None,
                                 y.shape[1] if y is not None else 0, _p(out), out.shape[1], None))

    def _pool(self, lvl, x, xoff, C, y):
        n = self.shape >> lvl
        check(lib().ngb_pool2(n, n, n, C, _p(x, xoff), x.shape[1], _p(y), y.shape[1], None))

    def _pool_bwd(self, lvl, dy, C, dx, dxoff, acc):
        n = self.shape >> lvl
        check(lib().ngb_pool2_bwd(n, n, n, C, _p(dy), dy.shape[1], _p(dx, dxoff), dx.shape[1], int(acc), None))

    def _up(self, lvl_fine, x, C, y, yoff):
        n = self.shape >> lvl_fine
        check(lib().ngb_up2(n, n, n, C, _p(x), x.shape[1], _p(y, yoff), y.shape[1], None))

    def _up_bwd(self, lvl_fine, dy, dyoff, C, dx):
        n = self.shape >> lvl_fine
        check(lib().ngb_up2_bwd(n, n, n, C, _p(dy, dyoff), dy.shape[1], _p(dx), dx.shape[1], None))

    # ------------------------------------------------------------------ network
    def forward(self, r, sync=True):
        """z = M(r) for a float32 field r of n^3 values (x fastest); returns z (float32).

        sync=False keeps the input scale on the device and skips the
        tensor-core time-out check (call check() later): no host round trip."""
        n = round(r.numel() ** (1.0 / 3.0))
        self._alloc(n)
        if sync:
            sigma = float(torch.sqrt(torch.mean(r.double() ** 2)).item()) or 1.0
        else:
            rms = torch.sqrt(torch.mean(r.double() ** 2)).float()
            sigma = torch.where(rms > 0, rms, torch.ones_like(rms))
        self.sigma = sigma
        self.in0.zero_()
        self.in0[:, 0] = (r / sigma).to(torch.bfloat16)
        self._layers()
        if sync:
            self._tc_check()
        return self.out[:, 0] * sigma

    def _layers(self):
        """The convolutions, poolings and upsamplings from in0 to out."""
        W = self.wb
        self._conv(0, self.in0, 0, 16, W["c0a"], self.a0, 0, 16, relu=True)
        self._conv(0, self.a0, 0, 16, W["c0b"], self.cat0, 32, 16, relu=True)
        self._pool(0, self.cat0, 32, 16, self.p0)
        self._conv(1, self.p0, 0, 16, W["c1a"], self.a1, 0, 32, relu=True)
        self._conv(1, self.a1, 0, 32, W["c1b"], self.cat1, 64, 32, relu=True)
        self._pool(1, self.cat1, 64, 32, self.p1)
        self._conv(2, self.p1, 0, 32, W["c2a"], self.a2, 0, 64, relu=True)
        self._conv(2, self.a2, 0, 64, W["c2b"], self.b2, 0, 64, relu=True)
        self._up(1, self.b2, 64, self.cat1, 0)
        self._conv(1, self.cat1, 0, 96, W["c1c"], self.d1a, 0, 32, relu=True)
        self._conv(1, self.d1a, 0, 32, W["c1d"], self.d1b, 0, 32, relu=True)
        self._up(0, self.d1b, 32, self.cat0, 0)
        self._conv(0, self.cat0, 0, 48, W["c0c"], self.d0a, 0, 16, relu=True)
        self._conv(0, self.d0a, 0, 16, W["c0d"], self.out, 0, 16, out_f32=True)

    def check(self):
        """Raise if a tensor-core convolution since the last check timed out (synchronises)."""
        self._tc_check()

    def apply(self, r, e, scale=1.0, rr=None, scratch=None):
        """e = scale * M(r), 0 on the box faces, entirely on the device (no
        host round trip, no torch arithmetic): |r|^2 by ngb_dot, the scaled
        BF16 input and the scaled output by ngb_unet_input / ngb_unet_output.
        Tensor-core time-outs are reported by check()."""
        n = round(r.numel() ** (1.0 / 3.0))
        self._alloc(n)
        L = lib()
        if rr is None:
            rr = torch.zeros(1, dtype=torch.float64, device=self.dev)
        if scratch is None:
            scratch = torch.empty(L.ngb_dot_scratch_doubles(r.numel()), dtype=torch.float64, device=self.dev)
        check(L.ngb_dot(r.numel(), STORE_F32, _ptr(r), _ptr(r), _ptr(rr), _ptr(scratch), None))
        check(L.ngb_unet_input(r.numel(), _ptr(r), _ptr(rr), _ptr(self.in0), self.in0.shape[1], None))
        self._layers()
        check(L.ngb_unet_output(n, n, n, _ptr(self.out), self.out.shape[1], _ptr(rr), scale, _ptr(e), None))
        return e

    def backward(self, dz, sync=True):
        """Accumulates dL/dw into self.g given dL/dz (float32 n^3) of the last
        forward. sync=False skips the tensor-core time-out check (call check() later)."""
        self._alloc_grads()
        G, Wt = self.grads, self.wt
        G["gout"].zero_()
        G["gout"][:, 0] = dz * self.sigma
        # c0d
        self._relu_bwd(G["gout"], 0, 16, None, 0, G["dyb0"])
        self._bwdw(0, self.d0a, 0, 16, G["dyb0"], 16, self.g["c0d"])
        self._conv(0, G["dyb0"], 0, 16, Wt["c0d"], G["g16"], 0, 16, out_f32=True)
        # c0c
        self._relu_bwd(G["g16"], 0, 16, self.d0a, 0, G["dyb0"])
        self._bwdw(0, self.cat0, 0, 48, G["dyb0"], 16, self.g["c0c"])
        self._conv(0, G["dyb0"], 0, 16, Wt["c0c"], G["gcat0"], 0, 48, out_f32=True)
        # up to level 0 <- d1b
        g1 = G["g1"]
        self._up_bwd(0, G["gcat0"], 0, 32, g1)
        # c1d
        self._relu_bwd(g1, 0, 32, self.d1b, 0, G["dyb1"])
        self._bwdw(1, self.d1a, 0, 32, G["dyb1"], 32, self.g["c1d"])
        self._conv(1, G["dyb1"], 0, 32, Wt["c1d"], g1, 0, 32, out_f32=True)
        # c1c (96 input channels: two backward-data calls of 64 and 32 channels)
        self._relu_bwd(g1, 0, 32, self.d1a, 0, G["dyb1"])
        self._bwdw(1, self.cat1, 0, 96, G["dyb1"], 32, self.g["c1c"])
        self._conv(1, G["dyb1"], 0, 32, Wt["c1c"], G["gcat1"], 0, 96, out_f32=True)
        # up to level 1 <- b2
        g2 = G["g2"]
        self._up_bwd(1, G["gcat1"], 0, 64, g2)
        # c2b
        self._relu_bwd(g2, 0, 64, self.b2, 0, G["dyb2"])
        self._bwdw(2, self.a2, 0, 64, G["dyb2"], 64, self.g["c2b"])
        self._conv(2, G["dyb2"], 0, 64, Wt["c2b"], g2, 0, 64, out_f32=True)
        # c2a
        self._relu_bwd(g2, 0, 64, self.a2, 0, G["dyb2"])
        self._bwdw(2, self.p1, 0, 32, G["dyb2"], 64, self.g["c2a"])
        self._conv(2, G["dyb2"], 0, 64, Wt["c2a"], G["gp1"], 0, 32, out_f32=True)
        # pool 1 -> skip1
        self._pool_bwd(1, G["gp1"], 32, G["gcat1"], 64, True)
        # c1b
        self._relu_bwd(G["gcat1"], 64, 32, self.cat1, 64, G["dyb1"])
        self._bwdw(1, self.a1, 0, 32, G["dyb1"], 32, self.g["c1b"])
        self._conv(1, G["dyb1"], 0, 32, Wt["c1b"], g1, 0, 32, out_f32=True)
        # c1a
        self._relu_bwd(g1, 0, 32, self.a1, 0, G["dyb1"])
        self._bwdw(1, self.p0, 0, 16, G["dyb1"], 32, self.g["c1a"])
        self._conv(1, G["dyb1"], 0, 32, Wt["c1a"], G["gp0"], 0, 16, out_f32=True)
        # pool 0 -> skip0
        self._pool_bwd(0, G["gp0"], 16, G["gcat0"], 32, True)
        # c0b
        self._relu_bwd(G["gcat0"], 32, 16, self.cat0, 32, G["dyb0"])
        self._bwdw(0, self.a0, 0, 16, G["dyb0"], 16, self.g["c0b"])
        self._conv(0, G["dyb0"], 0, 16, Wt["c0b"], G["g16"], 0, 16, out_f32=True)
        # c0a
        self._relu_bwd(G["g16"], 0, 16, self.a0, 0, G["dyb0"])
        self._bwdw(0, self.in0, 0, 16, G["dyb0"], 16, self.g["c0a"])
        if sync:
            self._tc_check()

    def zero_grad(self):
        for k in self.g:
            self.g[k].zero_()

    def adam_step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        for name, cin, cout in LAYERS:
            check(lib().ngb_adam(self.w[name].numel(), _ptr(self.w[name]), _ptr(self.g[name]), _ptr(self.m[name]),
                                 _ptr(self.s[name]), lr, b1, b2, eps, self.step_count, _ptr(self.wb[name]), None))
        self._refresh_flipped()

    def flops_forward(self, n):
        """Multiply-add FLOPs (2 per MAC) of one forward application at n^3."""
        per = {"c0a": 0, "c0b": 0, "c0c": 0, "c0d": 0, "c1a": 1, "c1b": 1, "c1c": 1, "c1d": 1, "c2a": 2, "c2b": 2}
        return sum(2 * 27 * cin * cout * (n >> per[name]) ** 3 for name, cin, cout in LAYERS)

    def state_dict(self):
        return {k: v.cpu() for k, v in self.w.items()}

    def flat_weights(self):
        """The FP32 master weights as one host array in the layer order of the weight file."""
        return torch.cat([self.w[name].reshape(-1).cpu() for name, _, _ in LAYERS]).contiguous()

    def save_weights(self, path):
        """Writes the weight file (BF16 values, the precision the network computes in)."""
        w = self.flat_weights()
        check(lib().ngb_unet_write_weights(str(path).encode(), ctypes.c_void_p(w.data_ptr()), w.numel()))

    def load_weights(self, path):
        """Reads a weight file written by save_weights (or by ngb_unet_write_weights)."""
        w = read_weights(path)
        off = 0
        for name, cin, cout in LAYERS:
            cnt = cout * 27 * cin
            self.w[name].copy_(w[off:off + cnt].reshape(cout, 27, cin).to(self.dev))
            self.wb[name].copy_(self.w[name].to(torch.bfloat16))
            off += cnt
        self._refresh_flipped()

    def load_state_dict(self, sd):
        for k, v in sd.items():
            self.w[k].copy_(v.to(self.dev))
            self.wb[k].copy_(self.w[k].to(torch.bfloat16))
        self._refresh_flipped()


def read_weights(path):
    """FP32 host tensor of a U-Net weight file (ngb_unet_read_weights)."""
    L = lib()
    w = torch.empty(int(L.ngb_unet_weight_count()), dtype=torch.float32)
    check(L.ngb_unet_read_weights(str(path).encode(), ctypes.c_void_p(w.data_ptr()), w.numel()))
    return w
