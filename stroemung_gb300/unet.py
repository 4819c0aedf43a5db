"""Learned pressure warm start: a small BF16 U-Net on the tcgen05 kernels.

The network maps (RHS, fluid mask, previous pressure) of a solver step to a
correction of the previous pressure; the pressure solve then starts from the
corrected field when that lowers the initial residual, else from the previous
pressure (plain SOR stays the judge and the fallback).

Architecture (about 1.9 M parameters): 4 levels with 32/64/128/256 channels,
two 3x3 convolutions + ReLU per level, 2x2 average pooling down, nearest
upsampling up with skip concatenation, a 1x1 FP32 head.  Every convolution
(forward, weight gradient, data gradient) runs on the library's tcgen05
implicit-GEMM kernels (include/stroemung_nn.h); pooling, upsampling, masks,
the head, the loss and Adam are the library's own CUDA kernels.  torch only
provides device memory and the stream; no torch operator runs in the
forward, backward or update.

Loss: the relative Poisson residual of the corrected pressure over fluid
cells, sum r^2 / sum rhs^2 per sample, r = Lap(p) - rhs with the solver's
boundary copy, averaged over the batch.
"""
from __future__ import annotations

import contextlib

import math

import numpy as np

from . import _lib

CHANNELS = (32, 64, 128, 256)
IN_CH = 8  # rhs, mask, previous pressure, 5 zero pads


def _kp(cin_p: int) -> int:
    return -(-9 * cin_p // 64) * 64


class _Conv:
    """One 3x3 convolution layer: FP32 master weights + BF16 copies."""

    def __init__(self, net, cin, cout, rng):
        import torch
        self.cin, self.cout = cin, cout
        self.cin_p = -(-cin // 8) * 8
        self.kp = _kp(self.cin_p)
        self.kp_t = _kp(cout)
        w = np.zeros((cout, self.kp), np.float32)
        std = math.sqrt(2.0 / (9 * cin))
        wt = rng.normal(0.0, std, size=(cout, cin, 3, 3)).astype(np.float32)
        for ky in range(3):
            for kx in range(3):
                t = ky * 3 + kx
                w[:, t * self.cin_p:t * self.cin_p + cin] = wt[:, :, ky, kx]
        self.w = net._param(w.ravel())
        self.b = net._param(np.zeros(cout, np.float32))
        self.wt_bf = torch.empty(self.cin_p, self.kp_t, dtype=torch.bfloat16, device=net.device)


class UNet:
    def __init__(self, seed: int = 0, device="cuda"):
        import torch
        self.device = torch.device(device)
        self.L = _lib.load()
        self._params = []
        rng = np.random.default_rng(seed)
        c0, c1, c2, c3 = CHANNELS
        self.enc = [(_Conv(self, IN_CH, c0, rng), _Conv(self, c0, c0, rng)),
                    (_Conv(self, c0, c1, rng), _Conv(self, c1, c1, rng)),
                    (_Conv(self, c1, c2, rng), _Conv(self, c2, c2, rng))]
        self.mid = (_Conv(self, c2, c3, rng), _Conv(self, c3, c3, rng))
        self.dec = [(_Conv(self, c3 + c2, c2, rng), _Conv(self, c2, c2, rng)),
                    (_Conv(self, c2 + c1, c1, rng), _Conv(self, c1, c1, rng)),
                    (_Conv(self, c1 + c0, c0, rng), _Conv(self, c0, c0, rng))]
        # the head starts at zero: the first prediction is the previous pressure
        self.wh = self._param(np.zeros(c0, np.float32))
        self.bh = self._param(np.zeros(1, np.float32))
        self._finalize()
        self._bufs = {}
        self.step = 0
        # the stream the forward launches on (None: the default stream; a
        # capture stream while forward_graphed records), and the recorded
        # forwards by (input buffer, sizes)
        self._stream = None
        self._graphs = {}

    # ---- parameters: one flat FP32 buffer (weights, grads, Adam moments) ----
    def _param(self, arr):
        self._params.append(np.asarray(arr, np.float32).ravel())
        return len(self._params) - 1

    def _finalize(self):
        import torch
        sizes = [p.size for p in self._params]
        self._offsets = np.cumsum([0] + sizes)
        flat = np.concatenate(self._params)
        self.theta = torch.tensor(flat, device=self.device)
        self.grad = torch.zeros_like(self.theta)
        self.m = torch.zeros_like(self.theta)
        self.v = torch.zeros_like(self.theta)
        # BF16 mirror of theta, written by the Adam kernel; each layer's forward
        # weights are a [cout][kp] view of it
        self.theta_bf = torch.zeros(flat.size, dtype=torch.bfloat16, device=self.device)
        self.n_params = int(flat.size)
        self._mirror()

    def _ptr(self, idx, which=None):
        t = self.theta if which is None else which
        return t.data_ptr() + 4 * int(self._offsets[idx])

    def layers(self):
        for pair in self.enc:
            yield from pair
        yield from self.mid
        for pair in self.dec:
            yield from pair

    def parameter_count(self) -> int:
        return sum(l.cout * l.cin * 9 + l.cout for l in self.layers()) + CHANNELS[0] + 1

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with status {rc}")

    @contextlib.contextmanager
    def _deferred(self):
        """The tensor-core kernels of one pass run without a host wait each;
        their timeout flag is checked once at the end."""
        self.L.strm_nn_set_sync(0)
        try:
            yield
        finally:
            self.L.strm_nn_set_sync(1)
        self._check(self.L.strm_nn_status(None), "tensor-core kernels")

    def _wbf(self, layer):
        return self.theta_bf.data_ptr() + 2 * int(self._offsets[layer.w])

    def _mirror(self):
        """BF16 mirror of the masters (an Adam step with lr 0 on zero moments)."""
        self._check(self.L.strm_nn_zero(self.grad.data_ptr(), 4 * self.n_params, None), "zero")
        self._check(self.L.strm_nn_adam(self.theta.data_ptr(), self.grad.data_ptr(),
                                        self.m.data_ptr(), self.v.data_ptr(), self.n_params,
                                        0.0, 0.9, 0.999, 1e-8, 1, self.theta_bf.data_ptr(),
                                        None), "mirror")
        self._flip()

    def _flip(self):
        """Data-gradient (flipped, transposed) weights from the BF16 forward weights."""
        for l in self.layers():
            self._check(self.L.strm_nn_flip_weights(self._wbf(l), l.cout, l.cin_p, l.kp,
                                                    l.wt_bf.data_ptr(), l.cout, l.kp_t, None),
                        "flip")

    # ---- buffers -------------------------------------------------------------
    def _buffers(self, b, h, w):
        import torch
        key = (b, h, w)
        if key in self._bufs:
            return self._bufs[key]
        if h % 8 or w % 8:
            raise ValueError("the network needs sizes divisible by 8")
        bf = torch.bfloat16
        dev = self.device
        c0, c1, c2, c3 = CHANNELS

        def t(hh, ww, c, dt=bf):
            return torch.zeros(b, hh, ww, c, dtype=dt, device=dev)
        B = {}
        B["x"] = t(h, w, IN_CH)
        B["a0"], B["cat0"] = t(h, w, c0), t(h, w, c1 + c0)           # cat0 = [up(d1), e0]
        B["p0"] = t(h // 2, w // 2, c0)
        B["a1"], B["cat1"] = t(h // 2, w // 2, c1), t(h // 2, w // 2, c2 + c1)
        B["p1"] = t(h // 4, w // 4, c1)
        B["a2"], B["cat2"] = t(h // 4, w // 4, c2), t(h // 4, w // 4, c3 + c2)
        B["p2"] = t(h // 8, w // 8, c2)
        B["b1"], B["b2"] = t(h // 8, w // 8, c3), t(h // 8, w // 8, c3)
        B["d2a"], B["d2"] = t(h // 4, w // 4, c2), t(h // 4, w // 4, c2)
        B["d1a"], B["d1"] = t(h // 2, w // 2, c1), t(h // 2, w // 2, c1)
        B["d0a"], B["d0"] = t(h, w, c0), t(h, w, c0)
        B["q"] = torch.zeros(b, h, w, dtype=torch.float32, device=dev)
        # gradients
        for name in ("a0", "p0", "a1", "p1", "a2", "p2", "b1", "b2", "d2a", "d2", "d1a", "d1",
                     "d0a", "d0"):
            B["g_" + name] = torch.zeros_like(B[name])
        B["g_e0"] = t(h, w, c0)
        B["g_e1"] = t(h // 2, w // 2, c1)
        B["g_e2"] = t(h // 4, w // 4, c2)
        B["g_up0"] = t(h, w, c1)
        B["g_up1"] = t(h // 2, w // 2, c2)
        B["g_up2"] = t(h // 4, w // 4, c3)
        B["gm"] = t(h, w, c3)  # masked-gradient scratch (largest channel count at full size)
        self._bufs[key] = B
        return B

    def _forward_buffers(self, b, h, w):
        """The forward pass's buffers as views of one shared pool (no
        gradients): for predictions over many grid shapes, which would
        otherwise each keep a full set.  Valid until the next such call."""
        import torch
        if h % 8 or w % 8:
            raise ValueError("the network needs sizes divisible by 8")
        c0, c1, c2, c3 = CHANNELS
        spec = [("a0", h, w, c0), ("cat0", h, w, c1 + c0), ("p0", h // 2, w // 2, c0),
                ("a1", h // 2, w // 2, c1), ("cat1", h // 2, w // 2, c2 + c1),
                ("p1", h // 4, w // 4, c1), ("a2", h // 4, w // 4, c2),
                ("cat2", h // 4, w // 4, c3 + c2), ("p2", h // 8, w // 8, c2),
                ("b1", h // 8, w // 8, c3), ("b2", h // 8, w // 8, c3),
                ("d2a", h // 4, w // 4, c2), ("d2", h // 4, w // 4, c2),
                ("d1a", h // 2, w // 2, c1), ("d1", h // 2, w // 2, c1),
                ("d0a", h, w, c0)]  # the last activations are not stored (fused head)
        offs, total = [], 0
        for _, hh, ww, c in spec:
            offs.append(total)
            total += (2 * b * hh * ww * c + 255) // 256 * 256
        q_off = total
        total += 4 * b * h * w
        pool = getattr(self, "_pool", None)
        if pool is None or pool.numel() < total:
            # zeroed once: the forward writes every buffer in full before it
            # reads it, so views of an earlier shape's data need no clearing.
            # Recorded forwards point into the old pool: drop them.
            if self._stream is not None:
                raise RuntimeError("the forward pool cannot grow while a forward is recorded")
            self._graphs.clear()
            pool = self._pool = torch.zeros(total, dtype=torch.uint8, device=self.device)
        B = {}
        for (name, hh, ww, c), o in zip(spec, offs):
            n = 2 * b * hh * ww * c
            B[name] = pool[o:o + n].view(torch.bfloat16).view(b, hh, ww, c)
        B["q"] = pool[q_off:q_off + 4 * b * h * w].view(torch.float32).view(b, h, w)
        return B

    # ---- forward ---------------------------------------------------------------
    def _conv(self, layer, x, cs_in, y, cs_out, b, h, w, relu=1):
        self._check(self.L.strm_nn_conv3x3(
            x, cs_in, layer.cin_p, self._wbf(layer), layer.kp, self._ptr(layer.b), y,
            None, cs_out, layer.cout, b, h, w, relu, self._stream), "conv3x3")

    def forward(self, xin, b, h, w, keep: bool = True):
        """xin: BF16 [b][h][w][8] device tensor (see strm_nn_prepare_input).
        Returns the FP32 correction q [b][h][w].  keep=False (prediction
        only, no backward to follow) runs in the shared forward pool: q is
        then valid until the next such call."""
        with self._deferred():
            return self._forward(xin, b, h, w, keep)

    def forward_graphed(self, xin, b, h, w):
        """forward(keep=False) replayed from a CUDA graph, recorded on the
        first call for this input buffer and these sizes: one launch instead
        of some twenty host calls, for predictions on small grids, where the
        host calls take longer than the kernels.  Same kernels, same q
        buffer (valid until the next forward); the tensor-core kernels'
        timeout flag is checked after each replay."""
        import ctypes
        import torch
        key = (xin.data_ptr(), b, h, w)
        rec = self._graphs.get(key)
        if rec is None:
            # a plain run first: sizes the pool and configures the kernels
            self.forward(xin, b, h, w, keep=False)
            torch.cuda.synchronize()
            graph = torch.cuda.CUDAGraph()
            self.L.strm_nn_set_sync(0)
            try:
                with torch.cuda.graph(graph):
                    self._stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
                    q = self._forward(xin, b, h, w, False)
            finally:
                self._stream = None
                self.L.strm_nn_set_sync(1)
            rec = self._graphs[key] = (graph, q)
        graph, q = rec
        graph.replay()
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        self._check(self.L.strm_nn_status(stream), "tensor-core kernels")
        return q

    def _forward(self, xin, b, h, w, keep):
        B = self._buffers(b, h, w) if keep else self._forward_buffers(b, h, w)
        B["x_in_ptr"] = xin.data_ptr()
        L = self.L
        c0, c1, c2, c3 = CHANNELS
        (e0a, e0b), (e1a, e1b), (e2a, e2b) = self.enc
        m1, m2 = self.mid
        (d2a, d2b), (d1a, d1b), (d0a, d0b) = self.dec
        ptr = lambda name: B[name].data_ptr()
        bf2 = 2  # bytes per BF16
        # encoder; each level's output lands in the skip slice of its concat buffer
        self._conv(e0a, xin.data_ptr(), IN_CH, ptr("a0"), c0, b, h, w)
        e0 = ptr("cat0") + bf2 * c1
        self._conv(e0b, ptr("a0"), c0, e0, c1 + c0, b, h, w)
        self._check(L.strm_nn_avgpool(e0, c1 + c0, ptr("p0"), c0, b, h, w, c0, self._stream), "pool")
        h1, w1 = h // 2, w // 2
        self._conv(e1a, ptr("p0"), c0, ptr("a1"), c1, b, h1, w1)
        e1 = ptr("cat1") + bf2 * c2
        self._conv(e1b, ptr("a1"), c1, e1, c2 + c1, b, h1, w1)
        self._check(L.strm_nn_avgpool(e1, c2 + c1, ptr("p1"), c1, b, h1, w1, c1, self._stream), "pool")
        h2, w2 = h // 4, w // 4
        self._conv(e2a, ptr("p1"), c1, ptr("a2"), c2, b, h2, w2)
        e2 = ptr("cat2") + bf2 * c3
        self._conv(e2b, ptr("a2"), c2, e2, c3 + c2, b, h2, w2)
        self._check(L.strm_nn_avgpool(e2, c3 + c2, ptr("p2"), c2, b, h2, w2, c2, self._stream), "pool")
        h3, w3 = h // 8, w // 8
        self._conv(m1, ptr("p2"), c2, ptr("b1"), c3, b, h3, w3)
        self._conv(m2, ptr("b1"), c3, ptr("b2"), c3, b, h3, w3)
        # decoder
        self._check(L.strm_nn_upsample(ptr("b2"), c3, ptr("cat2"), c3 + c2, b, h2, w2, c3, self._stream),
                    "up")
        self._conv(d2a, ptr("cat2"), c3 + c2, ptr("d2a"), c2, b, h2, w2)
        self._conv(d2b, ptr("d2a"), c2, ptr("d2"), c2, b, h2, w2)
        self._check(L.strm_nn_upsample(ptr("d2"), c2, ptr("cat1"), c2 + c1, b, h1, w1, c2, self._stream),
                    "up")
        self._conv(d1a, ptr("cat1"), c2 + c1, ptr("d1a"), c1, b, h1, w1)
        self._conv(d1b, ptr("d1a"), c1, ptr("d1"), c1, b, h1, w1)
        self._check(L.strm_nn_upsample(ptr("d1"), c1, ptr("cat0"), c1 + c0, b, h, w, c1, self._stream),
                    "up")
        self._conv(d0a, ptr("cat0"), c1 + c0, ptr("d0a"), c0, b, h, w)
        # the last convolution with the 1x1 head in its epilogue; its
        # activations are stored only for a backward
        self._check(L.strm_nn_conv3x3_head(
            ptr("d0a"), c0, d0b.cin_p, self._wbf(d0b), d0b.kp, self._ptr(d0b.b),
            ptr("d0") if keep else None, c0, d0b.cout, b, h, w, self._ptr(self.wh),
            self._ptr(self.bh), ptr("q"), self._stream), "conv3x3 + head")
        return B["q"]

    # ---- backward ----------------------------------------------------------------
    def _conv_back(self, layer, x, cs_in, y, cs_y, g, cs_g, gx_slices, b, h, w):
        """Weight/bias gradients of `layer` (input x, ReLU output y, output
        gradient g) and, when gx_slices is given, the data gradient split into
        [(first input channel, count, destination, destination stride)]."""
        L = self.L
        gptr_w = self._ptr(layer.w, self.grad)
        gptr_b = self._ptr(layer.b, self.grad)
        npix = b * h * w
        self._check(L.strm_nn_conv3x3_wgrad(x, cs_in, layer.cin_p, layer.kp, g, cs_g, y, cs_y,
                                            gptr_w, layer.cout, b, h, w, None), "wgrad")
        self._check(L.strm_nn_bias_grad(g, cs_g, y, cs_y, gptr_b, npix, layer.cout, None),
                    "bias grad")
        if not gx_slices:
            return
        gm = self._gm
        self._check(L.strm_nn_relu_mask(g, cs_g, y, cs_y, gm, layer.cout, npix, layer.cout,
                                        None), "mask")
        for (c_first, count, dst, cs_dst) in gx_slices:
            wt = layer.wt_bf.data_ptr() + 2 * c_first * layer.kp_t
            self._check(L.strm_nn_conv3x3(gm, layer.cout, layer.cout, wt, layer.kp_t, None, dst,
                                          None, cs_dst, count, b, h, w, 0, None), "dgrad")

    def backward(self, gq, b, h, w):
        """gq: FP32 [b][h][w] gradient of the loss with respect to the output.
        Accumulates every parameter gradient into self.grad."""
        with self._deferred():
            self._backward(gq, b, h, w)

    def _backward(self, gq, b, h, w):
        B = self._buffers(b, h, w)
        L = self.L
        c0, c1, c2, c3 = CHANNELS
        (e0a, e0b), (e1a, e1b), (e2a, e2b) = self.enc
        m1, m2 = self.mid
        (d2a, d2b), (d1a, d1b), (d0a, d0b) = self.dec
        ptr = lambda name: B[name].data_ptr()
        bf2 = 2
        self._gm = ptr("gm")
        h1, w1, h2, w2, h3, w3 = h // 2, w // 2, h // 4, w // 4, h // 8, w // 8
        self._check(L.strm_nn_head_bwd(ptr("d0"), c0, c0, self._ptr(self.wh), gq.data_ptr(),
                                       ptr("g_d0"), c0, self._ptr(self.wh, self.grad),
                                       self._ptr(self.bh, self.grad), b * h * w, None),
                    "head bwd")
        # level 0 decoder
        self._conv_back(d0b, ptr("d0a"), c0, ptr("d0"), c0, ptr("g_d0"), c0,
                        [(0, c0, ptr("g_d0a"), c0)], b, h, w)
        self._conv_back(d0a, ptr("cat0"), c1 + c0, ptr("d0a"), c0, ptr("g_d0a"), c0,
                        [(0, c1, ptr("g_up0"), c1), (c1, c0, ptr("g_e0"), c0)], b, h, w)
        self._check(L.strm_nn_upsample_bwd(ptr("g_up0"), c1, ptr("g_d1"), c1, b, h, w, c1, None),
                    "up bwd")
        # level 1 decoder
        self._conv_back(d1b, ptr("d1a"), c1, ptr("d1"), c1, ptr("g_d1"), c1,
                        [(0, c1, ptr("g_d1a"), c1)], b, h1, w1)
        self._conv_back(d1a, ptr("cat1"), c2 + c1, ptr("d1a"), c1, ptr("g_d1a"), c1,
                        [(0, c2, ptr("g_up1"), c2), (c2, c1, ptr("g_e1"), c1)], b, h1, w1)
        self._check(L.strm_nn_upsample_bwd(ptr("g_up1"), c2, ptr("g_d2"), c2, b, h1, w1, c2,
                                           None), "up bwd")
        # level 2 decoder
        self._conv_back(d2b, ptr("d2a"), c2, ptr("d2"), c2, ptr("g_d2"), c2,
                        [(0, c2, ptr("g_d2a"), c2)], b, h2, w2)
        self._conv_back(d2a, ptr("cat2"), c3 + c2, ptr("d2a"), c2, ptr("g_d2a"), c2,
                        [(0, c3, ptr("g_up2"), c3), (c3, c2, ptr("g_e2"), c2)], b, h2, w2)
        self._check(L.strm_nn_upsample_bwd(ptr("g_up2"), c3, ptr("g_b2"), c3, b, h2, w2, c3,
                                           None), "up bwd")
        # bottleneck
        self._conv_back(m2, ptr("b1"), c3, ptr("b2"), c3, ptr("g_b2"), c3,
                        [(0, c3, ptr("g_b1"), c3)], b, h3, w3)
        self._conv_back(m1, ptr("p2"), c2, ptr("b1"), c3, ptr("g_b1"), c3,
                        [(0, c2, ptr("g_p2"), c2)], b, h3, w3)
        # encoder level 2: the pooled path adds to the skip gradient
        self._check(L.strm_nn_avgpool_bwd(ptr("g_p2"), c2, ptr("g_e2"), c2, b, h2, w2, c2, 1,
                                          None), "pool bwd")
        e2 = ptr("cat2") + bf2 * c3
        self._conv_back(e2b, ptr("a2"), c2, e2, c3 + c2, ptr("g_e2"), c2,
                        [(0, c2, ptr("g_a2"), c2)], b, h2, w2)
        self._conv_back(e2a, ptr("p1"), c1, ptr("a2"), c2, ptr("g_a2"), c2,
                        [(0, c1, ptr("g_p1"), c1)], b, h2, w2)
        self._check(L.strm_nn_avgpool_bwd(ptr("g_p1"), c1, ptr("g_e1"), c1, b, h1, w1, c1, 1,
                                          None), "pool bwd")
        e1 = ptr("cat1") + bf2 * c2
        self._conv_back(e1b, ptr("a1"), c1, e1, c2 + c1, ptr("g_e1"), c1,
                        [(0, c1, ptr("g_a1"), c1)], b, h1, w1)
        self._conv_back(e1a, ptr("p0"), c0, ptr("a1"), c1, ptr("g_a1"), c1,
                        [(0, c0, ptr("g_p0"), c0)], b, h1, w1)
        self._check(L.strm_nn_avgpool_bwd(ptr("g_p0"), c0, ptr("g_e0"), c0, b, h, w, c0, 1,
                                          None), "pool bwd")
        e0 = ptr("cat0") + bf2 * c1
        self._conv_back(e0b, ptr("a0"), c0, e0, c1 + c0, ptr("g_e0"), c0,
                        [(0, c0, ptr("g_a0"), c0)], b, h, w)
        self._conv_back(e0a, B["x_in_ptr"], IN_CH, ptr("a0"), c0, ptr("g_a0"), c0, None, b, h, w)

    # ---- optimisation ----------------------------------------------------------
    def zero_grad(self):
        self._check(self.L.strm_nn_zero(self.grad.data_ptr(), 4 * self.n_params, None), "zero")

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step += 1
        self._check(self.L.strm_nn_adam(self.theta.data_ptr(), self.grad.data_ptr(),
                                        self.m.data_ptr(), self.v.data_ptr(), self.n_params,
                                        lr, b1, b2, eps, self.step, self.theta_bf.data_ptr(),
                                        None), "adam")
        self._flip()

    # ---- persistence -------------------------------------------------------------
    def state_dict(self):
        return {"theta": self.theta.detach().cpu().numpy().copy(), "step": self.step}

    def load_state_dict(self, d):
        import torch
        self.theta.copy_(torch.tensor(d["theta"], device=self.device))
        self.step = int(d.get("step", 0))
        self._mirror()
