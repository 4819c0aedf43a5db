"""Test infrastructure: torch-CPU FP32 restatement of the learned warm
start's network, input assembly and loss, for checking the library's
tcgen05 forward / backward kernels and its Adam step.  Not part of the
product; only tests import it.

Parity is unpinned by the reference (the Rust crate has no learned part);
this oracle restates the method itself:

* input (8 channels per interior cell): rhs/s, fluid mask, (p_prev - mean)
  /(s dx^2), five zeros, with s = max |rhs| over fluid cells and the mean of
  p_prev over fluid cells, stored as BF16;
* network: 4 levels of two 3x3 convolutions (zero padding) + ReLU with
  32/64/128/256 channels, 2x2 average pooling down, nearest upsampling up,
  the upsampled tensor concatenated before the skip, a 1x1 FP32 head.
  Weights are used as BF16 copies of the FP32 masters, activations are
  stored as BF16, products accumulate in FP32 — the same rounding points as
  the kernels (the rounding counts as identity for the gradients);
* loss: the corrected pressure p = p_prev + s dx^2 q on fluid cells, the
  solver's boundary copy (src/grid/mod.rs:343-412: one fluid neighbour, or
  the mean of two at a corner), r = 5-point Laplacian of p - rhs on fluid
  cells; loss = mean over samples of sum r^2 / sum rhs^2.

Parameters are one flat FP32 vector in this order: for each convolution
(encoder levels 0-2, the two bottleneck convolutions, decoder levels 2-0;
two per level) its weights [cout][kp] (K = tap * cin_p + channel, tap =
ky * 3 + kx, cin_p = cin rounded up to 8, kp = 9 cin_p rounded up to 64)
then its bias [cout]; then the head weights [32] and bias [1].
"""
from __future__ import annotations

import numpy as np

CHANNELS = (32, 64, 128, 256)
IN_CH = 8

# edge codes of the flag byte (kind in bits 0-2, edge in bits 3-6)
E_N, E_NE, E_E, E_SE, E_S, E_SW, E_W, E_NW = range(1, 9)


def conv_shapes():
    c0, c1, c2, c3 = CHANNELS
    pairs = [(IN_CH, c0), (c0, c0), (c0, c1), (c1, c1), (c1, c2), (c2, c2), (c2, c3), (c3, c3),
             (c3 + c2, c2), (c2, c2), (c2 + c1, c1), (c1, c1), (c1 + c0, c0), (c0, c0)]
    return pairs


def _kp(cin_p):
    return -(-9 * cin_p // 64) * 64


def unpack(theta):
    """Flat parameter vector -> ([(weight [cout, cin, 3, 3], bias)], wh, bh) as torch tensors."""
    import torch
    theta = torch.as_tensor(np.asarray(theta, np.float32))
    convs = []
    o = 0
    for cin, cout in conv_shapes():
        cin_p = -(-cin // 8) * 8
        kp = _kp(cin_p)
        w = theta[o:o + cout * kp].reshape(cout, kp)
        o += cout * kp
        b = theta[o:o + cout]
        o += cout
        wt = torch.stack([w[:, t * cin_p:t * cin_p + cin] for t in range(9)], dim=-1)
        convs.append((wt.reshape(cout, cin, 3, 3), b))
    wh = theta[o:o + CHANNELS[0]]
    o += CHANNELS[0]
    bh = theta[o:o + 1]
    o += 1
    assert o == theta.numel(), (o, theta.numel())
    return convs, wh, bh


def pack_grads(grads_convs, g_wh, g_bh):
    """Inverse layout of `unpack` for gradients (padding entries 0)."""
    out = []
    for (cin, cout), (gw, gb) in zip(conv_shapes(), grads_convs):
        cin_p = -(-cin // 8) * 8
        kp = _kp(cin_p)
        w = np.zeros((cout, kp), np.float32)
        gw = gw.detach().numpy()
        for ky in range(3):
            for kx in range(3):
                t = ky * 3 + kx
                w[:, t * cin_p:t * cin_p + cin] = gw[:, :, ky, kx]
        out += [w.ravel(), gb.detach().numpy().ravel()]
    out += [g_wh.detach().numpy().ravel(), g_bh.detach().numpy().ravel()]
    return np.concatenate(out)


_EMULATE_BF16 = [True]


def _bf(t):
    import torch
    if not _EMULATE_BF16[0]:
        return t
    return t.to(torch.bfloat16).to(torch.float32)


def _round_grad(t):
    """Identity forward; rounds the gradient arriving here to BF16 (the
    kernels store every activation gradient as BF16)."""
    import torch

    class _R(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x):
            return x.view_as(x)

        @staticmethod
        def backward(ctx, g):
            return _bf(g)

    return _R.apply(t)


def prepare_input(rhs, flags, pprev, dx2):
    """Planes [b][nx][ny] (numpy) -> (xin [b][h][w][8] float32 holding BF16 values, s, mean)."""
    import torch
    rhs = torch.as_tensor(np.asarray(rhs, np.float32))
    pprev = torch.as_tensor(np.asarray(pprev, np.float32))
    fl = torch.as_tensor(np.asarray(flags, np.uint8)).to(torch.int32)
    fluid = (fl & 7) == 0
    b = rhs.shape[0]
    s = torch.where(fluid, rhs.abs(), torch.zeros_like(rhs)).reshape(b, -1).max(dim=1).values
    s = torch.where(s > 0, s, torch.ones_like(s))
    cnt = fluid.reshape(b, -1).sum(dim=1).float()
    mean = torch.where(fluid, pprev, torch.zeros_like(pprev)).reshape(b, -1).sum(dim=1) / \
        cnt.clamp_min(1.0)
    sl = (slice(None), slice(1, -1), slice(1, -1))
    fi = fluid[sl]
    x = torch.zeros(b, rhs.shape[1] - 2, rhs.shape[2] - 2, IN_CH)
    x[..., 0] = torch.where(fi, rhs[sl] / s[:, None, None], 0.0)
    x[..., 1] = fi.float()
    x[..., 2] = torch.where(fi, (pprev[sl] - mean[:, None, None]) / (s[:, None, None] * dx2), 0.0)
    return _bf(x), s, mean


def forward(params, xin):
    """xin [b][h][w][8] -> q [b][h][w] (torch, differentiable in params)."""
    import torch
    import torch.nn.functional as F
    convs, wh, bh = params
    x = xin.permute(0, 3, 1, 2)

    def conv(i, t):
        w, b = convs[i]
        return _round_grad(_bf(F.conv2d(t, _bf(w), b, padding=1).clamp_min(0.0)))

    def pool(t):
        return _round_grad(_bf(F.avg_pool2d(t, 2)))

    def up(t):
        return _round_grad(F.interpolate(t, scale_factor=2, mode="nearest"))

    e0 = conv(1, conv(0, x))
    e1 = conv(3, conv(2, pool(e0)))
    e2 = conv(5, conv(4, pool(e1)))
    m = conv(7, conv(6, pool(e2)))
    d2 = conv(9, conv(8, torch.cat([up(m), e2], 1)))
    d1 = conv(11, conv(10, torch.cat([up(d2), e1], 1)))
    d0 = conv(13, conv(12, torch.cat([up(d1), e0], 1)))
    q = torch.einsum("bchw,c->bhw", d0, wh) + bh
    return q


def _shift(p, dx, dy):
    """out[x, y] = p[x + dx, y + dy] (zero outside)."""
    import torch
    out = torch.zeros_like(p)
    nx, ny = p.shape[1], p.shape[2]
    xs = slice(max(0, -dx), nx - max(0, dx))
    ys = slice(max(0, -dy), ny - max(0, dy))
    xd = slice(max(0, dx), nx - max(0, -dx))
    yd = slice(max(0, dy), ny - max(0, -dy))
    out[:, xs, ys] = p[:, xd, yd]
    return out


def boundary_copy(p, flags):
    """The solver's copy of fluid pressure onto boundary cells with an edge
    (north = y - 1, east = x + 1)."""
    import torch
    fl = torch.as_tensor(np.asarray(flags, np.uint8)).to(torch.int32)
    bnd = (fl & 7) != 0
    edge = (fl >> 3) & 15
    pn, ps = _shift(p, 0, -1), _shift(p, 0, 1)
    pe, pw = _shift(p, 1, 0), _shift(p, -1, 0)
    val = {E_N: pn, E_E: pe, E_S: ps, E_W: pw, E_NE: (pn + pe) * 0.5, E_SE: (ps + pe) * 0.5,
           E_SW: (ps + pw) * 0.5, E_NW: (pn + pw) * 0.5}
    out = p
    for e, v in val.items():
        out = torch.where(bnd & (edge == e), v, out)
    return out


def loss(q, rhs, flags, pprev, s, dx2, rdx2, rdy2):
    """Mean over samples of sum r^2 / sum rhs^2 (fluid cells) and the per-sample values."""
    import torch
    rhs = torch.as_tensor(np.asarray(rhs, np.float32))
    pprev = torch.as_tensor(np.asarray(pprev, np.float32))
    fl = torch.as_tensor(np.asarray(flags, np.uint8)).to(torch.int32)
    fluid = (fl & 7) == 0
    b, nx, ny = rhs.shape
    qf = torch.nn.functional.pad(q, (1, 1, 1, 1))
    p = torch.where(fluid, pprev + (s * dx2)[:, None, None] * qf, pprev)
    p = boundary_copy(p, flags)
    lap = (_shift(p, 1, 0) + _shift(p, -1, 0) - 2.0 * p) * rdx2 + \
        (_shift(p, 0, 1) + _shift(p, 0, -1) - 2.0 * p) * rdy2
    r = torch.where(fluid, lap - rhs, torch.zeros_like(rhs))
    b2 = torch.where(fluid, rhs * rhs, torch.zeros_like(rhs)).reshape(b, -1).sum(dim=1)
    per = (r * r).reshape(b, -1).sum(dim=1) / b2.clamp_min(1e-30)
    return per.mean(), per


def loss_and_grads(theta, rhs, flags, pprev, dx, dy, bf16=True):
    """Forward + loss + autograd: (loss, per-sample, q, flat gradient).
    bf16=False runs the same network in plain FP32 (no rounding points):
    the difference between the two measures the BF16 noise of a layer's
    gradient."""
    _EMULATE_BF16[0] = bool(bf16)
    try:
        return _loss_and_grads(theta, rhs, flags, pprev, dx, dy)
    finally:
        _EMULATE_BF16[0] = True


def _loss_and_grads(theta, rhs, flags, pprev, dx, dy):
    import torch
    convs, wh, bh = unpack(theta)
    # unpack returns views into one tensor; make them independent leaves
    convs = [(w.detach().clone().requires_grad_(True), b.detach().clone().requires_grad_(True))
             for w, b in convs]
    wh = wh.detach().clone().requires_grad_(True)
    bh = bh.detach().clone().requires_grad_(True)
    dx2 = dx * dx
    xin, s, _ = prepare_input(rhs, flags, pprev, dx2)
    q = forward((convs, wh, bh), xin)
    L, per = loss(q, rhs, flags, pprev, s, dx2, 1.0 / (dx * dx), 1.0 / (dy * dy))
    L.backward()
    grads = pack_grads([(w.grad, b.grad) for w, b in convs], wh.grad, bh.grad)
    return float(L.detach()), per.detach().numpy(), q.detach().numpy(), grads


def adam(theta, grad, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba 2015), every operation in float32 with the
    hyper-parameters rounded to float32 first; returns new (theta, m, v)."""
    f = np.float32
    theta, grad, m, v = (np.asarray(a, f) for a in (theta, grad, m, v))
    b1, b2, lr, eps = f(b1), f(b2), f(lr), f(eps)
    one = f(1.0)
    m = b1 * m + (one - b1) * grad
    v = b2 * v + ((one - b2) * grad) * grad
    c1 = one - b1 ** f(step)
    c2 = one - b2 ** f(step)
    theta = theta - lr * (m / c1) / (np.sqrt(v / c2) + eps)
    return theta.astype(f), m, v
