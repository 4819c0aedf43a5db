"""tcgen05 BF16 contractions of the learned warm start against torch (FP32
reference of the same products)."""
import ctypes

import pytest

from stroemung_gb300 import _lib

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (256, 128, 256), (384, 256, 576)])
def test_gemm_bf16_matches_torch(m, n, k):
    import torch
    L = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(m + n + k)
    a = torch.randn(m, k, device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn(n, k, device="cuda", generator=g).to(torch.bfloat16)
    d = torch.empty(m, n, device="cuda", dtype=torch.float32)
    torch.cuda.synchronize()
    rc = L.strm_nn_gemm_bf16(ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()),
                             ctypes.cast(d.data_ptr(), ctypes.POINTER(ctypes.c_float)),
                             m, n, k, None)
    assert rc == 0
    ref = a.float() @ b.float().T
    err = (d - ref).abs().max().item()
    assert err <= 1e-3 * max(1.0, ref.abs().max().item()), err


def _bf(t):
    return t.to(__import__("torch").bfloat16)


def _pack_weights(w, cin_p):
    """torch [cout, cin, 3, 3] -> [cout, kp] with K = tap*cin_p + ci, tap = ky*3 + kx."""
    import torch
    cout, cin = w.shape[:2]
    kp = -(-9 * cin_p // 64) * 64
    out = torch.zeros(cout, kp, dtype=w.dtype, device=w.device)
    for ky in range(3):
        for kx in range(3):
            t = ky * 3 + kx
            out[:, t * cin_p:t * cin_p + cin] = w[:, :, ky, kx]
    return out, kp


def _nhwc(x, cin_p):
    import torch
    b, c, h, w = x.shape
    out = torch.zeros(b, h, w, cin_p, dtype=x.dtype, device=x.device)
    out[..., :c] = x.permute(0, 2, 3, 1)
    return out.contiguous()


# the odd sizes leave partial pixel tiles and image rows (the gathering
# kernel); widths that are multiples of 128 with inputs in slices of 32 or 64
# channels, or of 8 (inputs of up to 8 channels), take the TMA-staged kernel
# (64-byte swizzled rows for 32-channel slices, 128-byte for 64, unswizzled
# 16-byte pixels for 8)
@pytest.mark.parametrize("cin,cout,h,w,relu", [(3, 32, 16, 128, 1), (32, 64, 8, 64, 1),
                                                (96, 32, 16, 32, 0), (128, 256, 4, 64, 1),
                                                (64, 16, 8, 16, 1), (32, 32, 7, 200, 1),
                                                (64, 64, 5, 300, 0), (8, 32, 3, 130, 1),
                                                (48, 32, 9, 140, 1), (96, 32, 4, 256, 1),
                                                (32, 32, 5, 128, 1), (64, 64, 3, 256, 0),
                                                (128, 128, 2, 128, 1), (256, 256, 2, 128, 1),
                                                (192, 64, 2, 128, 1), (64, 16, 3, 128, 1),
                                                (32, 256, 3, 128, 0), (384, 128, 1, 128, 0),
                                                (8, 32, 4, 256, 1), (8, 64, 3, 128, 0),
                                                (5, 16, 2, 384, 1), (8, 256, 2, 128, 1),
                                                (8, 128, 3, 256, 1)])
def test_conv3x3_forward_matches_torch(cin, cout, h, w, relu):
    import torch
    import torch.nn.functional as F
    L = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(cin * 7 + cout)
    b = 2
    cin_p = -(-cin // 8) * 8
    x = _bf(torch.randn(b, cin, h, w, device="cuda", generator=g))
    wt = _bf(torch.randn(cout, cin, 3, 3, device="cuda", generator=g) * 0.2)
    bias = torch.randn(cout, device="cuda", generator=g)
    wp, kp = _pack_weights(wt, cin_p)
    xn = _nhwc(x, cin_p)
    y = torch.empty(b, h, w, cout, device="cuda", dtype=torch.bfloat16)
    torch.cuda.synchronize()
    rc = L.strm_nn_conv3x3(xn.data_ptr(), cin_p, cin_p, wp.data_ptr(), kp, bias.data_ptr(),
                           y.data_ptr(), None, cout, cout, b, h, w, relu, None)
    assert rc == 0
    ref = F.conv2d(x.float(), wt.float(), bias, padding=1)
    if relu:
        ref = ref.clamp_min(0)
    ref = ref.permute(0, 2, 3, 1)
    err = (y.float() - ref).abs().max().item()
    assert err <= 1e-2 * max(1.0, ref.abs().max().item()), err


@pytest.mark.parametrize("cin,cout,h,w", [(32, 32, 16, 64), (64, 128, 8, 32), (16, 16, 16, 16),
                                          (32, 32, 8, 128), (64, 32, 4, 128)])
def test_conv3x3_weight_and_data_gradients_match_torch(cin, cout, h, w):
    import torch
    import torch.nn.functional as F
    L = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(cin + 3 * cout)
    b = 2
    cin_p = cin
    x = _bf(torch.randn(b, cin, h, w, device="cuda", generator=g))
    wt = _bf(torch.randn(cout, cin, 3, 3, device="cuda", generator=g) * 0.2)
    gy = _bf(torch.randn(b, cout, h, w, device="cuda", generator=g))
    # forward with ReLU to get the mask
    wp, kp = _pack_weights(wt, cin_p)
    xn = _nhwc(x, cin_p)
    y = torch.empty(b, h, w, cout, device="cuda", dtype=torch.bfloat16)
    assert L.strm_nn_conv3x3(xn.data_ptr(), cin_p, cin_p, wp.data_ptr(), kp, None, y.data_ptr(),
                             None, cout, cout, b, h, w, 1, None) == 0
    gyn = gy.permute(0, 2, 3, 1).contiguous()
    dw = torch.zeros(cout, kp, device="cuda", dtype=torch.float32)
    assert L.strm_nn_conv3x3_wgrad(xn.data_ptr(), cin_p, cin_p, kp, gyn.data_ptr(), cout,
                                   y.data_ptr(), cout, dw.data_ptr(), cout, b, h, w, None) == 0
    # torch reference of the same masked gradient
    mask = (y.float() > 0).permute(0, 3, 1, 2)
    gm = gy.float() * mask
    xr = x.float().requires_grad_(True)
    wr = wt.float().requires_grad_(True)
    out = F.conv2d(xr, wr, padding=1)
    (out * gm).sum().backward()
    ref_w, _ = _pack_weights(wr.grad, cin_p)
    err = (dw - ref_w).abs().max().item()
    assert err <= 2e-3 * max(1.0, ref_w.abs().max().item()), err
    # data gradient: conv of the masked gradient with flipped weights
    gmn = torch.empty(b, h, w, cout, device="cuda", dtype=torch.bfloat16)
    assert L.strm_nn_relu_mask(gyn.data_ptr(), cout, y.data_ptr(), cout, gmn.data_ptr(), cout,
                               b * h * w, cout, None) == 0
    kp_t = -(-9 * cout // 64) * 64
    wflip = torch.zeros(cin_p, kp_t, device="cuda", dtype=torch.bfloat16)
    assert L.strm_nn_flip_weights(wp.data_ptr(), cout, cin_p, kp, wflip.data_ptr(), cout, kp_t,
                                  None) == 0
    dx = torch.empty(b, h, w, cin_p, device="cuda", dtype=torch.bfloat16)
    assert L.strm_nn_conv3x3(gmn.data_ptr(), cout, cout, wflip.data_ptr(), kp_t, None,
                             dx.data_ptr(), None, cin_p, cin_p, b, h, w, 0, None) == 0
    torch.cuda.synchronize()
    ref_x = xr.grad.permute(0, 2, 3, 1)
    err = (dx.float() - ref_x).abs().max().item()
    assert err <= 1e-2 * max(1.0, ref_x.abs().max().item()), err


def test_deferred_waits_give_the_same_result():
    """strm_nn_set_sync(0): the convolution returns after its launch, the
    result equals the waiting call's, and strm_nn_status reports no
    timeout."""
    import torch
    L = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(5)
    cin, cout, h, w = 32, 64, 16, 96
    x = _bf(torch.randn(1, cin, h, w, device="cuda", generator=g))
    wt = _bf(torch.randn(cout, cin, 3, 3, device="cuda", generator=g) * 0.2)
    wp, kp = _pack_weights(wt, cin)
    xn = _nhwc(x, cin)
    y1 = torch.empty(1, h, w, cout, device="cuda", dtype=torch.bfloat16)
    y2 = torch.empty_like(y1)
    torch.cuda.synchronize()
    assert L.strm_nn_conv3x3(xn.data_ptr(), cin, cin, wp.data_ptr(), kp, None, y1.data_ptr(),
                             None, cout, cout, 1, h, w, 1, None) == 0
    assert L.strm_nn_set_sync(0) == 0
    try:
        assert L.strm_nn_conv3x3(xn.data_ptr(), cin, cin, wp.data_ptr(), kp, None,
                                 y2.data_ptr(), None, cout, cout, 1, h, w, 1, None) == 0
    finally:
        L.strm_nn_set_sync(1)
    assert L.strm_nn_status(None) == 0
    assert torch.equal(y1, y2)


@pytest.mark.parametrize("use_slice", [False, True], ids=["whole", "channel_slice"])
def test_tma_staged_forward_matches_the_gathering_kernel(use_slice):
    """The same convolution with TMA-staged operands and with gathered ones
    (strm_nn_set_conv_tma 1 / 0): both within BF16 rounding of torch and of
    each other; with use_slice the input is channels 32..95 of a 96-channel
    buffer (the decoder's concatenations read such slices)."""
    import torch
    import torch.nn.functional as F
    L = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(11)
    b, cin, cout, h, w = 2, 64, 64, 6, 256
    x = _bf(torch.randn(b, cin, h, w, device="cuda", generator=g))
    wt = _bf(torch.randn(cout, cin, 3, 3, device="cuda", generator=g) * 0.2)
    bias = torch.randn(cout, device="cuda", generator=g)
    wp, kp = _pack_weights(wt, cin)
    if use_slice:
        buf = torch.zeros(b, h, w, 96, dtype=torch.bfloat16, device="cuda")
        buf[..., 32:] = x.permute(0, 2, 3, 1)
        xptr, cs_in = buf.data_ptr() + 32 * 2, 96
    else:
        xn = _nhwc(x, cin)
        xptr, cs_in = xn.data_ptr(), cin
    outs = []
    try:
        for use in (1, 0):
            assert L.strm_nn_set_conv_tma(use) == 0
            y = torch.empty(b, h, w, cout, device="cuda", dtype=torch.bfloat16)
            torch.cuda.synchronize()
            assert L.strm_nn_conv3x3(xptr, cs_in, cin, wp.data_ptr(), kp, bias.data_ptr(),
                                     y.data_ptr(), None, cout, cout, b, h, w, 1, None) == 0
            outs.append(y.float())
    finally:
        L.strm_nn_set_conv_tma(1)
    ref = F.conv2d(x.float(), wt.float(), bias, padding=1).clamp_min(0).permute(0, 2, 3, 1)
    scale = max(1.0, ref.abs().max().item())
    for y in outs:
        assert (y - ref).abs().max().item() <= 1e-2 * scale
    assert (outs[0] - outs[1]).abs().max().item() <= 1e-2 * scale


@pytest.mark.parametrize("cin,cout", [(32, 32), (64, 64), (96, 32), (128, 128), (128, 256),
                                      (8, 32)])
def test_tma_forward_is_independent_of_its_launch_shape(cin, cout):
    """The TMA-fed forward gives the same bits for any launch shape — one,
    several or all tiles per CTA, any number of CTAs per SM and ring depth
    (each tile's K loop runs in one fixed order), including rings shallower
    than a tile's K chunks and more CTAs per SM than TMEM holds — for row
    boxes (three taps per box) and for one box per tap alike; both agree
    with torch within BF16 rounding.  The width leaves a tile at each image
    border, whose boxes reach one pixel outside the image."""
    import torch
    import torch.nn.functional as F
    L = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(5)
    b, h, w = 1, 7, 384
    x = _bf(torch.randn(b, cin, h, w, device="cuda", generator=g))
    wt = _bf(torch.randn(cout, cin, 3, 3, device="cuda", generator=g) * 0.1)
    bias = torch.randn(cout, device="cuda", generator=g)
    wp, kp = _pack_weights(wt, cin)
    xn = _nhwc(x, cin)
    ref = F.conv2d(x.float(), wt.float(), bias, padding=1).clamp_min(0).permute(0, 2, 3, 1)
    scale = max(1.0, ref.abs().max().item())
    shapes = ((0, 0, 0), (0, 0, 1), (1, 2, 64), (1, 32, 64), (2, 3, 7), (4, 0, 4),
              (8, 5, 3), (3, 6, 1), (1, 2, 1), (8, 2, 1), (0, 0, 2), (3, 2, 5))
    try:
        for rows in (1, 0):
            outs = []
            for ctas, stages, tiles in shapes:
                assert L.strm_nn_tune_conv_tma(ctas, stages, tiles, rows) == 0
                y = torch.empty(b, h, w, cout, device="cuda", dtype=torch.bfloat16)
                assert L.strm_nn_conv3x3(xn.data_ptr(), cin, cin, wp.data_ptr(), kp,
                                         bias.data_ptr(), y.data_ptr(), None, cout, cout, b, h,
                                         w, 1, None) == 0
                outs.append(y)
            for y in outs[1:]:
                assert torch.equal(y, outs[0]), rows
            assert (outs[0].float() - ref).abs().max().item() <= 1e-2 * scale, rows
    finally:
        L.strm_nn_tune_conv_tma(0, 0, 0, 1)


@pytest.mark.parametrize("b,h,w,c,cs_in,cs_out", [(1, 8, 12, 64, 64, 96), (2, 6, 4, 32, 96, 32),
                                                  (3, 4, 6, 8, 8, 8), (1, 2, 2, 16, 16, 16),
                                                  (2, 10, 6, 6, 6, 6)])
def test_avgpool_and_upsample_match_exact_references(b, h, w, c, cs_in, cs_out):
    """Average pooling and nearest upsampling on NHWC buffers with pixel
    strides (channel slices of concatenations): the pooled value is
    0.25 * (((a + b) + c) + d) in FP32 rounded to BF16, the upsampled one a
    copy; bit-exact, for the 16-byte row kernels and (c = 6, odd strides)
    the element kernels."""
    import torch
    L = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn(b, h, w, cs_in, device="cuda", generator=g).to(torch.bfloat16)
    # pooling: input h x w -> h/2 x w/2
    out = torch.full((b, h // 2, w // 2, cs_out), 7.0, device="cuda", dtype=torch.bfloat16)
    assert L.strm_nn_avgpool(x.data_ptr(), cs_in, out.data_ptr(), cs_out, b, h, w, c, None) == 0
    torch.cuda.synchronize()
    xf = x[..., :c].float()
    a, bb = xf[:, 0::2, 0::2], xf[:, 0::2, 1::2]
    cc, d = xf[:, 1::2, 0::2], xf[:, 1::2, 1::2]
    ref = (0.25 * (((a + bb) + cc) + d)).to(torch.bfloat16)
    assert torch.equal(out[..., :c], ref)
    assert bool((out[..., c:] == 7.0).all())  # channels beyond c untouched
    # upsampling: input h/2 x w/2 -> h x w
    lo = x[:, : h // 2, : w // 2].contiguous()
    up = torch.full((b, h, w, cs_out), 7.0, device="cuda", dtype=torch.bfloat16)
    assert L.strm_nn_upsample(lo.data_ptr(), cs_in, up.data_ptr(), cs_out, b, h, w, c,
                              None) == 0
    torch.cuda.synchronize()
    ref = lo[..., :c].repeat_interleave(2, dim=1).repeat_interleave(2, dim=2)
    assert torch.equal(up[..., :c], ref)
    assert bool((up[..., c:] == 7.0).all())


@pytest.mark.parametrize("cin,cout,h,w", [(32, 32, 3, 256), (64, 64, 2, 128), (8, 32, 3, 128),
                                          (32, 32, 5, 200), (96, 32, 2, 384)])
def test_conv_with_fused_head_equals_conv_then_head(cin, cout, h, w):
    """strm_nn_conv3x3_head gives the activations and the head output of
    strm_nn_conv3x3 (ReLU) followed by strm_nn_head bit for bit, on the
    TMA-fed kernel (widths of whole 128-pixel tiles) and on the gathering
    one (w = 200), with and without storing the activations."""
    import torch
    L = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(cin + 3 * cout + w)
    b = 2
    x = _bf(torch.randn(b, cin, h, w, device="cuda", generator=g))
    wt = _bf(torch.randn(cout, cin, 3, 3, device="cuda", generator=g) * 0.2)
    bias = torch.randn(cout, device="cuda", generator=g)
    wh = torch.randn(cout, device="cuda", generator=g)
    bh = torch.randn(1, device="cuda", generator=g)
    wp, kp = _pack_weights(wt, cin)
    xn = _nhwc(x, cin)
    y1 = torch.empty(b, h, w, cout, device="cuda", dtype=torch.bfloat16)
    q1 = torch.empty(b, h, w, device="cuda")
    assert L.strm_nn_conv3x3(xn.data_ptr(), cin, cin, wp.data_ptr(), kp, bias.data_ptr(),
                             y1.data_ptr(), None, cout, cout, b, h, w, 1, None) == 0
    assert L.strm_nn_head(y1.data_ptr(), cout, cout, wh.data_ptr(), bh.data_ptr(), q1.data_ptr(),
                          b * h * w, None) == 0
    y2 = torch.empty_like(y1)
    q2 = torch.empty_like(q1)
    q3 = torch.empty_like(q1)
    assert L.strm_nn_conv3x3_head(xn.data_ptr(), cin, cin, wp.data_ptr(), kp, bias.data_ptr(),
                                  y2.data_ptr(), cout, cout, b, h, w, wh.data_ptr(),
                                  bh.data_ptr(), q2.data_ptr(), None) == 0
    assert L.strm_nn_conv3x3_head(xn.data_ptr(), cin, cin, wp.data_ptr(), kp, bias.data_ptr(),
                                  None, cout, cout, b, h, w, wh.data_ptr(), bh.data_ptr(),
                                  q3.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert torch.equal(y2, y1)
    assert torch.equal(q2, q1) and torch.equal(q3, q1)
