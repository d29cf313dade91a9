"""The tensor-core (tcgen05 + TMA) form of the surrogate's 3x3x3 convolution
against a PyTorch FP32 conv3d on the same BF16-rounded inputs, and against
the warp-level mma.sync form: forward with bias / ReLU / mask, channel slices
of wider tensors, the data gradient (mirrored taps), grids that are not
multiples of the 16 x 8 voxel tile."""

import ctypes as C

import pytest
import torch
import torch.nn.functional as F

from test_gpu_unet import _bf, _cl, _close, _from_cl, _torch_w

pytestmark = pytest.mark.gpu


def _conv(entry, B, X, Y, Z, cin, cout, xin, in_stride, in_off, Wb, bias, relu, out, out_stride, out_off,
          mask=None, mask_stride=0, mask_off=0, mirror=0, wpack=None):
    import _native as N
    import kern

    a = N.gm_conv_args()
    a.grid[:] = [B, X, Y, Z]
    a.cin, a.cout = cin, cout
    a.in_, a.in_stride, a.in_off = xin.data_ptr(), in_stride, in_off
    a.w = Wb.data_ptr()
    a.bias = bias.data_ptr() if bias is not None else None
    a.relu, a.mirror = relu, mirror
    if mask is not None:
        a.mask, a.mask_stride, a.mask_off = mask.data_ptr(), mask_stride, mask_off
    a.out, a.out_stride, a.out_off = out.data_ptr(), out_stride, out_off
    if wpack is not None:
        a.wpack = wpack.data_ptr()
    rc = getattr(N.lib(), entry)(C.byref(a), kern.stream_ptr())
    torch.cuda.synchronize()
    return rc, a


@pytest.mark.parametrize("cin,cout,grid", [(16, 16, (1, 16, 8, 1)), (16, 32, (2, 12, 8, 6)), (32, 64, (1, 20, 10, 3)),
                                           (64, 128, (2, 16, 16, 4)), (192, 64, (1, 24, 8, 2)),
                                           (96, 32, (1, 17, 9, 3)), (128, 128, (1, 32, 16, 2))])
def test_conv3_tc_forward(cin, cout, grid):
    import _native as N

    torch.manual_seed(3)
    B, X, Y, Z = grid
    x = _bf(torch.randn(B, cin, Z, Y, X, device="cuda"))
    W = _bf(torch.randn(27, cout, cin, device="cuda") * 0.1)
    b = torch.randn(cout, device="cuda")
    ref = F.relu(F.conv3d(x, _torch_w(W), b, padding=1))
    xin = _cl(x)
    Wb = W.to(torch.bfloat16).contiguous()
    V = B * X * Y * Z
    outs = {}
    wp = torch.full((27 * cin * cout,), float("nan"), dtype=torch.bfloat16, device="cuda")
    for entry, wpack in (("gm_unet_conv3_tc", None), ("gm_unet_conv3_tc", wp), ("gm_unet_conv3_mma", None)):
        out = torch.full((V, cout), float("nan"), dtype=torch.bfloat16, device="cuda")
        rc, a = _conv(entry, B, X, Y, Z, cin, cout, xin, cin, 0, Wb, b, 1, out, cout, 0, wpack=wpack)
        assert rc == N.GM_OK, entry
        key = entry + ("+wpack" if wpack is not None else "")
        outs[key] = _from_cl(out, B, cout, Z, Y, X)
        _close(outs[key], ref, 1e-2)
    # the weight tiles by bulk copies of the prepacked layout or by tensor copies of 16-byte rows: same bits
    assert torch.equal(outs["gm_unet_conv3_tc"], outs["gm_unet_conv3_tc+wpack"])
    assert N.lib().gm_unet_conv3_tc_eligible(C.byref(a)) == 1
    assert N.lib().gm_unet_tc_status() == 0
    # the two tensor-core forms sum in different orders: agreement to BF16 rounding
    _close(outs["gm_unet_conv3_tc"], outs["gm_unet_conv3_mma"], 1e-2)


def test_conv3_tc_slices_mask_and_data_gradient():
    """Input and output as channel slices of wider tensors, a mask slice, and
    the mirrored-tap data gradient."""
    import _native as N

    torch.manual_seed(4)
    B, X, Y, Z, cin, cout = 1, 16, 16, 4, 32, 64
    x = _bf(torch.randn(B, cin, Z, Y, X, device="cuda"))
    W = _bf(torch.randn(27, cout, cin, device="cuda") * 0.1)
    V = B * X * Y * Z
    wide_in = torch.zeros(V, 48 + cin, dtype=torch.bfloat16, device="cuda")
    wide_in[:, 48:] = _cl(x)
    m = (torch.rand(V, cout, device="cuda") > 0.3).to(torch.bfloat16)
    maskw = torch.zeros(V, cout + 16, dtype=torch.bfloat16, device="cuda")
    maskw[:, 16:] = m
    out = torch.zeros(V, cout + 32, dtype=torch.bfloat16, device="cuda")
    rc, _ = _conv("gm_unet_conv3_tc", B, X, Y, Z, cin, cout, wide_in, 48 + cin, 48,
                  W.to(torch.bfloat16).contiguous(), None, 0, out, cout + 32, 16, maskw, cout + 16, 16)
    assert rc == N.GM_OK
    ref = F.conv3d(x, _torch_w(W), padding=1) * _from_cl(m, B, cout, Z, Y, X)
    _close(_from_cl(out[:, 16:16 + cout].contiguous(), B, cout, Z, Y, X), ref, 1e-2)
    assert torch.all(out[:, :16] == 0) and torch.all(out[:, 16 + cout:] == 0)  # outside the slice: untouched
    # data gradient: dx = conv of dy with the transposed weights and mirrored taps
    xr = x.clone().requires_grad_(True)
    Wt = _torch_w(W).requires_grad_(True)
    y = F.conv3d(xr, Wt, padding=1)
    dy = _bf(torch.randn_like(y))
    y.backward(dy)
    WT = W.permute(0, 2, 1).contiguous().to(torch.bfloat16)
    dx = torch.empty(V, cin, dtype=torch.bfloat16, device="cuda")
    rc, _ = _conv("gm_unet_conv3_tc", B, X, Y, Z, cout, cin, _cl(dy), cout, 0, WT, None, 0, dx, cin, 0, mirror=1)
    assert rc == N.GM_OK
    _close(_from_cl(dx, B, cin, Z, Y, X), xr.grad, 1e-2)
    dx2 = torch.empty_like(dx)
    wp = torch.empty(27 * cin * cout, dtype=torch.bfloat16, device="cuda")
    rc, _ = _conv("gm_unet_conv3_tc", B, X, Y, Z, cout, cin, _cl(dy), cout, 0, WT, None, 0, dx2, cin, 0, mirror=1,
                  wpack=wp)
    assert rc == N.GM_OK and torch.equal(dx, dx2)
    assert N.lib().gm_unet_tc_status() == 0


def test_conv3_tc_rejects_unaligned_slices():
    import _native as N

    t = torch.zeros(64, 40, dtype=torch.bfloat16, device="cuda")
    W = torch.zeros(27, 32, 16, dtype=torch.bfloat16, device="cuda")
    a = N.gm_conv_args()
    a.grid[:] = [1, 4, 4, 4]
    a.cin, a.cout = 16, 32
    a.in_, a.in_stride, a.in_off = t.data_ptr(), 40, 2  # offset not a multiple of 8 channels
    a.w = W.data_ptr()
    a.out, a.out_stride, a.out_off = t.data_ptr(), 40, 8
    assert N.lib().gm_unet_conv3_tc_eligible(C.byref(a)) == 0
    assert N.lib().gm_unet_conv3_tc(C.byref(a), None) == N.GM_ERR_UNSUPPORTED
