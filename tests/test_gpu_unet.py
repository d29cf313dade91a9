"""Surrogate tensor-core kernels against PyTorch FP32 references of the same
ops (conv3d and its gradients, pooling, upsampling, the whole U-Net), on
BF16-rounded inputs."""

import ctypes as C

import pytest
import torch
import torch.nn.functional as F

pytestmark = pytest.mark.gpu


def _bf(t):
    return t.to(torch.bfloat16).to(torch.float32)


def _cl(x):  # [B, C, Z, Y, X] -> channels-last BF16 [V, C]
    return x.permute(0, 2, 3, 4, 1).contiguous().reshape(-1, x.shape[1]).to(torch.bfloat16)


def _from_cl(y, B, Cn, Z, Y, X):
    return y.float().reshape(B, Z, Y, X, Cn).permute(0, 4, 1, 2, 3)


def _torch_w(W):  # [27][co][ci] (tap = dx + 3 dy + 9 dz) -> [co][ci][dz][dy][dx]
    co, ci = W.shape[1], W.shape[2]
    return W.reshape(3, 3, 3, co, ci).permute(3, 4, 0, 1, 2).contiguous()


def _close(a, b, rel):
    err = (a - b).abs().max().item()
    assert err <= rel * b.abs().max().item() + 1e-6, (err, b.abs().max().item())


@pytest.mark.parametrize("cin,cout", [(16, 32), (32, 64), (64, 128), (192, 64), (96, 32), (128, 128)])
def test_conv3_forward(cin, cout):
    import _native as N
    import kern

    torch.manual_seed(0)
    B, Z, Y, X = 2, 6, 8, 12
    x = _bf(torch.randn(B, cin, Z, Y, X, device="cuda"))
    W = _bf(torch.randn(27, cout, cin, device="cuda") * 0.1)
    b = torch.randn(cout, device="cuda")
    ref = F.relu(F.conv3d(x, _torch_w(W), b, padding=1))
    xin = _cl(x)
    out = torch.empty(B * Z * Y * X, cout, dtype=torch.bfloat16, device="cuda")
    a = N.gm_conv_args()
    a.grid[:] = [B, X, Y, Z]
    a.cin, a.cout = cin, cout
    a.in_, a.in_stride, a.in_off = xin.data_ptr(), cin, 0
    a.w, a.bias, a.relu = W.to(torch.bfloat16).contiguous().data_ptr(), b.data_ptr(), 1
    Wb = W.to(torch.bfloat16).contiguous()
    a.w = Wb.data_ptr()
    a.out, a.out_stride, a.out_off = out.data_ptr(), cout, 0
    N.call("gm_unet_conv3", C.byref(a), kern.stream_ptr())
    torch.cuda.synchronize()
    _close(_from_cl(out, B, cout, Z, Y, X), ref, 1e-2)


@pytest.mark.parametrize("cin,cout", [(32, 32), (64, 128), (96, 32), (16, 32), (192, 64)])
def test_conv3_gradients(cin, cout):
    import _native as N
    import kern

    torch.manual_seed(1)
    B, Z, Y, X = 2, 4, 8, 8
    x = _bf(torch.randn(B, cin, Z, Y, X, device="cuda")).requires_grad_(True)
    W = _bf(torch.randn(27, cout, cin, device="cuda") * 0.1)
    Wt = _torch_w(W).requires_grad_(True)
    y = F.conv3d(x, Wt, padding=1)
    dy = _bf(torch.randn_like(y))
    y.backward(dy)
    V = B * Z * Y * X
    # data gradient: conv of dy with W^T (mirrored taps)
    if cin % 16 == 0 and cin in (16, 32, 64, 96, 128, 192):
        dyc = _cl(dy)
        WT = W.permute(0, 2, 1).contiguous().to(torch.bfloat16)
        dx = torch.empty(V, cin, dtype=torch.bfloat16, device="cuda")
        a = N.gm_conv_args()
        a.grid[:] = [B, X, Y, Z]
        a.cin, a.cout = cout, cin
        a.in_, a.in_stride, a.in_off = dyc.data_ptr(), cout, 0
        a.w, a.relu, a.mirror = WT.data_ptr(), 0, 1
        a.out, a.out_stride, a.out_off = dx.data_ptr(), cin, 0
        N.call("gm_unet_conv3", C.byref(a), kern.stream_ptr())
        torch.cuda.synchronize()
        _close(_from_cl(dx, B, cin, Z, Y, X), x.grad, 1e-2)
    # weight gradient
    xc = _cl(x.detach())
    dyc = _cl(dy)
    need = int(N.lib().gm_unet_wgrad_scratch((C.c_int * 4)(B, X, Y, Z), cin, cout))
    scr = torch.empty(need, dtype=torch.float32, device="cuda")
    dw = torch.empty(27, cout, cin, dtype=torch.float32, device="cuda")
    g = N.gm_wgrad_args()
    g.grid[:] = [B, X, Y, Z]
    g.cin, g.cout = cin, cout
    g.in_, g.in_stride, g.in_off = xc.data_ptr(), cin, 0
    g.dy, g.dy_stride, g.dy_off = dyc.data_ptr(), cout, 0
    g.dw, g.scratch, g.scratch_cap = dw.data_ptr(), scr.data_ptr(), scr.numel()
    N.call("gm_unet_wgrad", C.byref(g), kern.stream_ptr())
    torch.cuda.synchronize()
    _close(_torch_w(dw), Wt.grad, 2e-3)


def test_pool_up():
    import _native as N
    import kern

    torch.manual_seed(2)
    B, Cn, Z, Y, X = 2, 32, 4, 8, 12
    x = _bf(torch.randn(B, Cn, Z, Y, X, device="cuda"))
    xc = _cl(x)
    V = B * Z * Y * X
    grid = (C.c_int * 4)(B, X, Y, Z)
    p = torch.empty(V // 8, Cn, dtype=torch.bfloat16, device="cuda")
    N.call("gm_unet_pool2", grid, Cn, xc.data_ptr(), Cn, 0, p.data_ptr(), Cn, 0, 0, kern.stream_ptr())
    u = torch.empty(V, Cn, dtype=torch.bfloat16, device="cuda")
    N.call("gm_unet_up2", grid, Cn, p.data_ptr(), Cn, 0, u.data_ptr(), Cn, 0, 0, kern.stream_ptr())
    torch.cuda.synchronize()
    pr = F.avg_pool3d(x, 2)
    _close(_from_cl(p, B, Cn, Z // 2, Y // 2, X // 2), pr, 1e-2)
    _close(_from_cl(u, B, Cn, Z, Y, X), F.interpolate(_from_cl(p, B, Cn, Z // 2, Y // 2, X // 2), scale_factor=2),
           1e-6)


def _torch_unet(net, x, grid):
    """FP32 PyTorch restatement of surrogate.UNet.forward with its weights."""
    B, X, Y, Z = grid
    P = {k: v["w"] for k, v in net.p.items()}

    def cv(t, name):
        return F.relu(F.conv3d(t, _torch_w(_bf(P[name])), P[name + "b"], padding=1))

    e1 = cv(cv(x, "c1"), "c2")
    e2 = cv(cv(F.avg_pool3d(e1, 2), "c3"), "c4")
    b = cv(cv(F.avg_pool3d(e2, 2), "c5"), "c6")
    d2 = cv(cv(torch.cat([F.interpolate(b, scale_factor=2), e2], 1), "c7"), "c8")
    d1 = cv(cv(torch.cat([F.interpolate(d2, scale_factor=2), e1], 1), "c9"), "c10")
    return (d1 * P["head"].reshape(1, -1, 1, 1, 1)).sum(1)


def test_unet_forward_backward():
    import surrogate

    torch.manual_seed(3)
    grid = (2, 16, 16, 8)
    B, X, Y, Z = grid
    net = surrogate.UNet("cuda", seed=4)
    with torch.no_grad():
        net.p["head"]["w"].normal_(0, 0.3)
    x = torch.zeros(B, 16, Z, Y, X, device="cuda")
    x[:, :6] = _bf(torch.randn(B, 6, Z, Y, X, device="cuda"))
    xc = _cl(x)
    pred = net.forward(xc, grid).clone()
    ref = _torch_unet(net, x, grid)
    _close(pred.reshape(B, Z, Y, X), ref, 5e-2)
    target = torch.randn(B * Z * Y * X, device="cuda")
    lmask = torch.ones_like(target)
    loss = net.backward(target, lmask, 1.0 / target.numel())
    torch.cuda.synchronize()
    # reference gradients
    Pw = {k: v["w"].clone().requires_grad_(True) for k, v in net.p.items()}

    def cv(t, name):
        return F.relu(F.conv3d(t, _torch_w(Pw[name]), Pw[name + "b"], padding=1))

    e1 = cv(cv(x, "c1"), "c2")
    e2 = cv(cv(F.avg_pool3d(e1, 2), "c3"), "c4")
    b = cv(cv(F.avg_pool3d(e2, 2), "c5"), "c6")
    d2 = cv(cv(torch.cat([F.interpolate(b, scale_factor=2), e2], 1), "c7"), "c8")
    d1 = cv(cv(torch.cat([F.interpolate(d2, scale_factor=2), e1], 1), "c9"), "c10")
    yr = (d1 * Pw["head"].reshape(1, -1, 1, 1, 1)).sum(1).reshape(-1)
    lr = ((yr - target) ** 2).mean()
    lr.backward()
    assert abs(loss.item() - lr.item()) <= 0.05 * lr.item()
    for name in ("c1", "c5", "c7", "c10", "c2b", "head"):
        g = net.p[name]["g"]
        gr = Pw[name].grad
        cos = torch.nn.functional.cosine_similarity(g.reshape(-1), gr.reshape(-1), dim=0).item()
        assert cos > 0.98, (name, cos)


def test_unet_training_reduces_loss():
    import surrogate

    torch.manual_seed(5)
    grid = (2, 16, 16, 8)
    B, X, Y, Z = grid
    net = surrogate.UNet("cuda", seed=6)
    x = torch.zeros(B * Z * Y * X, 16, device="cuda")
    x[:, :6] = torch.randn(B * Z * Y * X, 6, device="cuda")
    xc = x.to(torch.bfloat16)
    target = torch.tanh(x[:, 0] * 0.7 + 0.3 * x[:, 1]).contiguous()
    lmask = torch.ones_like(target)
    losses = []
    for _ in range(60):
        net.forward(xc, grid)
        losses.append(net.backward(target, lmask, 1.0 / target.numel()).item())
        net.step(lr=3e-3)
    assert losses[-1] < 0.3 * losses[0], losses[::10]


@pytest.mark.parametrize("backward", [0, 1])
def test_pool_up_vector_and_element_forms_agree(backward):
    """Pooling and up-sampling, forward and backward: the 8-channel vector
    form (aligned slices) and the element-wise form (a slice offset that is not
    a multiple of 8 channels) give the same bits."""
    import _native as N
    import kern

    torch.manual_seed(5)
    B, Cn, X, Y, Z = 2, 16, 10, 6, 4
    fine = B * X * Y * Z
    grid = (C.c_int * 4)(B, X, Y, Z)
    for entry in ("gm_unet_pool2", "gm_unet_up2"):
        # the input lives on the fine grid for pool forward / up backward, on the coarse grid otherwise
        src_fine = (entry == "gm_unet_pool2") != bool(backward)
        nin, nout = (fine, fine // 8) if src_fine else (fine // 8, fine)
        src = torch.randn(nin, Cn, device="cuda").to(torch.bfloat16)
        a_in = torch.zeros(nin, Cn + 8, dtype=torch.bfloat16, device="cuda")
        a_in[:, 8:] = src
        b_in = torch.zeros(nin, Cn + 2, dtype=torch.bfloat16, device="cuda")
        b_in[:, 2:] = src
        a_out = torch.zeros(nout, Cn + 8, dtype=torch.bfloat16, device="cuda")
        b_out = torch.zeros(nout, Cn + 2, dtype=torch.bfloat16, device="cuda")
        N.call(entry, grid, Cn, a_in.data_ptr(), Cn + 8, 8, a_out.data_ptr(), Cn + 8, 8, backward, kern.stream_ptr())
        N.call(entry, grid, Cn, b_in.data_ptr(), Cn + 2, 2, b_out.data_ptr(), Cn + 2, 2, backward, kern.stream_ptr())
        torch.cuda.synchronize()
        assert torch.equal(a_out[:, 8:], b_out[:, 2:]), entry
        assert torch.all(a_out[:, :8] == 0) and torch.all(b_out[:, :2] == 0)
