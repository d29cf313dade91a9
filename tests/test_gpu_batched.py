"""Batched level steps (many windows of uneven sizes in one launch) and the
launch-shape autotuner: results bit-identical to one gm_level_step per
window."""

import ctypes as C

import numpy as np
import pytest
import torch

import gomelt_oracle as O
from test_gpu_level import PHASE_PROPS

pytestmark = pytest.mark.gpu

SHAPES = [(41, 33, 21), (25, 29, 13), (57, 17, 9), (161, 161, 41)]


def windows(dtype, accum, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for i, (nx, ny, nz) in enumerate(SHAPES):
        n = nx * ny * nz
        h = (0.005, 0.005, 0.005)
        o = (0.1 * i, 0.2, -0.005 * (nz - 1))
        T = 300 + 2000 * rng.random(n)
        w = dict(nodes=(nx, ny, nz), h=h, origin=o, ne_planes=nz - 1,
                 T_in=torch.tensor(T, dtype=dtype, device="cuda"),
                 T_out=torch.empty(n, dtype=dtype, device="cuda"),
                 ph_in=torch.tensor(rng.integers(0, 4, n).astype(np.uint8), device="cuda"),
                 ph_out=torch.empty(n, dtype=torch.uint8, device="cuda"),
                 dt=torch.tensor([1e-6 * (1 + 0.1 * i)], dtype=torch.float64, device="cuda"),
                 laser=torch.tensor([o[0] + 0.05, o[1] + 0.04, 0.0, 1, 1, 1e-6, 150.0 + 30 * i],
                                    dtype=torch.float64, device="cuda"),
                 surface=1, clamp=1, bc_mode=3, bc_alpha=0.3, bc_beta=0.7,
                 bc_new=torch.tensor(300 + 50 * rng.random(n), dtype=dtype, device="cuda"),
                 bc_old=torch.tensor(300 + 50 * rng.random(n), dtype=dtype, device="cuda"),
                 substrate=nx * ny * 2)
        if accum:
            w["accum"] = torch.tensor(rng.random(n) * 1e-5, dtype=dtype, device="cuda")
            w["max_accum"] = torch.tensor(rng.random(n) * 1e-5, dtype=dtype, device="cuda")
        out.append(w)
    return out


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("accum", [False, True])
def test_batched_equals_single(dtype, accum):
    import _native as N
    import kern

    P = O.SetupProperties(PHASE_PROPS)
    ps = N.props_struct(P)
    single = windows(dtype, accum)
    batch = windows(dtype, accum)
    for w in single:
        kern.level_step(ps, **w)
    args = (N.gm_level_args * len(batch))(*[kern.level_args(**w) for w in batch])
    props = (N.gm_props * len(batch))(*[ps] * len(batch))
    nbytes = int(N.lib().gm_level_batched_desc_size(len(batch), kern.dtype_code(batch[0]["T_in"])))
    desc = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    N.call("gm_level_step_batched", C.cast(args, C.c_void_p), len(batch), C.cast(props, C.c_void_p),
           desc.data_ptr(), nbytes, kern.stream_ptr())
    torch.cuda.synchronize()
    for a, b in zip(single, batch):
        assert torch.equal(a["T_out"], b["T_out"])
        assert torch.equal(a["ph_out"], b["ph_out"])
        if accum:
            assert torch.equal(a["accum"], b["accum"]) and torch.equal(a["max_accum"], b["max_accum"])


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("accum", [False, True])
def test_batched_separable_equals_single(dtype, accum):
    """Constant-property windows take the separable kernel in both forms."""
    import _native as N
    import kern
    from test_gpu_separable import CONST_PROPS

    P = O.SetupProperties(CONST_PROPS)
    ps = N.props_struct(P)
    single = windows(dtype, accum, seed=3)
    batch = windows(dtype, accum, seed=3)
    for w in single:
        kern.level_step_shape(ps, kernel=1, rows=2, tile_y=4, zchunk=5, **w)
    args = (N.gm_level_args * len(batch))(*[kern.level_args(**w) for w in batch])
    props = (N.gm_props * len(batch))(*[ps] * len(batch))
    nbytes = int(N.lib().gm_level_batched_desc_size(len(batch), kern.dtype_code(batch[0]["T_in"])))
    desc = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    info = N.gm_batch_info()
    N.call("gm_level_batched_prepare", C.cast(args, C.c_void_p), len(batch), C.cast(props, C.c_void_p),
           desc.data_ptr(), nbytes, C.byref(info), kern.stream_ptr())
    assert info.kernel == 1 and info.rows == 2 and info.warps == 4
    N.call("gm_level_batched_launch", desc.data_ptr(), C.byref(info), kern.stream_ptr())
    torch.cuda.synchronize()
    for a, b in zip(single, batch):
        assert torch.equal(a["T_out"], b["T_out"])
        assert torch.equal(a["ph_out"], b["ph_out"])
        if accum:
            assert torch.equal(a["accum"], b["accum"]) and torch.equal(a["max_accum"], b["max_accum"])


def test_autotune_keeps_results():
    import _native as N
    import kern

    P = O.SetupProperties(PHASE_PROPS)
    ps = N.props_struct(P)
    w = windows(torch.float32, False)[3]
    kern.level_step(ps, **w)
    ref = w["T_out"].clone()
    tx, ty, zc, us, kernel, rows = kern.level_autotune(ps, reps=3, **w)
    assert kernel == 0 and (tx, ty) in ((32, 8), (16, 16)) and 2 <= zc <= 41 and us > 0
    w["T_out"].zero_()
    kern.level_step(ps, **w)  # uses the tuned shape
    torch.cuda.synchronize()
    assert torch.equal(w["T_out"], ref)


def test_batched_rejects_mixed_features():
    import _native as N
    import kern

    P = O.SetupProperties(PHASE_PROPS)
    ps = N.props_struct(P)
    ws = windows(torch.float32, False)[:2]
    ws[1]["laser"] = None
    args = (N.gm_level_args * 2)(*[kern.level_args(**w) for w in ws])
    props = (N.gm_props * 2)(ps, ps)
    desc = torch.empty(1 << 16, dtype=torch.uint8, device="cuda")
    with pytest.raises(N.GomeltError):
        N.call("gm_level_step_batched", C.cast(args, C.c_void_p), 2, C.cast(props, C.c_void_p), desc.data_ptr(),
               1 << 16, kern.stream_ptr())
