"""The separable coupling contraction (constant k and rho*c) against the
element reduction of gm_couple on the same fine fields, for the Level-3 ->
Level-2 and Level-3 -> Level-1 geometries (4 and 20 fine elements per coarse
element), flux and mass terms, FP64 and FP32."""

import ctypes as C

import numpy as np
import pytest
import torch

import gomelt_oracle as O
from test_gpu_separable import CFG, CONST_PROPS

pytestmark = pytest.mark.gpu


def coupling(method, dtype, fine, coarse, P, fields, scale=1.0, base=None):
    import _native as N
    import engine
    import kern

    arena = engine.TableArena(1 << 22, "cuda")
    arena.begin()
    np_dtype = np.float64 if dtype == torch.float64 else np.float32
    cg = engine.CoupleGeom(fine["node_coords"], coarse["node_coords"], np_dtype, arena)
    arena.upload(torch.cuda.current_stream())
    nodes = [int(n) for n in fine["nodes"]]
    h = [float(np.asarray(c)[1] - np.asarray(c)[0]) for c in fine["node_coords"]]
    out_n = [n + 2 for n in cg.box_n] if base is None else list(cg.box_n)
    out_lo = [lo - 1 for lo in cg.box_lo] if base is None else list(cg.box_lo)
    out = torch.zeros(int(np.prod(out_n)), dtype=dtype, device="cuda")
    part = torch.empty(cg.partials, dtype=dtype, device="cuda")
    a = N.gm_couple_args()
    a.dtype = kern.dtype_code(out)
    a.geom = cg.struct
    for d in range(3):
        a.fine_nodes[d] = nodes[d]
        a.fine_h[d] = h[d]
        a.out_lo[d] = out_lo[d]
        a.out_n[d] = out_n[d]
    T = fields["T"].to(dtype)
    ph = torch.zeros(T.numel(), dtype=torch.uint8, device="cuda")
    a.T = kern.ptr(T)
    a.ph = C.cast(ph.data_ptr(), C.POINTER(C.c_uint8))
    keep = [T, ph]
    for name in ("Tp", "dTa", "dTb"):
        if name in fields:
            t = fields[name].to(dtype)
            keep.append(t)
            setattr(a, name, kern.ptr(t))
    dt = torch.tensor([2e-6], dtype=torch.float64, device="cuda")
    a.dt = kern.ptr(dt)
    a.out = kern.ptr(out)
    a.scale = scale
    a.partials = part.data_ptr()
    a.partials_cap = part.numel()
    a.method = method
    if base is not None:
        base_t = torch.as_tensor(base(out.numel()), dtype=dtype, device="cuda")
        keep.append(base_t)
        a.base = kern.ptr(base_t)
    ps = N.props_struct(P)
    N.call("gm_couple", C.byref(a), C.byref(ps), kern.stream_ptr(None))
    torch.cuda.synchronize()
    return out.double().cpu().numpy()


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 2e-5)])
@pytest.mark.parametrize("coarse_lev", [2, 1])
@pytest.mark.parametrize("terms", ["flux", "mass", "both"])
def test_separable_matches_element_reduction(dtype, tol, coarse_lev, terms):
    P = O.SetupProperties(CONST_PROPS)
    L = O.SetupLevels(CFG, P)
    fine, coarse = L[3], L[coarse_lev]
    n = int(fine["nn"])
    rng = np.random.default_rng(coarse_lev)
    f = {"T": torch.tensor(300 + 1500 * rng.random(n), device="cuda")}
    if terms in ("flux", "both"):
        f["Tp"] = torch.tensor(50 * rng.standard_normal(n), device="cuda")
    if terms in ("mass", "both"):
        f["dTa"] = torch.tensor(20 * rng.standard_normal(n), device="cuda")
        f["dTb"] = torch.tensor(20 * rng.standard_normal(n), device="cuda")
    ref = coupling(1, dtype, fine, coarse, P, f, scale=0.7)
    got = coupling(2, dtype, fine, coarse, P, f, scale=0.7)
    assert np.abs(ref).max() > 0
    assert np.abs(got - ref).max() <= tol * np.abs(ref).max()
    # automatic choice: the separable path for constant properties
    auto = coupling(0, dtype, fine, coarse, P, f, scale=0.7)
    np.testing.assert_array_equal(auto, got)


def test_separable_refuses_variable_properties():
    import _native as N
    from test_gpu_level import PHASE_PROPS

    P = O.SetupProperties(PHASE_PROPS)
    L = O.SetupLevels(CFG, P)
    n = int(L[3]["nn"])
    f = {"T": torch.full((n,), 400.0, device="cuda"), "Tp": torch.zeros(n, device="cuda")}
    with pytest.raises(N.GomeltError):
        coupling(2, torch.float64, L[3], L[2], P, f)


@pytest.mark.parametrize("method", [1, 2])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_output_onto_base(method, dtype):
    """out = base + scale * terms equals base added to the terms alone (to a
    few ulps: base + scale * s may be one fused multiply-add)."""
    P = O.SetupProperties(CONST_PROPS)
    L = O.SetupLevels(CFG, P)
    n = int(L[3]["nn"])
    rng = np.random.default_rng(9)
    f = {"T": torch.tensor(300 + 1500 * rng.random(n), device="cuda"),
         "Tp": torch.tensor(50 * rng.standard_normal(n), device="cuda"),
         "dTa": torch.tensor(20 * rng.standard_normal(n), device="cuda"),
         "dTb": torch.tensor(20 * rng.standard_normal(n), device="cuda")}
    b = lambda m: np.random.default_rng(4).standard_normal(m)  # noqa: E731
    terms = coupling(method, dtype, L[3], L[2], P, f, scale=0.7, base=lambda m: np.zeros(m))
    got = coupling(method, dtype, L[3], L[2], P, f, scale=0.7, base=b)
    ref = torch.as_tensor(b(got.size), dtype=dtype).double().numpy() + terms
    rtol, atol = (1e-6, 1e-7) if dtype == torch.float32 else (1e-14, 1e-15)
    np.testing.assert_allclose(got, ref, rtol=rtol, atol=atol)
