"""gm_couple_noalloc: the coupling terms without caller-provided scratch.

Callers that cannot allocate device memory when they need the coupling terms
(a framework owning the allocator, a loop that must not synchronise) use this
entry point; its partial sums live in a fixed library-owned device array.  This
file runs last so that a failure here leaves every other test already run; it
also passes on its own in a fresh process.

Cases: a phase-dependent material (element reduction), a constant-property
material through the default path choice and the forced separable
contraction, and a window whose separable partials exceed the array while the
element reduction's fit (the call must take the element path, as gm_couple
does with that capacity).
"""

import copy
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

PHASE_MAT = {"thermal_conductivity_powder": 0.4, "thermal_conductivity_bulk_a0": 4.23,
             "thermal_conductivity_bulk_a1": 0.016, "thermal_conductivity_fluid_a0": 29.0,
             "heat_capacity_solid_a0": 383.1, "heat_capacity_solid_a1": 0.174, "heat_capacity_mushy": 3235.0,
             "heat_capacity_fluid": 769.0, "density": 8e-06, "T_amb": 298.15, "T_solidus": 1533,
             "T_liquidus": 1609, "layer_height": 0.02, "laser_center": [1.0, 1.0, 0, 0, 0, 0, 0]}
CONST_MAT = {"thermal_conductivity_powder": 22.0, "thermal_conductivity_bulk_a0": 22.0,
             "thermal_conductivity_bulk_a1": 0.0, "thermal_conductivity_fluid_a0": 22.0,
             "heat_capacity_solid_a0": 700.0, "heat_capacity_solid_a1": 0.0, "heat_capacity_mushy": 700.0,
             "heat_capacity_fluid": 700.0, "density": 4.4e-06, "T_amb": 300.0, "T_solidus": 1878,
             "T_liquidus": 1900, "layer_height": 0.02, "laser_center": [1.0, 1.0, 0, 0, 0, 0, 0]}

CFG = {
    "Level1": {"elements": [20, 20, 6], "bounds": {"x": [0, 2.0], "y": [0, 2.0], "z": [-0.6, 0]},
               "conditions": {"x": [300, 300], "y": [300, 300], "z": [300, 300]}},
    "Level2": {"elements": [40, 40, 10], "bounds": {"x": [0.6, 1.4], "y": [0.6, 1.4], "z": [-0.2, 0]}},
    "Level3": {"elements": [80, 40, 12], "bounds": {"x": [0.8, 1.2], "y": [0.9, 1.1], "z": [-0.06, 0]}},
}
# A 140 x 140 x 32-element fine window at 4x the coarse resolution: its
# separable partials (673,596 values) exceed the 4 MiB array in FP64 (524,288
# doubles), the element reduction's (78,400) fit.
BIG_L3 = {"elements": [140, 140, 32], "bounds": {"x": [0.64, 1.34], "y": [0.64, 1.34], "z": [-0.16, 0]}}
ARRAY_BYTES = 4 << 20


def _engine(mat, dtype, l3=None, seed=5):
    from engine import Engine
    from levels import setup_properties

    cfg = copy.deepcopy(CFG)
    cfg["properties"] = dict(mat)
    if l3 is not None:
        cfg["Level3"] = copy.deepcopy(l3)
    P = setup_properties(cfg["properties"])
    eng = Engine(cfg, P, 1, 1, dtype=dtype)
    rng = np.random.default_rng(seed)
    n3 = eng.geo.L[3].nn
    eng.T[3].copy_(torch.as_tensor(300 + 2500 * rng.random(n3), dtype=dtype))
    eng.Tp[3].copy_(torch.as_tensor(40 * rng.standard_normal(n3), dtype=dtype))
    eng.ph[3].copy_(torch.as_tensor(rng.integers(0, 4, n3).astype(np.uint8)))
    dTa = torch.as_tensor(40 * rng.standard_normal(n3), dtype=dtype, device="cuda")
    dTb = torch.as_tensor(40 * rng.standard_normal(n3), dtype=dtype, device="cuda")
    dt = torch.tensor([2e-5], dtype=torch.float64, device="cuda")
    eng.build_tables()
    return eng, P, dTa, dTb, dt


def _args(eng, cg, out, dTa, dTb, dt, partials, method=0):
    import _native as N
    import kern

    L = eng.geo.L[3]
    a = N.gm_couple_args()
    a.dtype = kern.dtype_code(out)
    a.geom = cg.struct
    for d in range(3):
        a.fine_nodes[d] = L.nodes[d]
        a.fine_h[d] = L.spacing()[d]
        a.out_lo[d] = cg.box_lo[d]
        a.out_n[d] = cg.box_n[d]
    a.T = eng.T[3].data_ptr()
    a.ph = C.cast(eng.ph[3].data_ptr(), C.POINTER(C.c_uint8))
    a.substrate = eng.substrate[3]
    a.Tp = eng.Tp[3].data_ptr()
    a.dTa, a.dTb, a.dt = dTa.data_ptr(), dTb.data_ptr(), dt.data_ptr()
    a.out = out.data_ptr()
    a.scale = 1.0
    a.method = method
    if partials is not None:
        a.partials, a.partials_cap = partials.data_ptr(), partials.numel()
    return a


def _reference(eng, P, cg, dTa, dTb, dt, dtype, method):
    """gm_couple with a caller-provided scratch of the full size."""
    import _native as N

    out = torch.zeros(int(np.prod(cg.box_n)), dtype=dtype, device="cuda")
    partials = torch.empty(cg.partials, dtype=dtype, device="cuda")
    a = _args(eng, cg, out, dTa, dTb, dt, partials, method)
    assert N.lib().gm_couple(C.byref(a), C.byref(N.props_struct(P)), None) == N.GM_OK
    torch.cuda.synchronize()
    assert torch.count_nonzero(out) > 0
    return out


def _check_noalloc(eng, P, cg, dTa, dTb, dt, dtype, method, ref, rtol):
    import _native as N

    for _ in range(2):  # two calls in a row share the library's scratch array
        out = torch.zeros(ref.numel(), dtype=dtype, device="cuda")
        b = _args(eng, cg, out, dTa, dTb, dt, None, method)
        assert N.lib().gm_couple_noalloc(C.byref(b), C.byref(N.props_struct(P)), None) == N.GM_OK
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.double().cpu().numpy(), ref.double().cpu().numpy(), rtol=rtol,
                                   atol=rtol * float(ref.abs().max()))


TOLS = [(torch.float32, 1e-6), (torch.float64, 1e-13)]


@pytest.mark.parametrize("dtype,rtol", TOLS)
@pytest.mark.parametrize("coarse", [2, 1])
def test_noalloc_matches_gm_couple(dtype, rtol, coarse):
    eng, P, dTa, dTb, dt = _engine(PHASE_MAT, dtype)
    cg = eng.tables["c32" if coarse == 2 else "c31"]
    ref = _reference(eng, P, cg, dTa, dTb, dt, dtype, 0)
    _check_noalloc(eng, P, cg, dTa, dTb, dt, dtype, 0, ref, rtol)


@pytest.mark.parametrize("dtype,rtol", TOLS)
@pytest.mark.parametrize("method", [0, 2])
@pytest.mark.parametrize("coarse", [2, 1])
def test_noalloc_constant_properties(dtype, rtol, method, coarse):
    """Constant k and rho*c: the separable contraction, chosen (method 0) or
    forced (method 2), through the library's array."""
    eng, P, dTa, dTb, dt = _engine(CONST_MAT, dtype)
    cg = eng.tables["c32" if coarse == 2 else "c31"]
    ref = _reference(eng, P, cg, dTa, dTb, dt, dtype, method)
    _check_noalloc(eng, P, cg, dTa, dTb, dt, dtype, method, ref, rtol)


def test_noalloc_falls_back_to_element_path():
    """Separable partials beyond the array, element partials within it: the
    call succeeds on the element reduction (same result as gm_couple's
    element path), while the forced separable contraction is refused."""
    import _native as N

    dtype = torch.float64
    eng, P, dTa, dTb, dt = _engine(CONST_MAT, dtype, l3=BIG_L3)
    cg = eng.tables["c32"]
    assert cg.partials * 8 > ARRAY_BYTES  # the larger (separable) scratch does not fit
    ref = _reference(eng, P, cg, dTa, dTb, dt, dtype, 1)  # element reduction
    _check_noalloc(eng, P, cg, dTa, dTb, dt, dtype, 0, ref, 1e-13)
    sep = _reference(eng, P, cg, dTa, dTb, dt, dtype, 2)  # separable, caller scratch
    np.testing.assert_allclose(sep.cpu().numpy(), ref.cpu().numpy(), rtol=1e-11,
                               atol=1e-11 * float(ref.abs().max()))
    out = torch.zeros(ref.numel(), dtype=dtype, device="cuda")
    b = _args(eng, cg, out, dTa, dTb, dt, None, 2)
    assert N.lib().gm_couple_noalloc(C.byref(b), C.byref(N.props_struct(P)), None) == N.GM_ERR_TOO_LARGE


def test_noalloc_rejects_oversize():
    import _native as N

    g = N.gm_couple_args()
    g.dtype = N.GM_F64
    fake = 256  # never dereferenced: the size check comes first
    for d in range(3):
        ax = g.geom.ax[d]
        ax.nfe, ax.ncb, ax.rmax, ax.H = 4000, 1000, 4, 0.02
        ax.cw, ax.flo, ax.fhi = fake, C.cast(fake, C.POINTER(C.c_int)), C.cast(fake, C.POINTER(C.c_int))
        g.out_n[d] = 1001
    g.T = g.Tp = g.out = fake
    assert N.lib().gm_couple_partials_size(C.byref(g.geom)) * 8 > ARRAY_BYTES
    rc = N.lib().gm_couple_noalloc(C.byref(g), C.byref(N.gm_props()), None)
    assert rc == N.GM_ERR_TOO_LARGE
