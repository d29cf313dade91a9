"""gm_couple_noalloc: the coupling terms without caller-provided scratch.

Callers that cannot allocate device memory when they need the coupling terms
(a framework owning the allocator, a loop that must not synchronise) use this
entry point; its partial sums live in a fixed library-owned device array.  This
file runs last so that a failure here leaves every other test already run; it
also passes on its own in a fresh process.
"""

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

CFG = {
    "Level1": {"elements": [20, 20, 6], "bounds": {"x": [0, 2.0], "y": [0, 2.0], "z": [-0.6, 0]},
               "conditions": {"x": [300, 300], "y": [300, 300], "z": [300, 300]}},
    "Level2": {"elements": [40, 40, 10], "bounds": {"x": [0.6, 1.4], "y": [0.6, 1.4], "z": [-0.2, 0]}},
    "Level3": {"elements": [80, 40, 12], "bounds": {"x": [0.8, 1.2], "y": [0.9, 1.1], "z": [-0.06, 0]}},
    "properties": {"thermal_conductivity_powder": 0.4, "thermal_conductivity_bulk_a0": 4.23,
                   "thermal_conductivity_bulk_a1": 0.016, "thermal_conductivity_fluid_a0": 29.0,
                   "heat_capacity_solid_a0": 383.1, "heat_capacity_solid_a1": 0.174, "heat_capacity_mushy": 3235.0,
                   "heat_capacity_fluid": 769.0, "density": 8e-06, "T_amb": 298.15, "T_solidus": 1533,
                   "T_liquidus": 1609, "layer_height": 0.02, "laser_center": [1.0, 1.0, 0, 0, 0, 0, 0]},
}


def _args(eng, cg, out, dTa, dTb, dt, partials):
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
    if partials is not None:
        a.partials, a.partials_cap = partials.data_ptr(), partials.numel()
    return a


@pytest.mark.parametrize("dtype,rtol", [(torch.float32, 1e-6), (torch.float64, 1e-13)])
@pytest.mark.parametrize("coarse", [2, 1])
def test_noalloc_matches_gm_couple(dtype, rtol, coarse):
    import _native as N
    from engine import Engine
    from levels import setup_properties

    P = setup_properties(CFG["properties"])
    eng = Engine(CFG, P, 1, 1, dtype=dtype)
    rng = np.random.default_rng(5)
    n3 = eng.geo.L[3].nn
    eng.T[3].copy_(torch.as_tensor(300 + 2500 * rng.random(n3), dtype=dtype))
    eng.Tp[3].copy_(torch.as_tensor(40 * rng.standard_normal(n3), dtype=dtype))
    eng.ph[3].copy_(torch.as_tensor(rng.integers(0, 4, n3).astype(np.uint8)))
    dTa = torch.as_tensor(40 * rng.standard_normal(n3), dtype=dtype, device="cuda")
    dTb = torch.as_tensor(40 * rng.standard_normal(n3), dtype=dtype, device="cuda")
    dt = torch.tensor([2e-5], dtype=torch.float64, device="cuda")
    eng.build_tables()
    cg = eng.tables["c32" if coarse == 2 else "c31"]
    nout = int(np.prod(cg.box_n))
    props = N.props_struct(P)
    lib = N.lib()

    ref = torch.zeros(nout, dtype=dtype, device="cuda")
    partials = torch.empty(cg.partials, dtype=dtype, device="cuda")
    a = _args(eng, cg, ref, dTa, dTb, dt, partials)
    assert lib.gm_couple(C.byref(a), C.byref(props), None) == N.GM_OK
    torch.cuda.synchronize()
    assert torch.count_nonzero(ref) > 0

    for _ in range(2):  # two calls in a row share the library's scratch array
        out = torch.zeros(nout, dtype=dtype, device="cuda")
        b = _args(eng, cg, out, dTa, dTb, dt, None)
        assert lib.gm_couple_noalloc(C.byref(b), C.byref(props), None) == N.GM_OK
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.double().cpu().numpy(), ref.double().cpu().numpy(), rtol=rtol,
                                   atol=rtol * float(ref.abs().max()))


def test_noalloc_rejects_oversize():
    import _native as N

    g = N.gm_couple_args()
    g.dtype = N.GM_F64
    for d in range(3):
        ax = g.geom.ax[d]
        ax.nfe, ax.ncb, ax.rmax, ax.H = 4000, 1000, 4, 0.02
        ax.cw, ax.flo, ax.fhi = 16, C.cast(16, C.POINTER(C.c_int)), C.cast(16, C.POINTER(C.c_int))
    assert N.lib().gm_couple_partials_size(C.byref(g.geom)) * 8 > (4 << 20)  # beyond the 4 MiB array
    rc = N.lib().gm_couple_noalloc(C.byref(g), C.byref(N.gm_props()), None)
    assert rc == N.GM_ERR_TOO_LARGE
