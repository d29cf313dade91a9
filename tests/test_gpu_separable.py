"""GPU parity of the separable level-step kernel (constant k and rho*c)
against the oracle, for the Level-3, Level-3 + melt time, Level-2 and
Level-1 feature sets of the subcycle, over launch shapes; the element-tile
kernel runs the same cases for comparison."""

import numpy as np
import pytest
import torch

import gomelt_oracle as O
from test_gpu_level import PHASE_PROPS, dev, geom, phase_of, relerr

pytestmark = pytest.mark.gpu

# constant conductivity and heat capacity in every phase; evaporation on
CONST_PROPS = dict(PHASE_PROPS, thermal_conductivity_powder=20.0, thermal_conductivity_bulk_a0=20.0,
                   thermal_conductivity_bulk_a1=0.0, thermal_conductivity_fluid_a0=20.0,
                   heat_capacity_solid_a0=700.0, heat_capacity_solid_a1=0.0, heat_capacity_mushy=700.0,
                   heat_capacity_fluid=700.0)

CFG = {
    "Level1": {"elements": [20, 20, 6], "bounds": {"x": [0, 2.0], "y": [0, 2.0], "z": [-0.6, 0]},
               "conditions": {"x": [300, 310], "y": [305, 300], "z": [300, 300]}},
    "Level2": {"elements": [40, 40, 10], "bounds": {"x": [0.6, 1.4], "y": [0.6, 1.4], "z": [-0.2, 0]}},
    "Level3": {"elements": [80, 40, 12], "bounds": {"x": [0.8, 1.2], "y": [0.9, 1.1], "z": [-0.06, 0]}},
}
# a Level-3 window 300 nodes wide (ten x-tiles)
CFG_WIDE = dict(CFG, Level3={"elements": [299, 12, 6], "bounds": {"x": [0.85, 1.149], "y": [0.94, 1.06],
                                                                   "z": [-0.03, 0]}})

# (kernel, rows, warps a CTA, zchunk); kernel None = the library's own choice
# (1, 4, 4, 6) and (1, 2, 2, 9) are the Level-3 and Level-1 shapes the autotuner chose on the part-scale
# workload; (1, 1, 2, 7) a one-row strip with an odd z-chunk
SHAPES = [(None, 0, 0, 0), (0, 0, 0, 5), (1, 4, 1, 2), (1, 2, 2, 3), (1, 4, 4, 5), (1, 2, 8, 32), (1, 4, 4, 6),
          (1, 2, 2, 9), (1, 1, 2, 7)]


def setup(cfg, seed):
    import _native as N

    P = O.SetupProperties(CONST_PROPS)
    L = O.SetupLevels(cfg, P)
    rng = np.random.default_rng(seed)
    for lev in (1, 2, 3):
        x, y, z = (np.asarray(c) for c in L[lev]["node_coords"])
        X = np.tile(x, len(y) * len(z))
        Y = np.repeat(np.tile(y, len(z)), len(x))
        Z = np.repeat(z, len(x) * len(y))
        T = P["T_amb"] + 2600 * np.exp(-((X - 1.0) ** 2 + (Y - 1.0) ** 2) / 0.01 + Z * 20)
        L[lev]["T0"] = T + 5 * rng.standard_normal(T.shape)
        L[lev]["S1"] = (rng.random(T.shape) > 0.4).astype(float)
        L[lev]["S2"] = rng.random(T.shape) > 0.7
    return P, L, N.props_struct(P)


def run(ps, shape, nn, dtype, **kw):
    """One level step with `shape`; T_out is a view into a larger buffer whose
    tail must stay untouched."""
    import kern

    big = torch.full((nn + 4096,), -7.0, dtype=dtype, device="cuda")
    T_out = big[:nn]
    kernel, rows, wys, zc = shape
    if kernel is None:
        kern.level_step(ps, T_out=T_out, **kw)
    elif kernel == 0:
        kern.level_step_shape(ps, kernel=0, tile_x=32, zchunk=zc, T_out=T_out, **kw)
    else:
        kern.level_step_shape(ps, kernel=1, rows=rows, tile_y=wys, zchunk=zc, T_out=T_out, **kw)
    torch.cuda.synchronize()
    assert torch.all(big[nn:] == -7.0)
    return T_out.cpu().numpy()


def level3_case(cfg, seed, dtype, accum):
    P, L, ps = setup(cfg, seed)
    L3 = L[3]
    nodes, h, o = geom(L3)
    nn3, ne3 = int(L3["nn"]), int(L3["ne"])
    ne_nn = (int(L[2]["ne"]), ne3, int(L[1]["nn"]), int(L[2]["nn"]), nn3)
    sub = nodes[0] * nodes[1] * 4
    v = np.array([1.013, 0.997, 0.0, 1, 1, 1.5e-6, 250.0])
    dt = v[5]
    rng = np.random.default_rng(seed + 100)
    bcn = 300 + 400 * rng.random(nn3)
    bco = 300 + 400 * rng.random(nn3)
    alpha = 0.3
    S1n, S2n, k, rc = O.computeStateProperties(L3["T0"], L3["S1"], P, sub)
    F = O.computeSourcesL3(L3, v, ne_nn, P, v[6])
    F = O.computeConvRadBC(L3, L3["T0"], ne3, nn3, P, F)
    T = O.solveMatrixFreeFE(L3, nn3, ne3, k, rc, dt, L3["T0"], F, 0)
    ref = np.maximum(P["T_amb"], O.assignBCsFine(T, alpha * bcn + (1 - alpha) * bco, L3["BC"]))
    kw = dict(T_in=dev(L3["T0"], dtype), nodes=nodes, h=h, origin=o, ne_planes=nodes[2] - 1,
              dt=dev([dt], torch.float64), ph_in=phase_of(L3), substrate=sub, laser=dev(v, torch.float64),
              surface=1, bc_mode=3, bc_new=dev(bcn, dtype), bc_old=dev(bco, dtype), bc_alpha=alpha,
              bc_beta=1 - alpha, clamp=1)
    extra = {}
    if accum:
        acc0 = rng.uniform(0, 1e-4, nn3)
        macc0 = rng.uniform(0, 1e-4, nn3)
        reset = ((1 - 2 * np.asarray(L3["S2"], dtype=float)) * S2n) == 1
        racc = acc0 * reset
        extra = dict(acc0=acc0, macc0=macc0, macc_ref=np.maximum(racc, macc0), acc_ref=acc0 + dt * S2n - racc)
    return ps, nn3, kw, ref, (S1n, S2n), extra


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
@pytest.mark.parametrize("accum", [False, True])
def test_level3(shape, dtype, tol, accum):
    ps, nn, kw, ref, (S1n, S2n), ex = level3_case(CFG, 1, dtype, accum)
    ph_out = torch.empty(nn, dtype=torch.uint8, device="cuda")
    if accum:
        acc, macc = dev(ex["acc0"], dtype), dev(ex["macc0"], dtype)
        kw.update(accum=acc, max_accum=macc)
    out = run(ps, shape, nn, dtype, ph_out=ph_out, **kw)
    assert relerr(out, ref) < tol
    ph = ph_out.cpu().numpy()
    np.testing.assert_array_equal(ph & 1, S1n.astype(np.uint8))
    np.testing.assert_array_equal((ph >> 1) & 1, S2n.astype(np.uint8))
    if accum:
        atol = 1e-16 if dtype == torch.float64 else 1e-10
        np.testing.assert_allclose(acc.cpu().numpy(), ex["acc_ref"], rtol=1e-6, atol=atol)
        np.testing.assert_allclose(macc.cpu().numpy(), ex["macc_ref"], rtol=1e-6, atol=atol)


@pytest.mark.parametrize("shape", [(None, 0, 0, 0), (1, 4, 1, 2), (1, 2, 1, 3)])
@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_level3_wide(shape, dtype, tol):
    ps, nn, kw, ref, _, _ = level3_case(CFG_WIDE, 4, dtype, False)
    out = run(ps, shape, nn, dtype, ph_out=torch.empty(nn, dtype=torch.uint8, device="cuda"), **kw)
    assert relerr(out, ref) < tol


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_level2(shape, dtype, tol):
    """Level-2 feature set: RHS on a box, surface flux, Dirichlet ring from a
    blend of two fields, clamp, phase in/out."""
    P, L, ps = setup(CFG, 2)
    L2 = L[2]
    nodes, h, o = geom(L2)
    nn2, ne2 = int(L2["nn"]), int(L2["ne"])
    sub = nodes[0] * nodes[1] * 3
    dt = 5e-6
    box = [4, 30, 6, 37, 2, 11]
    rng = np.random.default_rng(12)
    rb = rng.standard_normal((box[5] - box[4], box[3] - box[2], box[1] - box[0])) * 1e-2
    V = np.zeros((nodes[2], nodes[1], nodes[0]))
    V[box[4]:box[5], box[2]:box[3], box[0]:box[1]] = rb
    bcn = 300 + 400 * rng.random(nn2)
    bco = 300 + 400 * rng.random(nn2)
    alpha = 0.6
    S1n, S2n, k, rc = O.computeStateProperties(L2["T0"], L2["S1"], P, sub)
    F = O.computeConvRadBC(L2, L2["T0"], ne2, nn2, P, V.reshape(-1))
    T = O.solveMatrixFreeFE(L2, nn2, ne2, k, rc, dt, L2["T0"], F, 0)
    ref = np.maximum(P["T_amb"], O.assignBCsFine(T, alpha * bcn + (1 - alpha) * bco, L2["BC"]))
    ph_out = torch.empty(nn2, dtype=torch.uint8, device="cuda")
    out = run(ps, shape, nn2, dtype, T_in=dev(L2["T0"], dtype), nodes=nodes, h=h, origin=o,
              ne_planes=nodes[2] - 1, dt=dev([dt], torch.float64), ph_in=phase_of(L2), ph_out=ph_out,
              substrate=sub, rhs_box=dev(rb, dtype), box=box, surface=1, bc_mode=3, bc_new=dev(bcn, dtype),
              bc_old=dev(bco, dtype), bc_alpha=alpha, bc_beta=1 - alpha, clamp=1)
    assert relerr(out, ref) < tol
    ph = ph_out.cpu().numpy()
    np.testing.assert_array_equal(ph & 1, S1n.astype(np.uint8))
    np.testing.assert_array_equal((ph >> 1) & 1, S2n.astype(np.uint8))


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_level1(shape, dtype, tol):
    """Level-1 feature set: inactive top planes reset to T_amb, constant
    Dirichlet faces, surface flux on the top active plane, RHS on a box."""
    P, L, ps = setup(CFG, 3)
    L1 = L[1]
    nodes, h, o = geom(L1)
    nn1 = int(L1["nn"])
    ne_planes = nodes[2] - 1 - 2
    tmp = ((nodes[0] - 1) * (nodes[1] - 1) * ne_planes, nodes[0] * nodes[1] * (ne_planes + 1))
    ne_nn = (0, 0, nn1, 0, 0)
    sub = nodes[0] * nodes[1] * 2
    dt = 4e-5
    box = [3, 15, 5, 12, 1, 5]
    rng = np.random.default_rng(11)
    rb = rng.standard_normal((box[5] - box[4], box[3] - box[2], box[1] - box[0])) * 1e-2
    V = np.zeros((nodes[2], nodes[1], nodes[0]))
    V[box[4]:box[5], box[2]:box[3], box[0]:box[1]] = rb
    _, _, k, rc = O.computeStateProperties(L1["T0"], L1["S1"], P, sub)
    F = O.computeConvRadBC(L1, L1["T0"], tmp[0], nn1, P, 0)
    ref = np.maximum(P["T_amb"], O.computeL1Temperature(L, ne_nn, tmp, F, V.reshape(-1), k, rc, dt, P))
    c = L1["conditions"]
    out = run(ps, shape, nn1, dtype, T_in=dev(L1["T0"], dtype), nodes=nodes, h=h, origin=o,
              ne_planes=ne_planes, dt=dev([dt], torch.float64), ph_in=phase_of(L1), substrate=sub,
              rhs_box=dev(rb, dtype), box=box, surface=1, bc_mode=1,
              face=[c["x"][0], c["x"][1], c["y"][0], c["y"][1], c["z"][0]], inactive_amb=1, clamp=1)
    assert relerr(out, ref) < tol


def test_separable_rejects_other_calls():
    """The separable kernel serves only constant-property calls of the subcycle
    feature sets: temperature-dependent properties are refused."""
    import _native as N
    import kern

    P = O.SetupProperties(PHASE_PROPS)
    ps = N.props_struct(P)
    n = 21 * 21 * 7
    T = torch.full((n,), 400.0, dtype=torch.float64, device="cuda")
    with pytest.raises(N.GomeltError):
        kern.level_step_shape(ps, kernel=1, rows=4, tile_y=1, zchunk=3, T_in=T, T_out=torch.empty_like(T),
                              nodes=(21, 21, 7), h=(0.1, 0.1, 0.1), origin=(0, 0, 0), ne_planes=6,
                              dt=dev([1e-5], torch.float64), ph_in=torch.zeros(n, dtype=torch.uint8, device="cuda"),
                              ph_out=torch.empty(n, dtype=torch.uint8, device="cuda"), surface=1, clamp=1,
                              bc_mode=3, bc_new=T, bc_old=T, bc_alpha=1.0,
                              laser=dev([0.5, 0.5, 0, 1, 1, 1e-5, 100.0], torch.float64))


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_tabulated_laser_factors_bit_identical(dtype):
    """The Level-3 step with the laser factors from gm_fine_source_tables
    equals the step that evaluates them itself, bit for bit."""
    import ctypes as C

    import _native as N
    import kern

    ps, nn, kw, _, _, _ = level3_case(CFG, 5, dtype, False)
    rows = torch.tensor([[1.01, 0.99, 0.0, 1, 1, 1.5e-6, 250.0], [1.013, 0.997, 0.0, 1, 1, 1.5e-6, 250.0]],
                        dtype=torch.float64, device="cuda")
    nodes = (C.c_int * 3)(*kw["nodes"])
    origin = (C.c_double * 3)(*kw["origin"])
    h = (C.c_double * 3)(*kw["h"])
    L = sum(kw["nodes"])
    tab = torch.empty(2 * L, dtype=dtype, device="cuda")
    N.call("gm_fine_source_tables", kern.dtype_code(tab), nodes, origin, h, rows.data_ptr(), 2, C.byref(ps),
           tab.data_ptr(), kern.stream_ptr())
    kw["laser"] = rows[1]
    a = run(ps, (1, 2, 4, 5), nn, dtype, ph_out=torch.empty(nn, dtype=torch.uint8, device="cuda"), **kw)
    kw["src_tab"] = tab[L:]
    b = run(ps, (1, 2, 4, 5), nn, dtype, ph_out=torch.empty(nn, dtype=torch.uint8, device="cuda"), **kw)
    np.testing.assert_array_equal(a, b)


# tiny Level-3 windows: 2 node planes, 2 node rows (all on the Dirichlet ring), 4 node columns
SMALL = [
    {"elements": [3, 2, 1], "bounds": {"x": [0.99, 1.005], "y": [0.99, 1.0], "z": [-0.005, 0]}},
    {"elements": [40, 1, 3], "bounds": {"x": [0.95, 1.15], "y": [0.99, 0.995], "z": [-0.015, 0]}},
    {"elements": [5, 7, 2], "bounds": {"x": [0.99, 1.015], "y": [0.98, 1.015], "z": [-0.01, 0]}},
]


@pytest.mark.parametrize("l3", range(len(SMALL)))
@pytest.mark.parametrize("shape", [(None, 0, 0, 0), (1, 2, 2, 2), (1, 4, 1, 5), (1, 1, 8, 3)])
@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_level3_small_grids(l3, shape, dtype, tol):
    ps, nn, kw, ref, (S1n, S2n), _ = level3_case(dict(CFG, Level3=SMALL[l3]), 6 + l3, dtype, False)
    ph_out = torch.empty(nn, dtype=torch.uint8, device="cuda")
    out = run(ps, shape, nn, dtype, ph_out=ph_out, **kw)
    assert relerr(out, ref) < tol
    ph = ph_out.cpu().numpy()
    np.testing.assert_array_equal(ph & 1, S1n.astype(np.uint8))
    np.testing.assert_array_equal((ph >> 1) & 1, S2n.astype(np.uint8))
