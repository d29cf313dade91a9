"""GPU parity of the fused level step against the oracle (FP64 and FP32)."""

import numpy as np
import pytest
import torch

import gomelt_oracle as O

pytestmark = pytest.mark.gpu

CFG = {
    "Level1": {"elements": [20, 20, 6], "bounds": {"x": [0, 2.0], "y": [0, 2.0], "z": [-0.6, 0]},
               "conditions": {"x": [300, 310], "y": [305, 300], "z": [300, 300]}},
    "Level2": {"elements": [40, 40, 10], "bounds": {"x": [0.6, 1.4], "y": [0.6, 1.4], "z": [-0.2, 0]}},
    "Level3": {"elements": [80, 40, 12], "bounds": {"x": [0.8, 1.2], "y": [0.9, 1.1], "z": [-0.06, 0]}},
}
PHASE_PROPS = {
    "thermal_conductivity_powder": 0.4, "thermal_conductivity_bulk_a0": 4.23,
    "thermal_conductivity_bulk_a1": 0.016, "thermal_conductivity_fluid_a0": 29.0,
    "heat_capacity_solid_a0": 383.1, "heat_capacity_solid_a1": 0.174, "heat_capacity_mushy": 3235.0,
    "heat_capacity_fluid": 769.0, "density": 8e-06, "laser_radius": 0.04, "laser_depth": 0.03,
    "laser_power": 250.0, "laser_absorptivity": 0.45, "T_amb": 298.15, "T_solidus": 1533,
    "T_liquidus": 1609, "T_boiling": 3038.0, "h_conv": 1.5e-05, "emissivity": 0.3,
    "evaporation_coefficient": 0.82, "layer_height": 0.02,
}


def setup(seed=0):
    import _native as N

    P = O.SetupProperties(PHASE_PROPS)
    L = O.SetupLevels(CFG, P)
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


def dev(a, dtype):
    return torch.as_tensor(np.asarray(a), dtype=dtype, device="cuda").contiguous()


def phase_of(L):
    return torch.as_tensor(((np.asarray(L["S1"]) > 0.499) * 1 + np.asarray(L["S2"]) * 2).astype(np.uint8),
                           device="cuda")


def geom(L):
    o = [float(np.asarray(c)[0]) for c in L["node_coords"]]
    h = [float(np.asarray(c)[1] - np.asarray(c)[0]) for c in L["node_coords"]]
    return [int(n) for n in L["nodes"]], h, o


def relerr(a, b):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 2e-6)])
@pytest.mark.parametrize("lev,partial", [(3, False), (1, True)])
def test_raw_solve(dtype, tol, lev, partial):
    import kern

    P, L, ps = setup()
    nodes, h, o = geom(L[lev])
    nn = int(np.prod(nodes))
    ne_planes = nodes[2] - 1 - (2 if partial else 0)
    ne = (nodes[0] - 1) * (nodes[1] - 1) * ne_planes
    rng = np.random.default_rng(3)
    k = rng.uniform(0.005, 0.03, nn)
    rc = rng.uniform(0.002, 0.005, nn)
    F = rng.standard_normal(nn) * 1e-3
    Cr = rng.standard_normal(nn) * 1e-4
    dt = 2e-6
    ref = O.solveMatrixFreeFE(L[lev], nn, ne, k, rc, dt, L[lev]["T0"], F, Cr)
    T_in = dev(L[lev]["T0"], dtype)
    T_out = torch.empty_like(T_in)
    dtd = torch.tensor([dt], dtype=torch.float64, device="cuda")
    kern.level_step(ps, T_in=T_in, T_out=T_out, nodes=nodes, h=h, origin=o, ne_planes=ne_planes, dt=dtd,
                    k_arr=dev(k, dtype), rc_arr=dev(rc, dtype), F_full=dev(F, dtype), corr_full=dev(Cr, dtype))
    out = T_out.cpu().numpy()
    ok = np.isfinite(ref)
    if dtype == torch.float64:
        np.testing.assert_array_equal(np.isfinite(out), ok)
    assert relerr(out[ok], ref[ok]) < tol


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
@pytest.mark.parametrize("zchunk", [0, 5])
def test_fused_fine_step(dtype, tol, zchunk):
    """Level 3 step: phase/props + laser source + surface flux (evaporation on)
    + Dirichlet ring from a blended, prolongated Level-2 field + clamp + melt time."""
    import kern
    from geometry import axis_map

    P, L, ps = setup(1)
    L3, L2 = L[3], L[2]
    nodes, h, o = geom(L3)
    nn3, ne3 = int(L3["nn"]), int(L3["ne"])
    ne_nn = (int(L2["ne"]), ne3, int(L[1]["nn"]), int(L2["nn"]), nn3)
    sub = nodes[0] * nodes[1] * 4
    v = np.array([1.013, 0.997, 0.0, 1, 1, 1.5e-6, 250.0])
    dt = v[5]
    T2old = np.asarray(L2["T0"])
    T2new = T2old + 50 * np.random.default_rng(5).standard_normal(T2old.shape)
    alpha = 0.3
    # oracle
    S1n, S2n, k, rc = O.computeStateProperties(L3["T0"], L3["S1"], P, sub)
    F = O.computeSourcesL3(L3, v, ne_nn, P, v[6])
    F = O.computeConvRadBC(L3, L3["T0"], ne3, nn3, P, F)
    BC = alpha * T2new + (1 - alpha) * T2old
    C2F = O.interpolatePointsMatrix(L2, L3["node_coords"])
    ref = np.maximum(P["T_amb"], O.computeSolutions_L3(BC, C2F, L, ne_nn, L3["T0"], F, k, rc, dt))
    acc0 = np.random.default_rng(7).uniform(0, 1e-4, nn3)
    macc0 = np.random.default_rng(8).uniform(0, 1e-4, nn3)
    reset = ((1 - 2 * np.asarray(L3["S2"], dtype=float)) * S2n) == 1
    racc = acc0 * reset
    macc_ref = np.maximum(racc, macc0)
    acc_ref = acc0 + dt * S2n - racc
    # device
    bcmap = kern.DeviceMap3([axis_map(L2["node_coords"][d], L3["node_coords"][d]) for d in range(3)],
                            [int(x) for x in L2["nodes"]], dtype)
    T_in = dev(L3["T0"], dtype)
    T_out = torch.empty_like(T_in)
    ph_in = phase_of(L3)
    ph_out = torch.empty_like(ph_in)
    acc = dev(acc0, dtype)
    macc = dev(macc0, dtype)
    kern.level_step(ps, T_in=T_in, T_out=T_out, nodes=nodes, h=h, origin=o, ne_planes=nodes[2] - 1,
                    dt=dev([dt], torch.float64), ph_in=ph_in, ph_out=ph_out, substrate=sub,
                    laser=dev(v, torch.float64), surface=1, bc_mode=2, bc_new=dev(T2new, dtype),
                    bc_old=dev(T2old, dtype), bc_alpha=alpha, bc_beta=1 - alpha, bc_map=bcmap, clamp=1,
                    accum=acc, max_accum=macc, zchunk=zchunk)
    out = T_out.cpu().numpy()
    assert relerr(out, ref) < tol
    ph = ph_out.cpu().numpy()
    np.testing.assert_array_equal(ph & 1, S1n.astype(np.uint8))
    np.testing.assert_array_equal((ph >> 1) & 1, S2n.astype(np.uint8))
    # FP32 evaluates the reference's (acc + dt*S2) - reset*acc in single precision
    atol = 1e-16 if dtype == torch.float64 else 1e-10
    np.testing.assert_allclose(acc.cpu().numpy(), acc_ref, rtol=1e-6, atol=atol)
    np.testing.assert_allclose(macc.cpu().numpy(), macc_ref, rtol=1e-6, atol=atol)


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_fused_coarse_step(dtype, tol):
    """Level 1 step: inactive top planes, constant Dirichlet faces, surface flux
    on the top active plane, extra RHS on a box."""
    import kern

    P, L, ps = setup(2)
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
    S1n, S2n, k, rc = O.computeStateProperties(L1["T0"], L1["S1"], P, sub)
    F = O.computeConvRadBC(L1, L1["T0"], tmp[0], nn1, P, 0)
    ref = np.maximum(P["T_amb"], O.computeL1Temperature(L, ne_nn, tmp, F, V.reshape(-1), k, rc, dt, P))
    T_in = dev(L1["T0"], dtype)
    T_out = torch.empty_like(T_in)
    c = L1["conditions"]
    kern.level_step(ps, T_in=T_in, T_out=T_out, nodes=nodes, h=h, origin=o, ne_planes=ne_planes,
                    dt=dev([dt], torch.float64), ph_in=phase_of(L1), substrate=sub, rhs_box=dev(rb, dtype),
                    box=box, surface=1, bc_mode=1, face=[c["x"][0], c["x"][1], c["y"][0], c["y"][1], c["z"][0]],
                    inactive_amb=1, clamp=1)
    assert relerr(T_out.cpu().numpy(), ref) < tol
