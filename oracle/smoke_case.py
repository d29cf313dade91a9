"""Smoke check used by __graft_entry__.smoke(): one small moveEverything +
subcycleGOMELT on the GPU engine against the NumPy oracle (test
infrastructure; the oracle gives the expected values here, it is not the thing measured)."""

from __future__ import annotations

import copy

import numpy as np

import gomelt_oracle as O

CFG = {
    "Level1": {"elements": [12, 12, 6], "bounds": {"x": [0, 1.2], "y": [0, 1.2], "z": [-0.6, 0]},
               "conditions": {"x": [300, 300], "y": [300, 300], "z": [300, 300]}},
    "Level2": {"elements": [12, 12, 6], "bounds": {"x": [0.3, 0.9], "y": [0.3, 0.9], "z": [-0.3, 0]}},
    "Level3": {"elements": [16, 16, 8], "bounds": {"x": [0.5, 0.7], "y": [0.5, 0.7], "z": [-0.1, 0]}},
    "properties": {
        "thermal_conductivity_powder": 22.0, "thermal_conductivity_bulk_a0": 22.0,
        "thermal_conductivity_bulk_a1": 0.0, "thermal_conductivity_fluid_a0": 22.0,
        "heat_capacity_solid_a0": 700.0, "heat_capacity_solid_a1": 0.0, "heat_capacity_mushy": 700.0,
        "heat_capacity_fluid": 700.0, "density": 4.4e-6, "laser_radius": 0.05, "laser_depth": 0.05,
        "laser_power": 200.0, "laser_absorptivity": 0.35, "T_amb": 300.0, "T_solidus": 1878.0,
        "T_liquidus": 1900.0, "h_conv": 1e-5, "emissivity": 0.3, "evaporation_coefficient": 0.0,
        "layer_height": 0.05, "laser_center": [0.6, 0.6, 0.0, 0, 0, 0, 0],
    },
}
N2, N3 = 2, 3


def rows():
    dt = 5e-6
    r = np.zeros((N2 * N3, 7))
    r[:, 0] = 0.61 + 1e3 * dt * np.arange(1, N2 * N3 + 1)
    r[:, 1] = 0.6
    r[:, 3] = 1
    r[:, 4] = 1
    r[:, 5] = dt
    r[:, 6] = 200.0
    return r


def run(device):
    import torch

    from engine import Engine

    R = rows()
    vstart = np.array(CFG["properties"]["laser_center"], dtype=float)
    # oracle
    P = O.SetupProperties(CFG["properties"])
    L = O.SetupLevels(copy.deepcopy(CFG), P)
    r12 = [int(np.round(L[1]["h"][i] / L[2]["h"][i])) for i in range(2)] + [
        int(np.round(P["layer_height"] / L[2]["h"][2]))]
    r23 = [int(np.round(L[2]["h"][i] / L[3]["h"][i])) for i in range(3)]
    L, shapes, interp, _ = O.moveEverything(R[0], vstart, L, [0, 0, 0], [None, None], r12, r23, P["layer_height"])
    ne_nn = O.getStaticNodesAndElements(L)
    tmp = O.calcStaticTmpNodesAndElements(L, R[0])
    sub = O.getSubstrateNodes(L)
    nn3 = ne_nn[4]
    L, *_ = O.subcycleGOMELT(L, ne_nn, shapes, sub, interp, tmp, R, P, R[:, 6],
                             (N2, N3, N2 * N3, float(N2), float(N3), float(N2 * N3)), np.zeros(nn3), np.zeros(nn3))
    # GPU engine (FP32)
    eng = Engine(copy.deepcopy(CFG), O.SetupProperties(CFG["properties"]), N2, N3, dtype=torch.float32,
                 device=device)
    eng.set_layer(R[0])
    eng.move(R[0], vstart)
    eng.subcycle(R)
    torch.cuda.synchronize(device)
    err = 0.0
    for lev in (1, 2, 3):
        ref = np.asarray(L[lev]["T0"])
        got = eng.T[lev].double().cpu().numpy()
        err = max(err, float(np.max(np.abs(got - ref)) / np.max(np.abs(ref))))
    return err
