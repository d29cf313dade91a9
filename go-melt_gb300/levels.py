"""Host-side level geometry and bookkeeping (FP64, NumPy).

This is the part of GO-MELT that the reference also runs on the host or as
index arithmetic: input defaults, mesh set-up, window travel limits, the
integer shifts of the moving windows and the overlap index sets.  Device
fields (temperatures, phases, subgrid fields) are not stored here.

Levels follow the reference's ``SetupLevels`` (go_melt/computeFunctions.py
:115-264): Level 1 is the part, Level 2 and Level 3 are windows that follow
the laser, Level 0 is the part footprint at Level-3 resolution holding the
solidified (S1) state.
"""

from __future__ import annotations

import copy

import numpy as np


def setup_properties(p: dict) -> dict:
    """Defaults, unit fixes and derived coefficients (SetupProperties, :267-345)."""
    d = dict(p)
    g = p.get
    d.update(
        k_powder=g("thermal_conductivity_powder", 0.4),
        k_bulk_coeff_a0=g("thermal_conductivity_bulk_a0", 4.23),
        k_bulk_coeff_a1=g("thermal_conductivity_bulk_a1", 0.016),
        k_fluid_coeff_a0=g("thermal_conductivity_fluid_a0", 29.0),
        cp_solid_coeff_a0=g("heat_capacity_solid_a0", 383.1),
        cp_solid_coeff_a1=g("heat_capacity_solid_a1", 0.174),
        cp_mushy=g("heat_capacity_mushy", 3235.0),
        cp_fluid=g("heat_capacity_fluid", 769.0),
        rho=g("density", 8.0e-6),
        laser_radius=g("laser_radius", 0.110),
        laser_depth=g("laser_depth", 0.05),
        laser_power=g("laser_power", 300.0),
        laser_eta=g("laser_absorptivity", 0.25),
        laser_center=g("laser_center", []),
        T_amb=g("T_amb", 353.15),
        T_solidus=g("T_solidus", 1554.0),
        T_liquidus=g("T_liquidus", 1625.0),
        T_boiling=g("T_boiling", 3038.0),
        h_conv=g("h_conv", 1.473e-5) * 1e6,  # the reference stores W/m^2K (:318-319)
        vareps=g("emissivity", 0.600),
        evc=g("evaporation_coefficient", 0.82),
        kb=g("boltzmann_constant", 1.38e-23),
        mA=g("atomic_mass", 7.9485017e-26),
        Lev=g("latent_heat_evap", 4.22e6),
        molar_mass=g("molar_mass", 58.69) * 1e-3,
        layer_height=g("layer_height", 0.04),
        sigma_sb=5.67e-8,
        gas_const=8.314,
        atmospheric_pressure=101325,
    )
    d["CM_coeff"] = d["molar_mass"] / (2.0 * np.pi * d["gas_const"])
    d["CT_coeff"] = d["Lev"] * d["molar_mass"] / d["gas_const"]
    d["CP_coeff"] = 0.54 * d["atmospheric_pressure"]
    return d


NONMESH_DEFAULTS = {
    "timestep_L3": 1e-5, "subcycle_num_L2": 1, "subcycle_num_L3": 1, "dwell_time": 0.1,
    "Level1_record_step": 1, "save_path": "results/", "output_files": 1, "toolpath": "laserPath.txt",
    "wait_time": 500.0, "layer_num": 0, "restart_layer_num": 10000, "info_T": 0, "laser_velocity": 500,
    "wait_track": 0.0, "gcode": "./examples/gcodefiles/defaultName.gcode", "dwell_time_multiplier": 1,
    "use_txt": 0,
}


def setup_nonmesh(n: dict) -> dict:
    """SetupNonmesh (:348-419)."""
    d = dict(n)
    for k, v in NONMESH_DEFAULTS.items():
        d[k] = n.get(k, v)
    d["record_step"] = n.get("record_step", d["subcycle_num_L2"] * d["subcycle_num_L3"])
    return d


def linspace(a, b, n):
    return np.linspace(float(a), float(b), int(n))


def coarse_nodes_in_fine(xf, xc):
    """getCoarseNodesInFineRegion (:858-888)."""
    hc = (xc.max() - xc.min()) / (xc.size - 1)
    lo = np.round((xf.min() - xc.min()) / hc)
    hi = np.round((xf.max() - xc.min()) / hc) + 1
    return np.arange(lo, hi).astype(np.int64)


def fine_nodes_at_coarse(xc, xf):
    """getCoarseNodesInLargeFineRegion (:891-925)."""
    hf = (xf.max() - xf.min()) / (xf.size - 1)
    hc = (xc.max() - xc.min()) / (xc.size - 1)
    lo = np.round((xc.min() - xf.min()) / hf)
    hi = np.round((xc.max() - xf.min()) / hf) + 1
    return np.arange(lo, hi, int(np.round(hc / hf))).astype(np.int64)


def _trunc(x) -> int:
    return int(np.trunc(x))


class Level:
    """Geometry of one structured level (node coordinates per axis)."""

    def __init__(self, elements, bounds):
        self.elements = [int(e) for e in elements]
        self.nodes = [e + 1 for e in self.elements]
        self.bounds = {k: [float(v[0]), float(v[1])] for k, v in bounds.items()}
        self.length = [self.bounds[a][1] - self.bounds[a][0] for a in "xyz"]
        self.h = [self.length[i] / self.elements[i] for i in range(3)]
        self.init_coords = [linspace(self.bounds[a][0], self.bounds[a][1], self.nodes[i])
                            for i, a in enumerate("xyz")]
        self.coords = copy.deepcopy(self.init_coords)

    @property
    def nn(self):
        return self.nodes[0] * self.nodes[1] * self.nodes[2]

    @property
    def ne(self):
        return self.elements[0] * self.elements[1] * self.elements[2]

    def origin(self):
        return [float(c[0]) for c in self.coords]

    def spacing(self):
        return [float(c[1] - c[0]) for c in self.coords]


class Geometry:
    """All four levels plus the moving-window state, as in SetupLevels."""

    def __init__(self, solver_input: dict, props: dict):
        P = props
        self.props = P
        L1 = Level(solver_input["Level1"]["elements"], solver_input["Level1"]["bounds"])
        L2 = Level(solver_input["Level2"]["elements"], solver_input["Level2"]["bounds"])
        L3 = Level(solver_input["Level3"]["elements"], solver_input["Level3"]["bounds"])
        cond = solver_input["Level1"].get("conditions", {"x": [P["T_amb"]] * 2, "y": [P["T_amb"]] * 2,
                                                          "z": [P["T_amb"]] * 2})
        self.conditions = {k: [float(v[0]), float(v[1])] for k, v in cond.items()}
        self.L = [None, L1, L2, L3]
        self.s1_storage_rows = int(round(L1.h[2] / P["layer_height"]))
        # travel limits of the windows inside Level 1 (find_max_const, :1886-1913)
        for Lw in (L2, L3):
            b, c = L1.bounds, Lw.bounds
            Lw.limits = [[b["x"][0] - c["x"][0], b["x"][1] - c["x"][1]],
                         [b["y"][0] - c["y"][0], b["y"][1] - c["y"][1]],
                         [b["z"][0] - c["z"][0], b["z"][1] - c["z"][1]]]
        # Level 1 is shifted by layer heights until a node meets Level 2's top (:176-182)
        L1.orig_coords = copy.deepcopy(L1.coords)
        z = L1.orig_coords[2].copy()
        while not np.isclose(z - L2.coords[2][-1], 0, atol=1e-4).any():
            z = z + P["layer_height"]
        L1.coords[2] = z
        # overlap node sets (:184-209)
        L2.orig_overlap_nodes = [coarse_nodes_in_fine(L2.coords[i], L1.coords[i]) for i in range(3)]
        L2.orig_overlap_coors = [L1.coords[i][L2.orig_overlap_nodes[i]] for i in range(3)]
        L3.orig_overlap_nodes = [coarse_nodes_in_fine(L3.coords[i], L2.coords[i]) for i in range(3)]
        L3.orig_overlap_coors = [L2.coords[i][L3.orig_overlap_nodes[i]] for i in range(3)]
        for Lw in (L2, L3):
            Lw.overlap_nodes = copy.deepcopy(Lw.orig_overlap_nodes)
            Lw.overlap_coords = copy.deepcopy(Lw.orig_overlap_coors)
        # Level 0 (:211-246)
        e0 = [round(L1.length[0] / L3.h[0]), round(L1.length[1] / L3.h[1]), round(L2.length[2] / L3.h[2])]
        self.L0_nodes = [e + 1 for e in e0]
        L0c = [linspace(L1.bounds["x"][0], L1.bounds["x"][1], self.L0_nodes[0]),
               linspace(L1.bounds["y"][0], L1.bounds["y"][1], self.L0_nodes[1]),
               linspace(L2.bounds["z"][0], L2.bounds["z"][1], self.L0_nodes[2])]
        self.L0_coords = L0c
        self.L0_orig_coords = copy.deepcopy(L0c)
        self.L0_orig_overlap = [coarse_nodes_in_fine(L3.coords[i], L0c[i]) for i in range(3)]
        self.L0_orig_overlap_L2 = [fine_nodes_at_coarse(L2.coords[i], L0c[i]) for i in range(3)]
        self.L0_overlap = copy.deepcopy(self.L0_orig_overlap)
        self.L0_overlap_L2 = copy.deepcopy(self.L0_orig_overlap_L2)
        self.layer_idx_delta = int(round(P["layer_height"] / L3.h[2]))
        # element ratios used by the driver's move logic (go_melt.py:42-49)
        self.L1L2Eratio = [int(np.round(L1.h[i] / L2.h[i])) for i in range(2)] + [
            int(np.round(P["layer_height"] / L2.h[2]))]
        self.L2L3Eratio = [int(np.round(L2.h[i] / L3.h[i])) for i in range(3)]

    @property
    def L0_nn(self):
        return self.L0_nodes[0] * self.L0_nodes[1] * self.L0_nodes[2]

    # -- static counts -------------------------------------------------
    def ne_nn(self):
        """getStaticNodesAndElements (:447-470)."""
        L = self.L
        return (L[2].ne, L[3].ne, L[1].nn, L[2].nn, L[3].nn)

    def tmp_ne_nn(self, v):
        """calcStaticTmpNodesAndElements (:495-517)."""
        L1 = self.L[1]
        n = int((L1.coords[2] <= v[2] + 1e-5).sum())
        return (L1.elements[0] * L1.elements[1] * (n - 1), L1.nodes[0] * L1.nodes[1] * n)

    def substrate(self):
        """getSubstrateNodes (:562-579), Level 0 counted as 0 planes like the reference does
        from its own z coordinates."""
        out = [int((self.L0_coords[2] < 1e-5).sum()) * self.L0_nodes[0] * self.L0_nodes[1]]
        for lev in (1, 2, 3):
            L = self.L[lev]
            out.append(int((L.coords[2] < 1e-5).sum()) * L.nodes[0] * L.nodes[1])
        return tuple(out)

    # -- moving windows (moveEverything, :2400-2510) ---------------------
    def move(self, v, vstart):
        """Shift Level 3 (by Level-2 cells) and Level 2 (by Level-1 cells in x, y
        and layer heights in z) after the laser; update overlap sets.

        Returns the new coordinates of both windows (old ones remain in
        self.L[...].coords until ``commit_move``) and the Level-2 move in
        Level-2 cells."""
        P = self.props
        L1, L2, L3 = self.L[1], self.L[2], self.L[3]
        vtot = np.asarray(v, dtype=float)[:3] - np.asarray(vstart, dtype=float)[:3]
        v3 = [float(np.clip(vtot[d], L3.limits[d][0], L3.limits[d][1])) for d in range(3)]
        v2 = [float(np.clip(vtot[d], L2.limits[d][0], L2.limits[d][1])) for d in range(3)]
        h2 = L2.h  # the reference moves with the set-up spacings (Levels[i]["h"])
        h1 = L1.h
        s3 = [_trunc(v3[d] / h2[d] + 1e-2) for d in range(3)]
        new3 = [L3.init_coords[d] + h2[d] * s3[d] for d in range(3)]
        L3.overlap_nodes = [L3.orig_overlap_nodes[d] + s3[d] for d in range(3)]
        L3.overlap_coords = [L3.orig_overlap_coors[d] + h2[d] * s3[d] for d in range(3)]
        height = P["layer_height"]
        es2 = [h1[0], h1[1], height]
        s2m = [_trunc(v2[d] / es2[d] + 1e-2) for d in range(3)]
        new2 = [L2.init_coords[d] + es2[d] * s2m[d] for d in range(3)]
        move_v = [s2m[d] * self.L1L2Eratio[d] for d in range(3)]
        s2 = [_trunc(v2[d] / h1[d] + 1e-2) for d in range(3)]
        szp = height * _trunc(v2[2] / height + 1e-2)
        L2.overlap_nodes = [L2.orig_overlap_nodes[0] + s2[0], L2.orig_overlap_nodes[1] + s2[1],
                            L2.orig_overlap_nodes[2] + s2[2]]
        L2.overlap_coords = [L2.orig_overlap_coors[0] + h1[0] * s2[0], L2.orig_overlap_coors[1] + h1[1] * s2[1],
                             L2.orig_overlap_coors[2] + szp]
        L3.overlap_nodes = [L3.overlap_nodes[d] - move_v[d] for d in range(3)]
        r12, r23 = self.L1L2Eratio, self.L2L3Eratio
        self.L0_overlap = [self.L0_orig_overlap[d] + r23[d] * s3[d] for d in range(3)]
        e0 = [h1[0], h1[1], h2[2]]
        s0 = [_trunc(v2[d] / e0[d] + 1e-2) for d in range(3)]
        rr = [r12[0] * r23[0], r12[1] * r23[1], r23[2]]
        self.L0_overlap_L2 = [self.L0_orig_overlap_L2[d] + rr[d] * s0[d] for d in range(3)]
        self.L0_overlap[2] = self.L0_overlap[2] - move_v[2] * r23[2]
        self.L0_overlap_L2[2] = self.L0_overlap_L2[2] - move_v[2] * r23[2]
        return new3, new2, move_v

    def layer_shift_L1(self, laser_z):
        """Level-1 z coordinates for a new layer at height laser_z (go_melt.py
        :208-221): shift the original coordinates by layer heights until a node
        is within 1e-4 of the laser height.  Returns (coords_z, state_index)."""
        z = self.L[1].orig_coords[2].copy()
        idx = 0
        while not np.isclose(z - laser_z, 0, atol=1e-4).any():
            z = z + self.props["layer_height"]
            idx += 1
        return z, idx
