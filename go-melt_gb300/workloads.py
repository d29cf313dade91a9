"""Input files (the reference's JSON schema) of the benchmark workloads.

All use a constant-property material (k = 22 W/mK, rho = 4400 kg/m^3,
cp = 700 J/kgK in every phase), a 200 W Gaussian laser of radius 50 um and
absorptivity 0.35 moving at 1 m/s, convection h = 10 W/m^2K and radiation with
emissivity 0.3 on the top surface, 300 K Dirichlet faces and 300 K initial
temperature.  The reference always adds evaporation (computeConvRadBC,
go_melt/computeFunctions.py:2284-2287); these workloads name convection and
radiation only, so evaporation_coefficient = 0.  laser_depth is not given by
the workload descriptions: the reference default 0.05 mm is used.

The fine time step is 0.9 x the explicit limit of the lumped hex8 operator on
the finest level, h^2 / (2 alpha) with alpha = k / (rho cp): 1.575 us at 5 um.
Level-2 and Level-1 steps are 10x and 100x longer (N2 = N3 = 10).
"""

from __future__ import annotations

import copy

MATERIAL = {
    "thermal_conductivity_powder": 22.0, "thermal_conductivity_bulk_a0": 22.0,
    "thermal_conductivity_bulk_a1": 0.0, "thermal_conductivity_fluid_a0": 22.0,
    "heat_capacity_solid_a0": 700.0, "heat_capacity_solid_a1": 0.0, "heat_capacity_mushy": 700.0,
    "heat_capacity_fluid": 700.0, "density": 4.4e-6,
    "laser_radius": 0.05, "laser_depth": 0.05, "laser_power": 200.0, "laser_absorptivity": 0.35,
    "T_amb": 300.0, "T_solidus": 1878.0, "T_liquidus": 1900.0, "T_boiling": 3038.0,
    "h_conv": 1e-5, "emissivity": 0.3, "evaporation_coefficient": 0.0, "layer_height": 0.05,
}

ALPHA = 0.022 / (4.4e-6 * 700.0)  # mm^2/s


def dt_fine(h):
    return 0.9 * h * h / (2.0 * ALPHA)


def _cond(T=300.0):
    return {"x": [T, T], "y": [T, T], "z": [T, T]}


def single_track():
    """Single 4 mm track on a 5x5x1 mm block (L1 50x50x10 @ 100 um, L2 1x1x0.2 mm
    window 50x50x10 @ 20 um, L3 0.4x0.4x0.1 mm window 80x80x20 @ 5 um)."""
    return {
        "Level1": {"elements": [50, 50, 10], "bounds": {"x": [0.0, 5.0], "y": [0.0, 5.0], "z": [-1.0, 0.0]},
                   "conditions": _cond()},
        "Level2": {"elements": [50, 50, 10], "bounds": {"x": [0.0, 1.0], "y": [2.0, 3.0], "z": [-0.2, 0.0]}},
        "Level3": {"elements": [80, 80, 20], "bounds": {"x": [0.3, 0.7], "y": [2.3, 2.7], "z": [-0.1, 0.0]}},
        "properties": dict(copy.deepcopy(MATERIAL), laser_center=[0.5, 2.5, 0.0, 0, 0, 0, 0]),
        "nonmesh": {"timestep_L3": dt_fine(0.005), "subcycle_num_L2": 10, "subcycle_num_L3": 10,
                    "laser_velocity": 1000.0, "output_files": 0, "wait_time": 10, "dwell_time": 1e-4,
                    "info_T": 0},
        "gcode": "G0 X0.5 Y2.5 Z0.0\nG1 X4.5 Y2.5 Z0.0\n",
    }


def part_scale_raster():
    """Part-scale raster: L1 20x20x5 mm, 200x200x50 @ 100 um; L2 2x2x0.3 mm window,
    100x100x15 @ 20 um; L3 0.8x0.8x0.2 mm window, 160x160x40 @ 5 um (element counts:
    with these the windows sit on the coarser grids' nodes, which the reference's
    overlap and restriction logic needs); serpentine tracks 100 um apart, centred
    in the part, first layer."""
    return {
        "Level1": {"elements": [200, 200, 50], "bounds": {"x": [0.0, 20.0], "y": [0.0, 20.0], "z": [-5.0, 0.0]},
                   "conditions": _cond()},
        "Level2": {"elements": [100, 100, 15], "bounds": {"x": [9.0, 11.0], "y": [9.0, 11.0], "z": [-0.3, 0.0]}},
        "Level3": {"elements": [160, 160, 40], "bounds": {"x": [9.6, 10.4], "y": [9.6, 10.4], "z": [-0.2, 0.0]}},
        "properties": dict(copy.deepcopy(MATERIAL), laser_center=[10.0, 10.0, 0.0, 0, 0, 0, 0]),
        "nonmesh": {"timestep_L3": dt_fine(0.005), "subcycle_num_L2": 10, "subcycle_num_L3": 10,
                    "laser_velocity": 1000.0, "output_files": 0, "wait_time": 10, "dwell_time": 1e-4,
                    "info_T": 0},
        "raster": {"x0": 8.0, "y0": 8.0, "length": 4.0, "hatch": 0.1, "ntracks": 40},
    }


def part_scale_layers(layers=3, ntracks=40, length=4.0, l1_xy=20.0):
    """The part-scale raster over several layers of 50 um: Level 1 extended to
    z = 0.3 mm above the part top (53 element planes; the elements above the
    current layer are inactive), serpentine layers at z = 0.05, 0.10, ... mm.
    The Level-2 window keeps its 2 x 2 x 0.3 mm extent with 12 element planes
    (25 um) instead of 15 (20 um): a new layer moves the windows up by one
    layer height in whole Level-2 cells (the driver's integer ratio
    round(layer_height / h2z), go_melt.py:42-44), which 20 um cells (2.5 a
    layer) cannot do, and the Level-3 overlap would leave Level 2.
    ``l1_xy`` < 20 crops Level 1 (and with it Level 0) to a square of that size
    around the windows, for tests."""
    import createPath

    c = part_scale_raster()
    c["Level2"]["elements"] = [100, 100, 12]
    lo = 10.0 - l1_xy / 2
    ne = int(round(l1_xy / 0.1))
    c["Level1"] = {"elements": [ne, ne, 53], "bounds": {"x": [lo, lo + l1_xy], "y": [lo, lo + l1_xy], "z": [-5.0, 0.3]},
                   "conditions": _cond()}
    x0 = 10.0 - length / 2
    y0 = 10.0 - (ntracks - 1) * 0.05
    c["raster"] = {"x0": x0, "y0": y0, "length": length, "hatch": 0.1, "ntracks": ntracks, "layers": layers}
    c["gcode"] = createPath.serpentine_gcode(x0, y0, length, 0.1, ntracks, z=0.05, layers=layers, layer_height=0.05)
    return c


def precision_window():
    """Precision study: the part-scale raster with a fine Level-3 window of 0.5 x 0.5 x 0.1 mm
    at 2.5 um (200 x 200 x 40 elements; Level-2 to Level-3 ratio 8), placed on
    Level-2 nodes around the raster start.  dt3 = 0.394 us."""
    c = part_scale_raster()
    c["Level3"] = {"elements": [200, 200, 40], "bounds": {"x": [9.76, 10.26], "y": [9.76, 10.26], "z": [-0.1, 0.0]}}
    c["nonmesh"]["timestep_L3"] = dt_fine(0.0025)
    return c


def batched_instances(n=64, seed=0):
    """Batched single-track instances: Level-1 meshes of U{30..120} x U{30..120}
    x U{8..20} elements at 100 um, Level-2 / Level-3 windows as in the single track
    (1 x 1 x 0.2 mm at 20 um, 0.4 x 0.4 x 0.1 mm at 5 um); laser power
    U[100, 400] W, speed U[0.5, 1.5] m/s, radius U[35, 70] um, track angle
    U[0, 180) deg; the track is centred with length min(4 mm, what fits with
    0.6 mm to every edge).  numpy default_rng(seed); returns n input dicts."""
    import numpy as np

    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        ex, ey = (int(v) for v in rng.integers(30, 121, 2))
        ez = int(rng.integers(8, 21))
        P = float(rng.uniform(100.0, 400.0))
        vel = float(rng.uniform(500.0, 1500.0))
        r = float(rng.uniform(0.035, 0.070))
        ang = float(rng.uniform(0.0, 180.0))
        Lx, Ly = ex * 0.1, ey * 0.1
        cx, cy = 0.5 * Lx, 0.5 * Ly
        ux, uy = np.cos(np.radians(ang)), np.sin(np.radians(ang))
        m = 0.6
        lim = []
        for u, L in ((ux, Lx), (uy, Ly)):
            if abs(u) > 1e-9:
                lim.append((L - 2 * m) / abs(u))
        length = min([4.0] + lim)
        x0, y0 = cx - 0.5 * length * ux, cy - 0.5 * length * uy
        x1, y1 = cx + 0.5 * length * ux, cy + 0.5 * length * uy
        # windows around the track start, on the coarser grids' nodes
        bx2 = round(min(max(round((x0 - 0.5) / 0.1) * 0.1, 0.0), Lx - 1.0), 6)
        by2 = round(min(max(round((y0 - 0.5) / 0.1) * 0.1, 0.0), Ly - 1.0), 6)
        bx3 = round(min(max(bx2 + round((x0 - 0.2 - bx2) / 0.02) * 0.02, bx2), bx2 + 0.6), 6)
        by3 = round(min(max(by2 + round((y0 - 0.2 - by2) / 0.02) * 0.02, by2), by2 + 0.6), 6)
        props = dict(copy.deepcopy(MATERIAL), laser_power=P, laser_radius=r,
                     laser_center=[bx3 + 0.2, by3 + 0.2, 0.0, 0, 0, 0, 0])
        out.append({
            "Level1": {"elements": [ex, ey, ez], "bounds": {"x": [0.0, Lx], "y": [0.0, Ly], "z": [-0.1 * ez, 0.0]},
                       "conditions": _cond()},
            "Level2": {"elements": [50, 50, 10],
                       "bounds": {"x": [bx2, bx2 + 1.0], "y": [by2, by2 + 1.0], "z": [-0.2, 0.0]}},
            "Level3": {"elements": [80, 80, 20],
                       "bounds": {"x": [bx3, bx3 + 0.4], "y": [by3, by3 + 0.4], "z": [-0.1, 0.0]}},
            "properties": props,
            "nonmesh": {"timestep_L3": dt_fine(0.005), "subcycle_num_L2": 10, "subcycle_num_L3": 10,
                        "laser_velocity": vel, "output_files": 0, "wait_time": 10, "dwell_time": 1e-4,
                        "info_T": 0},
            "gcode": f"G0 X{x0:.4f} Y{y0:.4f} Z0.0000\nG1 X{x1:.4f} Y{y1:.4f} Z0.0000\n",
            "instance": {"power": P, "speed": vel, "radius": r, "angle": ang, "length": length},
        })
    return out
