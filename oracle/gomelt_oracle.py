"""CPU oracle: NumPy FP64 restatement of GO-MELT's multilevel explicit thermal step.

TEST INFRASTRUCTURE.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
legs of ``bench.py`` use this module, and only as the expected values / CPU baseline;
the product (``go-melt_gb300/``) never imports it.

Each function restates the reference function of the same name in
``go_melt/computeFunctions.py`` (JLnorthwestern/GO-MELT), vectorised over
elements/points with NumPy instead of ``jax.vmap``, keeping the reference's data
model (``Levels`` = list of four dicts) and its arithmetic (same formulas, same
element-mean properties, same validity-masked interpolation, same BCOO
projection through the coarse nodes of quadrature point 0).  Citations are
``file:line`` of that file unless another file is named.

Parity pin: ``tests/test_oracle_golden.py`` checks this module against golden
vectors produced by running the unmodified reference on the same inputs
(``tests/golden/make_golden.py``; JAX replaced by the NumPy primitives of
``oracle/jaxshim.py``).
"""

from __future__ import annotations

import copy
import json
import os

import numpy as np

SQ3 = np.sqrt(3.0)


# ---------------------------------------------------------------------------
# small helpers
# ---------------------------------------------------------------------------
def _i(x) -> int:
    return int(np.asarray(x).item())


def _f(x) -> float:
    return float(np.asarray(x).item())


def _arr(x):
    return np.asarray(x, dtype=float) if not isinstance(x, np.ndarray) else x


def elem_nodes(ex, ey, nx, ny, elems):
    """Node ids of hex8 elements, in the reference's local order.

    ``convert2XYZ`` (:645-689): element i -> (ix, iy, iz), base node
    ix + iy*nx + iz*nx*ny, local nodes base + {0, 1, 1+nx, nx} (+ nx*ny).
    Returns (len(elems), 8) and ix, iy, iz.
    """
    elems = np.asarray(elems)
    exy = ex * ey
    iz = elems // exy
    iy = elems // ex - iz * ey
    ix = elems % ex
    nxy = nx * ny
    base = ix + iy * nx + iz * nxy
    off = np.array([0, 1, 1 + nx, nx, nxy, 1 + nxy, 1 + nx + nxy, nx + nxy])
    return base[:, None] + off[None, :], ix, iy, iz


def level_dims(L):
    ex, ey, ez = (L["connect"][i].shape[0] for i in range(3))
    return ex, ey, ez, ex + 1, ey + 1, ez + 1


# ---------------------------------------------------------------------------
# Set-up (host side; :18-64, :115-579, :1886-1942)
# ---------------------------------------------------------------------------
def calcNumNodes(elements):
    """:18-29."""
    return [elements[0] + 1, elements[1] + 1, elements[2] + 1]


def createMesh3D(x, y, z):
    """:32-64: node coordinates (linspace) and per-axis 8-node connectivity."""
    nx, ny, nz = [np.linspace(*axis) for axis in (x, y, z)]
    cx0 = np.arange(0, x[2] - 1).reshape(-1, 1)
    cx1 = np.arange(1, x[2]).reshape(-1, 1)
    nconn_x = np.concatenate([cx0, cx1, cx1, cx0, cx0, cx1, cx1, cx0], axis=1)
    cy0 = np.arange(0, y[2] - 1).reshape(-1, 1)
    cy1 = np.arange(1, y[2]).reshape(-1, 1)
    nconn_y = np.concatenate([cy0, cy0, cy1, cy1, cy0, cy0, cy1, cy1], axis=1)
    cz0 = np.arange(0, z[2] - 1).reshape(-1, 1)
    cz1 = np.arange(1, z[2]).reshape(-1, 1)
    nconn_z = np.concatenate([cz0, cz0, cz0, cz0, cz1, cz1, cz1, cz1], axis=1)
    return [nx, ny, nz], [nconn_x, nconn_y, nconn_z]


def calc_length_h(bounds, elements):
    """:1916-1942."""
    L = [bounds[a][1] - bounds[a][0] for a in "xyz"]
    return L, [L[i] / elements[i] for i in range(3)]


def find_max_const(coarse_bounds, fine_bounds):
    """:1886-1913: signed travel limits of a window inside its parent (mm)."""
    iE = coarse_bounds["x"][1] - fine_bounds["x"][1]
    iN = coarse_bounds["y"][1] - fine_bounds["y"][1]
    iT = coarse_bounds["z"][1] - fine_bounds["z"][1]
    iW = coarse_bounds["x"][0] - fine_bounds["x"][0]
    iS = coarse_bounds["y"][0] - fine_bounds["y"][0]
    iB = coarse_bounds["z"][0] - fine_bounds["z"][0]
    return [iW, iE], [iS, iN], [iB, iT]


def getBCindices(nodes):
    """:520-559: [west, east, south, north, bottom, top] node ids."""
    nx, ny, nz = nodes
    nn = nx * ny * nz
    bidx = np.arange(0, nx * ny)
    tidx = np.arange(nx * ny * (nz - 1), nn)
    widx = np.arange(0, nn, nx)
    eidx = np.arange(nx - 1, nn, nx)
    sidx = (np.arange(0, nx)[:, None] + (nx * ny * np.arange(0, nz))[None, :]).reshape(-1)
    nidx = (np.arange(nx * (ny - 1), nx * ny)[:, None] + (nx * ny * np.arange(0, nz))[None, :]).reshape(-1)
    return [widx, eidx, sidx, nidx, bidx, tidx]


def getCoarseNodesInFineRegion(xnf, xnc):
    """:858-888: coarse node ids covering the extent of a fine axis."""
    xfmin, xfmax, xcmin, xcmax = xnf.min(), xnf.max(), xnc.min(), xnc.max()
    hc = (xcmax - xcmin) / (xnc.size - 1)
    lo = np.round((xfmin - xcmin) / hc)
    hi = np.round((xfmax - xcmin) / hc) + 1
    return np.arange(lo, hi).astype(int)


def getCoarseNodesInLargeFineRegion(xnc, xnf):
    """:891-925: fine (Level-0) node ids that coincide with coarse nodes."""
    xfmin, xfmax, xcmin, xcmax = xnf.min(), xnf.max(), xnc.min(), xnc.max()
    hf = (xfmax - xfmin) / (xnf.size - 1)
    hc = (xcmax - xcmin) / (xnc.size - 1)
    lo = np.round((xcmin - xfmin) / hf)
    hi = np.round((xcmax - xfmin) / hf) + 1
    step = int(np.round(hc / hf))
    return np.arange(lo, hi, step).astype(int)


def getOverlapRegion(node_ids, nx, ny):
    """:1642-1669: flattened ids of a tensor product of per-axis node ids."""
    x, y, z = (np.asarray(a) for a in node_ids)
    X = np.tile(x, y.shape[0] * z.shape[0]).reshape(-1)
    Y = np.repeat(np.tile(y, z.shape[0]), x.shape[0]).reshape(-1)
    Z = np.repeat(z, x.shape[0] * y.shape[0])
    return X + Y * _i(nx) + Z * _i(nx) * _i(ny)


def SetupProperties(p):
    """:267-345: defaults, unit fixes and derived evaporation coefficients."""
    q = dict(p)
    q["k_powder"] = p.get("thermal_conductivity_powder", 0.4)
    q["k_bulk_coeff_a0"] = p.get("thermal_conductivity_bulk_a0", 4.23)
    q["k_bulk_coeff_a1"] = p.get("thermal_conductivity_bulk_a1", 0.016)
    q["k_fluid_coeff_a0"] = p.get("thermal_conductivity_fluid_a0", 29.0)
    q["cp_solid_coeff_a0"] = p.get("heat_capacity_solid_a0", 383.1)
    q["cp_solid_coeff_a1"] = p.get("heat_capacity_solid_a1", 0.174)
    q["cp_mushy"] = p.get("heat_capacity_mushy", 3235.0)
    q["cp_fluid"] = p.get("heat_capacity_fluid", 769.0)
    q["rho"] = p.get("density", 8.0e-6)
    q["laser_radius"] = p.get("laser_radius", 0.110)
    q["laser_depth"] = p.get("laser_depth", 0.05)
    q["laser_power"] = p.get("laser_power", 300.0)
    q["laser_eta"] = p.get("laser_absorptivity", 0.25)
    q["laser_center"] = p.get("laser_center", [])
    q["T_amb"] = p.get("T_amb", 353.15)
    q["T_solidus"] = p.get("T_solidus", 1554.0)
    q["T_liquidus"] = p.get("T_liquidus", 1625.0)
    q["T_boiling"] = p.get("T_boiling", 3038.0)
    q["h_conv"] = p.get("h_conv", 1.473e-5) * 1e6  # :318-319
    q["vareps"] = p.get("emissivity", 0.600)
    q["evc"] = p.get("evaporation_coefficient", 0.82)
    q["kb"] = p.get("boltzmann_constant", 1.38e-23)
    q["mA"] = p.get("atomic_mass", 7.9485017e-26)
    q["Lev"] = p.get("latent_heat_evap", 4.22e6)
    q["molar_mass"] = p.get("molar_mass", 58.69) * 1e-3
    q["layer_height"] = p.get("layer_height", 0.04)
    q["sigma_sb"] = 5.67e-8
    q["gas_const"] = 8.314
    q["atmospheric_pressure"] = 101325
    q["CM_coeff"] = q["molar_mass"] / (2.0 * np.pi * q["gas_const"])
    q["CT_coeff"] = q["Lev"] * q["molar_mass"] / q["gas_const"]
    q["CP_coeff"] = 0.54 * q["atmospheric_pressure"]
    return q


NONMESH_DEFAULTS = {
    # :348-419
    "timestep_L3": 1e-5, "subcycle_num_L2": 1, "subcycle_num_L3": 1, "dwell_time": 0.1,
    "Level1_record_step": 1, "save_path": "results/", "output_files": 1,
    "toolpath": "laserPath.txt", "wait_time": 500.0, "layer_num": 0, "restart_layer_num": 10000,
    "info_T": 0, "laser_velocity": 500, "wait_track": 0.0,
    "gcode": "./examples/gcodefiles/defaultName.gcode", "dwell_time_multiplier": 1, "use_txt": 0,
}


def SetupNonmesh(n, make_dirs=False):
    """:348-419 (``record_step`` defaults to N2*N3)."""
    q = dict(n)
    for k, v in NONMESH_DEFAULTS.items():
        q[k] = n.get(k, v)
    q["record_step"] = n.get("record_step", q["subcycle_num_L2"] * q["subcycle_num_L3"])
    if make_dirs and not os.path.exists(q["save_path"]):
        os.makedirs(q["save_path"])
    return q


def SetupLevels(solver_input, properties):
    """:115-264: Levels[0..3] with meshes, fields, overlaps and Level 0."""
    P = properties
    lv = {}
    for name in ("Level1", "Level2", "Level3"):
        src = json.loads(json.dumps(solver_input.get(name, {})))
        L = {"elements": list(src["elements"]), "bounds": dict(src["bounds"])}
        if "conditions" in src:
            L["conditions"] = src["conditions"]
        L["length"], L["h"] = calc_length_h(L["bounds"], L["elements"])
        L["nodes"] = calcNumNodes(L["elements"])
        L["ne"] = L["elements"][0] * L["elements"][1] * L["elements"][2]
        L["nn"] = L["nodes"][0] * L["nodes"][1] * L["nodes"][2]
        L["BC"] = getBCindices(L["nodes"])
        b = L["bounds"]
        L["node_coords"], L["connect"] = createMesh3D(
            (b["x"][0], b["x"][1], L["nodes"][0]), (b["y"][0], b["y"][1], L["nodes"][1]),
            (b["z"][0], b["z"][1], L["nodes"][2]))
        nn = L["nn"]
        L["T"] = P["T_amb"] * np.ones(nn)
        L["T0"] = P["T_amb"] * np.ones(nn)
        L["S1"] = np.zeros(nn)
        L["S2"] = np.zeros(nn, dtype=bool)
        L["k"] = P["k_powder"] * np.ones(nn)
        L["rhocp"] = P["cp_solid_coeff_a0"] * P["rho"] * np.ones(nn)
        lv[name] = L
    L1, L2, L3 = lv["Level1"], lv["Level2"], lv["Level3"]
    L1["S1_storage"] = np.zeros([int(round(L1["h"][2] / P["layer_height"])), L1["nn"]])
    for L in (L2, L3):
        L["bounds"]["ix"], L["bounds"]["iy"], L["bounds"]["iz"] = find_max_const(L1["bounds"], L["bounds"])
        L["init_node_coors"] = copy.deepcopy(L["node_coords"])
        L["Tprime"] = np.zeros(L["nn"])
        L["Tprime0"] = np.zeros(L["nn"])
    # :176-182 shift Level 1 in z by layer heights until a node meets L2's top
    L1["orig_node_coords"] = copy.deepcopy(L1["node_coords"])
    tmp = copy.deepcopy(L1["orig_node_coords"])
    while not np.isclose(tmp[2] - L2["node_coords"][-1][-1], 0, atol=1e-4).any():
        tmp[2] = tmp[2] + P["layer_height"]
    L1["node_coords"] = copy.deepcopy(tmp)

    def get_overlap(fine, coarse):
        nodes = [getCoarseNodesInFineRegion(fine["node_coords"][i], coarse["node_coords"][i]) for i in range(3)]
        coors = [np.array([coarse["node_coords"][i][j] for j in nodes[i]]) for i in range(3)]
        return nodes, coors

    L2["orig_overlap_nodes"], L2["orig_overlap_coors"] = get_overlap(L2, L1)
    L3["orig_overlap_nodes"], L3["orig_overlap_coors"] = get_overlap(L3, L2)
    for L in (L2, L3):
        L["overlapNodes"] = copy.deepcopy(L["orig_overlap_nodes"])
        L["overlapCoords"] = copy.deepcopy(L["orig_overlap_coors"])

    L0 = {}
    L0["elements"] = [round(L1["length"][0] / L3["h"][0]), round(L1["length"][1] / L3["h"][1]),
                      round(L2["length"][2] / L3["h"][2])]
    L0["nodes"] = calcNumNodes(L0["elements"])
    L0["ne"] = L0["elements"][0] * L0["elements"][1] * L0["elements"][2]
    L0["nn"] = L0["nodes"][0] * L0["nodes"][1] * L0["nodes"][2]
    L0["node_coords"], L0["connect"] = createMesh3D(
        (L1["bounds"]["x"][0], L1["bounds"]["x"][1], L0["nodes"][0]),
        (L1["bounds"]["y"][0], L1["bounds"]["y"][1], L0["nodes"][1]),
        (L2["bounds"]["z"][0], L2["bounds"]["z"][1], L0["nodes"][2]))
    L0["orig_node_coords"] = copy.deepcopy(L0["node_coords"])
    L0["orig_overlap_nodes"], L0["orig_overlap_coors"] = get_overlap(L3, L0)
    L0["overlapNodes"] = copy.deepcopy(L0["orig_overlap_nodes"])
    L0["overlapCoords"] = copy.deepcopy(L0["orig_overlap_coors"])
    L0["orig_overlap_nodes_L2"] = [getCoarseNodesInLargeFineRegion(L2["node_coords"][i], L0["node_coords"][i])
                                   for i in range(3)]
    L0["orig_overlap_coors_L2"] = [np.array([L0["node_coords"][i][j] for j in L0["orig_overlap_nodes_L2"][i]])
                                   for i in range(3)]
    L0["overlapNodes_L2"] = copy.deepcopy(L0["orig_overlap_nodes_L2"])
    L0["overlapCoords_L2"] = copy.deepcopy(L0["orig_overlap_coors_L2"])
    L0["S1"] = np.zeros(L0["nn"])
    L0["S2"] = np.zeros(L0["nn"], dtype=bool)
    L0["idx"] = getOverlapRegion(L0["overlapNodes"], L0["nodes"][0], L0["nodes"][1])
    L0["idx_L2"] = getOverlapRegion(L0["overlapNodes_L2"], L0["nodes"][0], L0["nodes"][1])
    L0["layer_idx_delta"] = int(round(P["layer_height"] / L3["h"][2]))
    for L in (L0, L1, L2, L3):
        for a in ("elements", "h", "length", "nodes"):
            if a in L:
                L[a] = [np.array(v) for v in L[a]]
        for a in ("ne", "nn", "layer_idx_delta"):
            if a in L:
                L[a] = np.array(L[a])
    return [L0, L1, L2, L3]


def getStaticNodesAndElements(L):
    """:447-470."""
    return (_i(L[2]["ne"]), _i(L[3]["ne"]), _i(L[1]["nn"]), _i(L[2]["nn"]), _i(L[3]["nn"]))


def getStaticSubcycle(N):
    """:473-492."""
    N2, N3 = N["subcycle_num_L2"], N["subcycle_num_L3"]
    return (N2, N3, N2 * N3, float(N2), float(N3), float(N2 * N3))


def calcStaticTmpNodesAndElements(L, v):
    """:495-517: active Level-1 element/node counts below the laser height."""
    n = int((np.asarray(L[1]["node_coords"][2]) <= v[2] + 1e-5).sum())
    e = L[1]["elements"]
    nodes = L[1]["nodes"]
    return (_i(e[0]) * _i(e[1]) * (n - 1), _i(nodes[0]) * _i(nodes[1]) * n)


def getSubstrateNodes(Levels):
    """:562-579: number of nodes on planes with z < 1e-5 per level."""
    return tuple(int((np.asarray(L["node_coords"][2]) < 1e-5).sum()) * _i(L["nodes"][0]) * _i(L["nodes"][1])
                 for L in Levels[:4])


# ---------------------------------------------------------------------------
# FE basis (:692-855, :1361-1393, :3135-3166)
# ---------------------------------------------------------------------------
_KSI = np.array([-1, 1, 1, -1, -1, 1, 1, -1], dtype=float)
_ETA = np.array([-1, -1, 1, 1, -1, -1, 1, 1], dtype=float)
_ZETA = np.array([-1, -1, -1, -1, 1, 1, 1, 1], dtype=float)


def getSampleCoords(L):
    """:3135-3148: coordinates of the nodes of element 0."""
    c = L["node_coords"]
    k = L["connect"]
    return np.stack([np.asarray(c[i])[np.asarray(k[i])[0, :]] for i in range(3)], axis=1)


def hex8_basis(coords):
    """:692-775 computeQuad3dFemShapeFunctions_jax: N (8x8), dNdx (8x8x3), wq (8x1)."""
    kq, eq, zq = _KSI / SQ3, _ETA / SQ3, _ZETA / SQ3
    _k = 1 + kq[:, None] @ _KSI[None, :]
    _e = 1 + eq[:, None] @ _ETA[None, :]
    _z = 1 + zq[:, None] @ _ZETA[None, :]
    N = (1 / 8) * _k * _e * _z
    dk = (1 / 8) * _KSI[None, :] * _e * _z
    de = (1 / 8) * _ETA[None, :] * _k * _z
    dz = (1 / 8) * _ZETA[None, :] * _k * _e
    dxdk = (dk @ coords[:, 0])[0]
    dyde = (de @ coords[:, 1])[0]
    dzdz = (dz @ coords[:, 2])[0]
    J = np.array([[dxdk, 0.0, 0.0], [0.0, dyde, 0.0], [0.0, 0.0, dzdz]])
    Jinv = np.array([[1.0 / dxdk, 0.0, 0.0], [0.0, 1.0 / dyde, 0.0], [0.0, 0.0, 1.0 / dzdz]])
    dNdx = np.zeros((8, 8, 3))
    for q in range(8):
        dNdx[q] = np.stack([dk[q], de[q], dz[q]], axis=1) @ Jinv
    wq = np.full((8, 1), np.linalg.det(J))
    return N, dNdx, wq


def quad4_basis(coords):
    """:778-855 computeQuad2dFemShapeFunctions_jax (top face, coords[4:])."""
    ki = np.array([-1, 1, 1, -1], dtype=float)
    ei = np.array([-1, -1, 1, 1], dtype=float)
    kq, eq = ki / SQ3, ei / SQ3
    _k = 1 + kq[:, None] @ ki[None, :]
    _e = 1 + eq[:, None] @ ei[None, :]
    N = (1 / 4) * _k * _e
    dk = (1 / 4) * ki[None, :] * _e
    de = (1 / 4) * ei[None, :] * _k
    dxdk = (dk @ coords[4:, 0])[0]
    dyde = (de @ coords[4:, 1])[0]
    J = np.array([[dxdk, 0.0], [0.0, dyde]])
    wq = np.full((4, 1), np.linalg.det(J))
    return N, wq


def compute3DN(q, x, y, z, h):
    """:1361-1393: trilinear shape functions at points q (vectorised over points)."""
    inv_vol = 1.0 / (h[0] * h[1] * h[2])
    qx, qy, qz = q
    return np.stack([
        (x[1] - qx) * (y[1] - qy) * (z[1] - qz),
        (qx - x[0]) * (y[1] - qy) * (z[1] - qz),
        (qx - x[0]) * (qy - y[0]) * (z[1] - qz),
        (x[1] - qx) * (qy - y[0]) * (z[1] - qz),
        (x[1] - qx) * (y[1] - qy) * (qz - z[0]),
        (qx - x[0]) * (y[1] - qy) * (qz - z[0]),
        (qx - x[0]) * (qy - y[0]) * (qz - z[0]),
        (x[1] - qx) * (qy - y[0]) * (qz - z[0]),
    ], axis=-1) * inv_vol


def quad_coords(L, elems):
    """:3151-3166 getQuadratureCoords for many elements: (n, 8) x, y, z."""
    ex, ey, ez, nx, ny, nz = level_dims(L)
    N, _, _ = hex8_basis(getSampleCoords(L))
    _, ix, iy, iz = elem_nodes(ex, ey, nx, ny, elems)
    c = L["node_coords"]
    k = L["connect"]
    cx = np.asarray(c[0])[np.asarray(k[0])[ix, :]]
    cy = np.asarray(c[1])[np.asarray(k[1])[iy, :]]
    cz = np.asarray(c[2])[np.asarray(k[2])[iz, :]]
    return cx @ N.T, cy @ N.T, cz @ N.T


# ---------------------------------------------------------------------------
# a1: matrix-free level solve (:582-642)
# ---------------------------------------------------------------------------
def solveMatrixFreeFE(Level, nn, ne, k, rhocp, dt, T, Fc, Corr):
    """Explicit lumped-mass hex8 update over elements [0, ne).

    newT = sum_e (diag(Me) - Ke) T_e, newM = sum_e Me, return (newT+F+Corr)/newM
    with Me = colsum(N^T N) * wq * mean(rhocp_e)/dt and Ke = BTB * mean(k_e) * wq.
    """
    ex, ey, ez, nx, ny, nz = level_dims(Level)
    N, dNdx, wq = hex8_basis(getSampleCoords(Level))
    wq = wq[0][0]
    NTN = N.T @ N
    BTB = np.zeros((8, 8))
    for d in range(3):
        BTB += dNdx[:, :, d].T @ dNdx[:, :, d]
    idx, _, _, _ = elem_nodes(ex, ey, nx, ny, np.arange(_i(ne)))
    kvec = np.asarray(k)[idx].mean(axis=1)
    mvec = np.asarray(rhocp)[idx].mean(axis=1) / dt
    Me = (NTN * wq).sum(axis=0)[None, :] * mvec[:, None]
    Te = np.asarray(T)[idx]
    aT = Me * Te - (Te @ BTB.T) * (kvec * wq)[:, None]
    nn = _i(nn)
    newT = np.bincount(idx.reshape(-1), aT.reshape(-1), minlength=nn)[:nn]
    newM = np.bincount(idx.reshape(-1), Me.reshape(-1), minlength=nn)[:nn]
    with np.errstate(divide="ignore", invalid="ignore"):
        return (newT + Fc + Corr) / newM


# ---------------------------------------------------------------------------
# a2: phase state and properties (:2513-2614)
# ---------------------------------------------------------------------------
def computeStateProperties(T, S1, properties, nsub):
    """:2567-2614: S1 (bulk), S2 (fluid), k [W/mmK], rhocp [J/mm^3K]."""
    p = properties
    T = np.asarray(T, dtype=float)
    S2 = T >= p["T_liquidus"]
    S3 = (T > p["T_solidus"]) & (T < p["T_liquidus"])
    S1 = 1.0 * ((np.asarray(S1) > 0.499) | S2)
    S1[: _i(nsub)] = 1
    k = ((1 - S1) * (1 - S2) * p["k_powder"]
         + S1 * (1 - S2) * (p["k_bulk_coeff_a1"] * T + p["k_bulk_coeff_a0"])
         + S2 * p["k_fluid_coeff_a0"]) / 1000
    cp = ((1 - S2) * (1 - S3) * (p["cp_solid_coeff_a1"] * T + p["cp_solid_coeff_a0"])
          + S3 * p["cp_mushy"] + S2 * p["cp_fluid"])
    return S1, S2, k, p["rho"] * cp


def updateStateProperties(Levels, properties, substrate):
    """:2513-2564."""
    Levels[3]["S1"], Levels[3]["S2"], L3k, L3rc = computeStateProperties(
        Levels[3]["T0"], Levels[3]["S1"], properties, substrate[3])
    Levels[2]["S1"], _, L2k, L2rc = computeStateProperties(
        Levels[2]["T0"], Levels[2]["S1"], properties, substrate[2])
    val = interpolatePoints(Levels[2], Levels[2]["S1"], Levels[2]["overlapCoords"])
    idx = getOverlapRegion(Levels[2]["overlapNodes"], Levels[1]["nodes"][0], Levels[1]["nodes"][1])
    S1 = np.array(Levels[1]["S1"], dtype=float)
    S1[idx] = val
    S1[: substrate[1]] = 1
    Levels[1]["S1"] = S1
    _, _, L1k, L1rc = computeStateProperties(Levels[1]["T0"], Levels[1]["S1"], properties, substrate[1])
    return Levels, [0, L1k, L2k, L3k], [0, L1rc, L2rc, L3rc]


# ---------------------------------------------------------------------------
# a3/a4: Gaussian source (:928-1025, :2667-2730, :2960-3012)
# ---------------------------------------------------------------------------
def computeSourceFunction(x, y, z, v, properties, P):
    """:991-1025: separable Gaussian volumetric source [W/mm^3]."""
    p = properties
    pc = 6 * np.sqrt(3) * P * p["laser_eta"]
    rc = 1 / (p["laser_radius"] * np.sqrt(np.pi))
    dc = 1 / (p["laser_depth"] * np.sqrt(np.pi))
    rsq = p["laser_radius"] ** 2
    dsq = p["laser_depth"] ** 2
    Qx = rc * np.exp(-3 * (x - v[0]) ** 2 / rsq)
    Qy = rc * np.exp(-3 * (y - v[1]) ** 2 / rsq)
    Qz = dc * np.exp(-3 * (z - v[2]) ** 2 / dsq)
    return pc * Qx * Qy * Qz


def _fine_source(L3, v, properties, P):
    """Q*w at the 8 Gauss points of every fine element: (nef, 8)."""
    ex, ey, ez, nx, ny, nz = level_dims(L3)
    _, _, wq = hex8_basis(getSampleCoords(L3))
    x, y, z = quad_coords(L3, np.arange(ex * ey * ez))
    return computeSourceFunction(x, y, z, v, properties, P) * wq[0, 0]


def computeSourcesL3(Level, v, ne_nn, properties, laserP):
    """:2960-3012: F_a = sum_q N[a,q] Q_q w, assembled over fine elements."""
    ex, ey, ez, nx, ny, nz = level_dims(Level)
    N, _, wq = hex8_basis(getSampleCoords(Level))
    idx, _, _, _ = elem_nodes(ex, ey, nx, ny, np.arange(ne_nn[1]))
    x, y, z = quad_coords(Level, np.arange(ne_nn[1]))
    Q = computeSourceFunction(x, y, z, v, properties, laserP)
    data = (Q @ N.T) * wq[:, 0][None, :]
    return np.bincount(idx.reshape(-1), data.reshape(-1), minlength=ne_nn[4])[: ne_nn[4]]


def shape_apply(shape, data, nnc):
    """BCOO projection of Shapes[i][2]: scatter (nef, 8) into coarse nodes."""
    nodes = shape[2]
    return np.bincount(nodes.reshape(-1), data.reshape(-1), minlength=nnc)[:nnc]


def computeLevelSource(Levels, ne_nn, laser_position, LevelShape, properties, laserP, nnc):
    """:2667-2730: coarse source = BCOO( mean_p sum_q Nc[e,q,a] Q_p w ).

    ``nnc`` is the coarse node count (the BCOO's row count).
    """
    L3 = Levels[3]
    acc = 0.0
    lp = np.asarray(laser_position)
    for p in range(lp.shape[0]):
        acc = acc + _fine_source(L3, lp[p], properties, np.asarray(laserP)[p])
    data = np.einsum("eqa,eq->ea", LevelShape[0], acc) / lp.shape[0]
    return shape_apply(LevelShape, data, nnc)


def computeSources(Level, v, Shapes, ne_nn, properties, laserP, nn1, nn2):
    """:928-988: L3-quadrature source assembled on L1, L2 and L3."""
    Qw = _fine_source(Level, v, properties, laserP)
    Fc = shape_apply(Shapes[1], np.einsum("eqa,eq->ea", Shapes[1][0], Qw), nn1)
    Fm = shape_apply(Shapes[2], np.einsum("eqa,eq->ea", Shapes[2][0], Qw), nn2)
    Ff = computeSourcesL3(Level, v, ne_nn, properties, laserP)
    return Fc, Fm, Ff


# ---------------------------------------------------------------------------
# a5: top-surface convection / radiation / evaporation (:2207-2301)
# ---------------------------------------------------------------------------
def computeConvRadBC(Level, LevelT0, ne, nn, properties, F):
    p = properties
    ex, ey, ez, nx, ny, nz = level_dims(Level)
    c = Level["node_coords"]
    k = Level["connect"]
    coords = np.stack([np.asarray(c[0])[np.asarray(k[0])[0, :]], np.asarray(c[1])[np.asarray(k[1])[0, :]]], axis=1)
    N, wq = quad4_basis(coords)
    top = ex * ey
    elems = np.arange(_i(ne) - top, _i(ne))
    idx, _, _, _ = elem_nodes(ex, ey, nx, ny, elems)
    idx4 = idx[:, 4:]
    Tq = np.asarray(LevelT0)[idx4] @ N.T
    Tq = np.minimum(Tq, p["T_boiling"] + 1000)
    invT = 1.0 / Tq
    E_pv = p["Lev"] + p["cp_fluid"] * (Tq - p["T_amb"])
    MolMot = np.sqrt(p["CM_coeff"] * invT)
    S = p["evc"] * p["CP_coeff"] * np.exp(-p["CT_coeff"] * (invT - 1.0 / p["T_boiling"])) * MolMot * E_pv
    q = p["h_conv"] * (p["T_amb"] - Tq) + p["sigma_sb"] * p["vareps"] * (p["T_amb"] ** 4 - Tq ** 4) - S
    q = q * 1e-6
    data = (q * wq[:, 0][None, :]) @ N
    nn = _i(nn)
    return F + np.bincount(idx4.reshape(-1), data.reshape(-1), minlength=nn)[:nn]


# ---------------------------------------------------------------------------
# a6: Dirichlet conditions (:1568-1620, :1848-1883)
# ---------------------------------------------------------------------------
def assignBCs(RHS, Levels):
    R = np.array(RHS, dtype=float)
    BC = Levels[1]["BC"]
    cond = Levels[1]["conditions"]
    R[BC[2]] = _f(cond["y"][0])
    R[BC[3]] = _f(cond["y"][1])
    R[BC[0]] = _f(cond["x"][0])
    R[BC[1]] = _f(cond["x"][1])
    R[BC[4]] = _f(cond["z"][0])
    return R


def assignBCsFine(RHS, TfAll, BC):
    R = np.array(RHS, dtype=float)
    for j in (2, 3, 0, 1, 4):
        R[BC[j]] = TfAll[BC[j]]
    return R


def substitute_Tbar(Tbar, idx, val):
    R = np.array(Tbar, dtype=float)
    R[_i(idx):] = val
    return R


# ---------------------------------------------------------------------------
# a8/a9: prolongation (:1028-1210)
# ---------------------------------------------------------------------------
def _interp_weights(Level, node_coords_new):
    ex, ey, ez, nx, ny, nz = level_dims(Level)
    c = [np.asarray(a, dtype=float) for a in Level["node_coords"]]
    kk = [np.asarray(a) for a in Level["connect"]]
    xn, yn, zn = (np.asarray(a, dtype=float) for a in node_coords_new)
    tot = len(xn) * len(yn) * len(zn)
    i = np.arange(tot)
    izn, rem = np.divmod(i, len(xn) * len(yn))
    iyn, ixn = np.divmod(rem, len(xn))
    _x, _y, _z = xn[ixn], yn[iyn], zn[izn]
    h = [c[d][1] - c[d][0] for d in range(3)]
    ie = [np.clip(np.floor((q - c[d][0]) / h[d]).astype(int), 0, (ex, ey, ez)[d] - 1)
          for d, q in enumerate((_x, _y, _z))]
    nodex, nodey, nodez = kk[0][ie[0], :], kk[1][ie[1], :], kk[2][ie[2], :]
    node = nodex + nodey * nx + nodez * (nx * ny)
    xx, yy, zz = c[0][nodex], c[1][nodey], c[2][nodez]
    Nc = compute3DN([_x, _y, _z], [xx[:, 0], xx[:, 1]], [yy[:, 0], yy[:, 3]], [zz[:, 0], zz[:, 5]], h)
    valid = ((Nc >= -1e-2).all(axis=1)) & ((Nc <= 1 + 1e-2).all(axis=1))
    Nc = np.where(valid[:, None], np.clip(Nc, 0.0, 1.0), 0.0)
    return Nc, node


def interpolatePointsMatrix(Level, node_coords_new):
    """:1028-1107: [Nc (npts, 8), node (npts, 8)]."""
    Nc, node = _interp_weights(Level, node_coords_new)
    return [Nc, node]


def interpolate_w_matrix(C2F, T):
    """:1110-1128."""
    return (C2F[0] * np.asarray(T)[C2F[1]]).sum(axis=1)


def interpolatePoints(Level, u, node_coords_new):
    """:1131-1210."""
    Nc, node = _interp_weights(Level, node_coords_new)
    return (Nc * np.asarray(u)[node]).sum(axis=1)


# ---------------------------------------------------------------------------
# a11: coarse shape functions at fine quadrature points (:1213-1358)
# ---------------------------------------------------------------------------
def computeCoarseFineShapeFunctions(Coarse, Fine):
    """Returns [Nc, [dNcdx, dNcdy, dNcdz], nodes] with arrays (nef, 8q, 8a) and
    ``nodes`` (nef, 8): coarse node ids of quadrature point 0 (the BCOO rows)."""
    exc, eyc, ezc, nxc, nyc, nzc = level_dims(Coarse)
    c = [np.asarray(a, dtype=float) for a in Coarse["node_coords"]]
    kc = [np.asarray(a) for a in Coarse["connect"]]
    h = [c[d][1] - c[d][0] for d in range(3)]
    hxyz = h[0] * h[1] * h[2]
    exf, eyf, ezf, _, _, _ = level_dims(Fine)
    x, y, z = quad_coords(Fine, np.arange(exf * eyf * ezf))
    ie = [np.clip(np.floor((q - c[d][0]) / h[d]).astype(int), 0, (exc, eyc, ezc)[d] - 1)
          for d, q in enumerate((x, y, z))]
    ncx, ncy, ncz = kc[0][ie[0]], kc[1][ie[1]], kc[2][ie[2]]  # (nef, 8q, 8a)
    nodes = ncx + ncy * nxc + ncz * nxc * nyc
    xc0, xc1 = c[0][ncx[..., 0]], c[0][ncx[..., 1]]
    yc0, yc3 = c[1][ncy[..., 0]], c[1][ncy[..., 3]]
    zc0, zc5 = c[2][ncz[..., 0]], c[2][ncz[..., 5]]
    Nc = compute3DN([x, y, z], [xc0, xc1], [yc0, yc3], [zc0, zc5], h)
    X, Y, Z = x[..., None], y[..., None], z[..., None]
    a = [xc0[..., None], xc1[..., None], yc0[..., None], yc3[..., None], zc0[..., None], zc5[..., None]]
    x0, x1, y0, y1, z0, z1 = a
    sx = np.array([-1, 1, 1, -1, -1, 1, 1, -1], dtype=float)
    wy = np.where(np.array([0, 0, 1, 1, 0, 0, 1, 1]) == 1, Y - y0, y1 - Y)
    wz = np.where(np.array([0, 0, 0, 0, 1, 1, 1, 1]) == 1, Z - z0, z1 - Z)
    wx = np.where(np.array([0, 1, 1, 0, 0, 1, 1, 0]) == 1, X - x0, x1 - X)
    sy = np.array([-1, -1, 1, 1, -1, -1, 1, 1], dtype=float)
    sz = np.array([-1, -1, -1, -1, 1, 1, 1, 1], dtype=float)
    dNdx = sx * wy * wz / hxyz
    dNdy = wx * sy * wz / hxyz
    dNdz = wx * wy * sz / hxyz
    return [Nc, [dNdx, dNdy, dNdz], nodes[:, 0, :]]


# ---------------------------------------------------------------------------
# a12/a13: subgrid coupling terms (:1396-1565, :2733-2810, :2857-2914,
#          :3057-3132, :3169-3221)
# ---------------------------------------------------------------------------
def _fine_flux(L, Tp, k):
    """k_mean_e * dT'/dx_d at the 8 Gauss points: list of 3 (nef, 8q), and wq."""
    ex, ey, ez, nx, ny, nz = level_dims(L)
    N, dNdx, wq = hex8_basis(getSampleCoords(L))
    idx, _, _, _ = elem_nodes(ex, ey, nx, ny, np.arange(ex * ey * ez))
    Te = np.asarray(Tp)[idx]
    kmean = (np.asarray(k)[idx] @ N.T).mean(axis=1)
    return [(Te @ dNdx[:, :, d].T) * kmean[:, None] for d in range(3)], wq[0, 0]


def _fine_mass(L, dTp, rhocp, dt):
    ex, ey, ez, nx, ny, nz = level_dims(L)
    N, _, wq = hex8_basis(getSampleCoords(L))
    idx, _, _, _ = elem_nodes(ex, ey, nx, ny, np.arange(ex * ey * ez))
    rmean = (np.asarray(rhocp)[idx] @ N.T).mean(axis=1)
    return (np.asarray(dTp)[idx] @ N.T) * rmean[:, None], wq[0, 0] / dt


def _flux_project(shape, flux, wq, nnc):
    data = -sum(np.einsum("eqa,eq->ea", shape[1][d], flux[d]) for d in range(3)) * wq
    return shape_apply(shape, data, nnc)


def _mass_project(shape, mass, w, nnc):
    data = -np.einsum("eqa,eq->ea", shape[0], mass) * w
    return shape_apply(shape, data, nnc)


def computeL1TprimeTerms_Part1(Levels, ne_nn, L3k, Shapes, L2k):
    """:2733-2810."""
    nn1 = _i(Levels[1]["nn"])
    f3, w3 = _fine_flux(Levels[3], Levels[3]["Tprime0"], L3k)
    f2, w2 = _fine_flux(Levels[2], Levels[2]["Tprime0"], L2k)
    return _flux_project(Shapes[1], f3, w3, nn1) + _flux_project(Shapes[0], f2, w2, nn1)


def computeL2TprimeTerms_Part1(Levels, ne_nn, L3Tprime0, L3k, Shapes):
    """:2857-2914."""
    f3, w3 = _fine_flux(Levels[3], L3Tprime0, L3k)
    return _flux_project(Shapes[2], f3, w3, _i(Levels[2]["nn"]))


def computeL1TprimeTerms_Part2(Levels, ne_nn, L3Tp, L2Tp, L3rhocp, L2rhocp, dt, Shapes, Vcu):
    """:3057-3132."""
    nn1 = _i(Levels[1]["nn"])
    m3, w3 = _fine_mass(Levels[3], np.asarray(L3Tp) - np.asarray(Levels[3]["Tprime0"]), L3rhocp, dt)
    m2, w2 = _fine_mass(Levels[2], np.asarray(L2Tp) - np.asarray(Levels[2]["Tprime0"]), L2rhocp, dt)
    return Vcu + _mass_project(Shapes[1], m3, w3, nn1) + _mass_project(Shapes[0], m2, w2, nn1)


def computeL2TprimeTerms_Part2(Levels, ne_nn, L3Tp, L3Tp0, L3rhocp, dt, Shapes, L2V):
    """:3169-3221."""
    m3, w3 = _fine_mass(Levels[3], np.asarray(L3Tp) - np.asarray(L3Tp0), L3rhocp, dt)
    return L2V + _mass_project(Shapes[2], m3, w3, _i(Levels[2]["nn"]))


def computeCoarseTprimeTerm_jax(Levels, L3k, L2k, Shapes):
    """:1477-1565 (single-step predictor terms)."""
    nn1, nn2 = _i(Levels[1]["nn"]), _i(Levels[2]["nn"])
    f3, w3 = _fine_flux(Levels[3], Levels[3]["Tprime0"], L3k)
    f2, w2 = _fine_flux(Levels[2], Levels[2]["Tprime0"], L2k)
    Vcu = _flux_project(Shapes[1], f3, w3, nn1) + _flux_project(Shapes[0], f2, w2, nn1)
    Vmu = _flux_project(Shapes[2], f3, w3, nn2)
    return Vcu, Vmu


def computeCoarseTprimeMassTerm_jax(Levels, Tprimef, Tprimem, L3rhocp, L2rhocp, dt, Shapes, Vcu, Vmu):
    """:1396-1474 (single-step corrector terms)."""
    nn1, nn2 = _i(Levels[1]["nn"]), _i(Levels[2]["nn"])
    m3, w3 = _fine_mass(Levels[3], np.asarray(Tprimef) - np.asarray(Levels[3]["Tprime0"]), L3rhocp, dt)
    m2, w2 = _fine_mass(Levels[2], np.asarray(Tprimem) - np.asarray(Levels[2]["Tprime0"]), L2rhocp, dt)
    Vcu = Vcu + _mass_project(Shapes[1], m3, w3, nn1) + _mass_project(Shapes[0], m2, w2, nn1)
    Vmu = Vmu + _mass_project(Shapes[2], m3, w3, nn2)
    return Vcu, Vmu


# ---------------------------------------------------------------------------
# a10: restriction + T' (:2060-2132)
# ---------------------------------------------------------------------------
def getNewTprime(Fine, FineT0, CoarseT, Coarse, C2F):
    val = interpolatePoints(Fine, FineT0, Fine["overlapCoords"])
    idx = getOverlapRegion(Fine["overlapNodes"], Coarse["nodes"][0], Coarse["nodes"][1])
    CoarseT = np.array(CoarseT, dtype=float)
    CoarseT[idx] = val
    return np.asarray(FineT0) - interpolate_w_matrix(C2F, CoarseT), CoarseT


def getBothNewTprimes(Levels, FineT, MesoT, M2F, CoarseT, C2M):
    lTp, mT0 = getNewTprime(Levels[3], FineT, MesoT, Levels[2], M2F)
    mTp, uT0 = getNewTprime(Levels[2], mT0, CoarseT, Levels[1], C2M)
    return lTp, mTp, mT0, uT0


# ---------------------------------------------------------------------------
# a7: level-solve call surface (:2135-2204, :2813-2854, :2917-2957, :3015-3054)
# ---------------------------------------------------------------------------
def computeL1Temperature(Levels, ne_nn, tmp_ne_nn, L1F, L1V, L1k, L1rhocp, dt, properties):
    T = solveMatrixFreeFE(Levels[1], ne_nn[2], tmp_ne_nn[0], L1k, L1rhocp, dt, Levels[1]["T0"], L1F, L1V)
    T = substitute_Tbar(T, tmp_ne_nn[1], properties["T_amb"])
    return assignBCs(T, Levels)


def computeL2Temperature(L1T, L1L2Interp, Levels, ne_nn, L2T0, L2F, L2V, L2k, L2rhocp, dt):
    TfAll = interpolate_w_matrix(L1L2Interp, L1T)
    T = solveMatrixFreeFE(Levels[2], ne_nn[3], ne_nn[0], L2k, L2rhocp, dt, L2T0, L2F, L2V)
    return assignBCsFine(T, TfAll, Levels[2]["BC"])


def computeSolutions_L3(FinalL2, L2L3Interp, Levels, ne_nn, L3T0, L3F, L3k, L3rhocp, dt):
    TfAll = interpolate_w_matrix(L2L3Interp, FinalL2)
    T = solveMatrixFreeFE(Levels[3], ne_nn[4], ne_nn[1], L3k, L3rhocp, dt, L3T0, L3F, 0)
    return assignBCsFine(T, TfAll, Levels[3]["BC"])


def computeSolutions(Levels, ne_nn, tmp_ne_nn, LF, L1V, LInterp, Lk, Lrhocp, L2V, dt, properties):
    L1T = solveMatrixFreeFE(Levels[1], ne_nn[2], tmp_ne_nn[0], Lk[1], Lrhocp[1], dt, Levels[1]["T0"], LF[1], L1V)
    L1T = substitute_Tbar(L1T, tmp_ne_nn[1], properties["T_amb"])
    F1 = assignBCs(L1T, Levels)
    TfAll = interpolate_w_matrix(LInterp[0], F1)
    L2T = solveMatrixFreeFE(Levels[2], ne_nn[3], ne_nn[0], Lk[2], Lrhocp[2], dt, Levels[2]["T0"], LF[2], L2V)
    F2 = assignBCsFine(L2T, TfAll, Levels[2]["BC"])
    TfAll = interpolate_w_matrix(LInterp[1], F2)
    L3T = solveMatrixFreeFE(Levels[3], ne_nn[4], ne_nn[1], Lk[3], Lrhocp[3], dt, Levels[3]["T0"], LF[3], 0)
    F3 = assignBCsFine(L3T, TfAll, Levels[3]["BC"])
    return F1, F2, F3


# ---------------------------------------------------------------------------
# a14: moving-window remap (:1672-1845, :2400-2510)
# ---------------------------------------------------------------------------
def _trunc(x):
    return int(np.asarray(x).astype(int))


def jit_constrain_v(vtot, Level):
    b = Level["bounds"]
    return [np.clip(vtot[0], b["ix"][0], b["ix"][1]), np.clip(vtot[1], b["iy"][0], b["iy"][1]),
            np.clip(vtot[2], b["iz"][0], b["iz"][1])]


def move_fine_mesh(node_coords, element_size, v):
    s = [_trunc(v[d] / element_size[d] + 1e-2) for d in range(3)]
    return [np.asarray(node_coords[d]) + element_size[d] * s[d] for d in range(3)], s


def update_overlap_nodes_coords(Level, vcon, element_size, ele_ratio):
    s = [_trunc(vcon[d] / element_size[d] + 1e-2) for d in range(3)]
    Level["overlapNodes"] = [np.asarray(Level["orig_overlap_nodes"][d]) + ele_ratio[d] * s[d] for d in range(3)]
    Level["overlapCoords"] = [np.asarray(Level["orig_overlap_coors"][d]) + element_size[d] * s[d] for d in range(3)]
    return Level


def update_overlap_nodes_coords_L1L2(Level, vcon, element_size, powder_layer):
    sx, sy, sz = (_trunc(vcon[d] / element_size[d] + 1e-2) for d in range(3))
    szp = powder_layer * _trunc(vcon[2] / powder_layer + 1e-2)
    o = Level["orig_overlap_nodes"]
    c = Level["orig_overlap_coors"]
    Level["overlapNodes"] = [np.asarray(o[0]) + sx, np.asarray(o[1]) + sy, np.asarray(o[2]) + sz]
    Level["overlapCoords"] = [np.asarray(c[0]) + element_size[0] * sx, np.asarray(c[1]) + element_size[1] * sy,
                              np.asarray(c[2]) + szp]
    return Level


def update_overlap_nodes_coords_L2(Level, vcon, element_size, ele_ratio):
    s = [_trunc(vcon[d] / element_size[d] + 1e-2) for d in range(3)]
    Level["overlapNodes_L2"] = [np.asarray(Level["orig_overlap_nodes_L2"][d]) + ele_ratio[d] * s[d]
                                for d in range(3)]
    Level["overlapCoords_L2"] = [np.asarray(Level["orig_overlap_coors_L2"][d]) + element_size[d] * s[d]
                                 for d in range(3)]
    return Level


def moveEverything(v, vstart, Levels, move_v, LInterp, L1L2Eratio, L2L3Eratio, height):
    """:2400-2510. Returns (Levels, Shapes, LInterp, move_v)."""
    v = np.asarray(v, dtype=float)
    vtot = v - np.asarray(vstart, dtype=float)
    h2 = [_f(x) for x in Levels[2]["h"]]
    h1 = [_f(x) for x in Levels[1]["h"]]
    v3 = jit_constrain_v(vtot, Levels[3])
    new3, _ = move_fine_mesh(Levels[3]["init_node_coors"], h2, v3)
    Levels[3] = update_overlap_nodes_coords(Levels[3], v3, h2, [1, 1, 1])
    T3 = interpolatePoints(Levels[1], Levels[1]["T0"], new3)
    Tp2 = interpolatePoints(Levels[2], Levels[2]["Tprime0"], new3)
    Tp3 = interpolatePoints(Levels[3], Levels[3]["Tprime0"], new3)
    Levels[3]["T0"] = T3 + (Tp2 + Tp3)
    Levels[3]["Tprime0"] = Tp3
    Levels[3]["node_coords"] = new3

    v2 = jit_constrain_v(vtot, Levels[2])
    new2, mv = move_fine_mesh(Levels[2]["init_node_coors"], [h1[0], h1[1], float(height)], v2)
    move_v = [mv[i] * L1L2Eratio[i] for i in range(3)]
    Levels[2] = update_overlap_nodes_coords_L1L2(Levels[2], v2, h1, height)
    T2 = interpolatePoints(Levels[1], Levels[1]["T0"], new2)
    Levels[2]["Tprime0"] = interpolatePoints(Levels[2], Levels[2]["Tprime0"], new2)
    Levels[2]["T0"] = T2 + Levels[2]["Tprime0"]
    Levels[2]["node_coords"] = new2
    L2L1Shape = computeCoarseFineShapeFunctions(Levels[1], Levels[2])
    LInterp = list(LInterp)
    LInterp[0] = interpolatePointsMatrix(Levels[1], new2)

    Levels[3]["overlapNodes"] = [np.asarray(Levels[3]["overlapNodes"][i]) - move_v[i] for i in range(3)]
    Levels[0] = update_overlap_nodes_coords(Levels[0], v3, h2, L2L3Eratio)
    Levels[0] = update_overlap_nodes_coords_L2(
        Levels[0], v2, [h1[0], h1[1], h2[2]],
        [L1L2Eratio[0] * L2L3Eratio[0], L1L2Eratio[1] * L2L3Eratio[1], L2L3Eratio[2]])
    Levels[0]["overlapNodes"][2] = Levels[0]["overlapNodes"][2] - move_v[2] * L2L3Eratio[2]
    Levels[0]["overlapNodes_L2"][2] = Levels[0]["overlapNodes_L2"][2] - move_v[2] * L2L3Eratio[2]
    Levels[0]["idx"] = getOverlapRegion(Levels[0]["overlapNodes"], Levels[0]["nodes"][0], Levels[0]["nodes"][1])
    Levels[0]["idx_L2"] = getOverlapRegion(Levels[0]["overlapNodes_L2"], Levels[0]["nodes"][0],
                                           Levels[0]["nodes"][1])
    Levels[2]["S1"] = np.asarray(Levels[0]["S1"])[Levels[0]["idx_L2"]].astype(float)
    Levels[3]["S1"] = np.asarray(Levels[0]["S1"])[Levels[0]["idx"]].astype(float)
    Levels[3]["S2"] = np.asarray(Levels[0]["S2"])[Levels[0]["idx"]].astype(bool)
    L3L1Shape = computeCoarseFineShapeFunctions(Levels[1], Levels[3])
    L3L2Shape = computeCoarseFineShapeFunctions(Levels[2], Levels[3])
    LInterp[1] = interpolatePointsMatrix(Levels[2], new3)
    return Levels, [L2L1Shape, L3L1Shape, L3L2Shape], LInterp, move_v


# ---------------------------------------------------------------------------
# a15: subcycled predictor-corrector step (:3224-3632)
# ---------------------------------------------------------------------------
def _clampT(p, T):
    return np.maximum(p["T_amb"], T)


def subcycleGOMELT(Levels, ne_nn, Shapes, substrate, LInterp, tmp_ne_nn, laser_position, properties, laserP,
                   subcycle, max_accum_L3, accum_L3):
    p = properties
    lp = np.asarray(laser_position, dtype=float)
    lP = np.asarray(laserP, dtype=float)
    N2, N3 = subcycle[0], subcycle[1]
    nn1, nn2 = _i(Levels[1]["nn"]), _i(Levels[2]["nn"])
    _, _, L3k_L1, L3rc_L1 = computeStateProperties(Levels[3]["T0"], Levels[3]["S1"], p, substrate[3])
    _, _, L2k_L1, L2rc_L1 = computeStateProperties(Levels[2]["T0"], Levels[2]["S1"], p, substrate[2])
    val = interpolatePoints(Levels[2], Levels[2]["S1"], Levels[2]["overlapCoords"])
    idx = getOverlapRegion(Levels[2]["overlapNodes"], Levels[1]["nodes"][0], Levels[1]["nodes"][1])
    S1 = np.array(Levels[1]["S1"], dtype=float)
    S1[idx] = val
    S1[: substrate[1]] = 1
    Levels[1]["S1"] = S1
    _, _, L1k, L1rc = computeStateProperties(Levels[1]["T0"], Levels[1]["S1"], p, substrate[1])

    dt1 = lp[:, 5].sum()
    L1F = computeLevelSource(Levels, ne_nn, lp, Shapes[1], p, lP, nn1)
    L1F = computeConvRadBC(Levels[1], Levels[1]["T0"], tmp_ne_nn[0], ne_nn[2], p, L1F)
    L1V = computeL1TprimeTerms_Part1(Levels, ne_nn, L3k_L1, Shapes, L2k_L1)
    L1T = computeL1Temperature(Levels, ne_nn, tmp_ne_nn, L1F, L1V, L1k, L1rc, dt1, p)
    L1T = _clampT(p, L1T)

    def l2_step(carry, l2sub, part2, L3Tp_hist):
        L2T0c, L2S1c, L3Tc, L3Tpc, L3S1c = carry[:5]
        aL2 = (l2sub + 1) / subcycle[3]
        bL2 = 1 - aL2
        Lidx = l2sub * N3 + np.arange(N3)
        _, _, L3k_L2, L3rc_L2 = computeStateProperties(L3Tc, L3S1c, p, substrate[3])
        L2S1, _, L2k, L2rc = computeStateProperties(L2T0c, L2S1c, p, substrate[2])
        L2F = computeLevelSource(Levels, ne_nn, lp[Lidx], Shapes[2], p, lP[Lidx], nn2)
        L2F = computeConvRadBC(Levels[2], L2T0c, ne_nn[0], ne_nn[3], p, L2F)
        L2V = computeL2TprimeTerms_Part1(Levels, ne_nn, L3Tpc, L3k_L2, Shapes)
        dt2 = lp[Lidx, 5].sum()
        if part2:
            L2V = computeL2TprimeTerms_Part2(Levels, ne_nn, L3Tp_hist[l2sub], L3Tpc, L3rc_L2, dt2, Shapes, L2V)
        BC = aL2 * L1T + bL2 * np.asarray(Levels[1]["T0"])
        L2T = computeL2Temperature(BC, LInterp[0], Levels, ne_nn, L2T0c, L2F, L2V, L2k, L2rc, dt2)
        L2T = _clampT(p, L2T)
        L3T, L3S1 = L3Tc, L3S1c
        if part2:
            L3S2, max_acc, acc = carry[5], carry[6], carry[7]
        for l3sub in range(N3):
            S1n, S2n, L3k, L3rc = computeStateProperties(L3T, L3S1, p, substrate[3])
            li = l3sub + l2sub * N3
            L3F = computeSourcesL3(Levels[3], lp[li], ne_nn, p, lP[li])
            L3F = computeConvRadBC(Levels[3], L3T, ne_nn[1], ne_nn[4], p, L3F)
            aL3 = (l3sub + 1) / subcycle[4]
            BC3 = aL3 * L2T + (1 - aL3) * L2T0c
            L3Tn = computeSolutions_L3(BC3, LInterp[1], Levels, ne_nn, L3T, L3F, L3k, L3rc, lp[li, 5])
            L3Tn = _clampT(p, L3Tn)
            if part2:
                reset = ((1 - 2 * np.asarray(L3S2, dtype=float)) * S2n) == 1
                racc = acc * reset
                max_acc = np.maximum(racc, max_acc)
                acc = acc + lp[li, 5] * S2n - racc
                L3S2 = S2n
            L3T, L3S1 = L3Tn, S1n
        L3Tp, L2T = getNewTprime(Levels[3], L3T, L2T, Levels[2], LInterp[1])
        if part2:
            return [L2T, L2S1, L3T, L3Tp, L3S1, L3S2, max_acc, acc]
        return [L2T, L2S1, L3T, L3Tp, L3S1]

    carry = [np.asarray(Levels[2]["T0"]), np.asarray(Levels[2]["S1"]), np.asarray(Levels[3]["T0"]),
             np.asarray(Levels[3]["Tprime0"]), np.asarray(Levels[3]["S1"])]
    hist = []
    for l2sub in range(N2):
        carry = l2_step(carry, l2sub, False, None)
        hist.append(carry[3])
    L2T, L3Tp = carry[0], carry[3]

    L2Tp, L1T = getNewTprime(Levels[2], L2T, L1T, Levels[1], LInterp[0])
    L1V = computeL1TprimeTerms_Part2(Levels, ne_nn, L3Tp, L2Tp, L3rc_L1, L2rc_L1, dt1, Shapes, L1V)
    L1T = computeL1Temperature(Levels, ne_nn, tmp_ne_nn, L1F, L1V, L1k, L1rc, dt1, p)
    L1T = _clampT(p, L1T)

    carry = [np.asarray(Levels[2]["T0"]), np.asarray(Levels[2]["S1"]), np.asarray(Levels[3]["T0"]),
             np.asarray(Levels[3]["Tprime0"]), np.asarray(Levels[3]["S1"]), np.asarray(Levels[3]["S2"]),
             np.asarray(max_accum_L3, dtype=float), np.asarray(accum_L3, dtype=float)]
    L2all, L3all, L3pall = [], [], []
    for l2sub in range(N2):
        carry = l2_step(carry, l2sub, True, hist)
        L2all.append(carry[0])
        L3all.append(carry[2])
        L3pall.append(carry[3])
    (Levels[2]["T0"], Levels[2]["S1"], Levels[3]["T0"], Levels[3]["Tprime0"], Levels[3]["S1"], Levels[3]["S2"],
     max_accum_L3, accum_L3) = carry
    Levels[2]["Tprime0"], Levels[1]["T0"] = getNewTprime(Levels[2], Levels[2]["T0"], L1T, Levels[1], LInterp[0])
    S1_0 = np.array(Levels[0]["S1"], dtype=float)
    S1_0[Levels[0]["idx"]] = Levels[3]["S1"]
    Levels[0]["S1"] = S1_0
    S2_0 = np.zeros_like(np.asarray(Levels[0]["S2"]), dtype=bool)
    S2_0[Levels[0]["idx"]] = Levels[3]["S2"]
    Levels[0]["S2"] = S2_0
    return Levels, np.array(L2all), np.array(L3all), np.array(L3pall), max_accum_L3, accum_L3


# ---------------------------------------------------------------------------
# a16/a17: single step and dwell step (:2304-2397, :2617-2664)
# ---------------------------------------------------------------------------
def stepGOMELT(Levels, ne_nn, tmp_ne_nn, Shapes, LInterp, v, properties, dt, laserP, substrate):
    p = properties
    preS2 = np.asarray(Levels[3]["S2"])
    Levels, Lk, Lrc = updateStateProperties(Levels, p, substrate)
    L1, L2, L3 = Levels[1], Levels[2], Levels[3]
    nn1, nn2 = _i(L1["nn"]), _i(L2["nn"])
    Fc, Fm, Ff = computeSources(L3, v, Shapes, ne_nn, p, laserP, nn1, nn2)
    Fc = computeConvRadBC(L1, L1["T0"], tmp_ne_nn[0], ne_nn[2], p, Fc)
    Fm = computeConvRadBC(L2, L2["T0"], ne_nn[0], ne_nn[3], p, Fm)
    Ff = computeConvRadBC(L3, L3["T0"], ne_nn[1], ne_nn[4], p, Ff)
    F = [0, Fc, Fm, Ff]
    Vcu, Vmu = computeCoarseTprimeTerm_jax(Levels, Lk[3], Lk[2], Shapes)
    L1T, L2T, L3T = computeSolutions(Levels, ne_nn, tmp_ne_nn, F, Vcu, LInterp, Lk, Lrc, Vmu, dt, p)
    L1T, L2T, L3T = _clampT(p, L1T), _clampT(p, L2T), _clampT(p, L3T)
    L3Tp, L2Tp, L2T, L1T = getBothNewTprimes(Levels, L3T, L2T, LInterp[1], L1T, LInterp[0])
    Vcu, Vmu = computeCoarseTprimeMassTerm_jax(Levels, L3Tp, L2Tp, Lrc[3], Lrc[2], dt, Shapes, Vcu, Vmu)
    L1T, L2T, T3 = computeSolutions(Levels, ne_nn, tmp_ne_nn, F, Vcu, LInterp, Lk, Lrc, Vmu, dt, p)
    L1T, L2T = _clampT(p, L1T), _clampT(p, L2T)
    Levels[3]["T0"] = _clampT(p, T3)
    (Levels[3]["Tprime0"], Levels[2]["Tprime0"], Levels[2]["T0"], Levels[1]["T0"]) = getBothNewTprimes(
        Levels, Levels[3]["T0"], L2T, LInterp[1], L1T, LInterp[0])
    S1_0 = np.array(Levels[0]["S1"], dtype=float)
    S1_0[Levels[0]["idx"]] = Levels[3]["S1"]
    Levels[0]["S1"] = S1_0
    S2_0 = np.zeros_like(np.asarray(Levels[0]["S2"]), dtype=bool)
    S2_0[Levels[0]["idx"]] = Levels[3]["S2"]
    Levels[0]["S2"] = S2_0
    reset = ((1 - 2 * preS2.astype(float)) * np.asarray(Levels[3]["S2"])) == 1
    return Levels, reset


def stepGOMELTDwellTime(Levels, tmp_ne_nn, ne_nn, properties, dt, substrate):
    p = properties
    L1 = Levels[1]
    Fc = computeConvRadBC(L1, L1["T0"], tmp_ne_nn[0], ne_nn[2], p, F=0)
    _, _, k, rc = computeStateProperties(L1["T0"], L1["S1"], p, substrate[1])
    T = solveMatrixFreeFE(L1, ne_nn[2], tmp_ne_nn[0], k, rc, dt, L1["T0"], Fc, 0)
    T = substitute_Tbar(T, tmp_ne_nn[1], p["T_amb"])
    Levels[1]["T0"] = assignBCs(T, Levels)
    return Levels


def melting_temp(temps, delt_T, T_melt, accum_time, idx):
    """:3696-3712."""
    out = np.array(accum_time, dtype=float)
    np.add.at(out, idx, (np.asarray(temps) > T_melt) * delt_T)
    return out
