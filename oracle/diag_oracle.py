"""CPU definitions of the diagnostics that the GB300 implementation reports beside its
results: energy balance of a level window over an interval, melt-pool extent
at an isotherm, max / RMS field difference.

TEST INFRASTRUCTURE (like ``gomelt_oracle``): used by ``tests/`` only, as the
expected values of the device reductions in ``go-melt_gb300/csrc/gm_diag.cu``.  The
reference has no counterpart of these quantities; they are assembled here
from the oracle's restatements of the reference's own operators
(``solveMatrixFreeFE`` lumped mass and stiffness, ``computeSourcesL3``,
``computeConvRadBC``, ``computeStateProperties``), in FP64.
"""

from __future__ import annotations

import numpy as np

import gomelt_oracle as O


def box_level(nodes, h, origin):
    """A Level dict (node coordinates and per-axis connectivity) of a
    structured box, as createMesh3D (:32-64) builds it."""
    ax = [(origin[d], origin[d] + h[d] * (nodes[d] - 1), nodes[d]) for d in range(3)]
    coords, connect = O.createMesh3D(*ax)
    return {"node_coords": coords, "connect": connect}


def interior_mask(nodes, ne_planes):
    """Nodes off the Dirichlet ring: 1 <= ix <= nx-2, 1 <= iy <= ny-2,
    1 <= iz <= ne_planes.  Flat, node-major with x fastest."""
    nx, ny, nz = nodes
    iz, iy, ix = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    m = (ix >= 1) & (ix <= nx - 2) & (iy >= 1) & (iy <= ny - 2) & (iz >= 1) & (iz <= ne_planes)
    return m.reshape(-1)


def energy_balance(nodes, h, origin, ne_planes, T0, T1, ph, substrate, interval, rows, props):
    """(stored, source, surface, conduction) [J] of the interior nodes; see
    include/gomelt.h gm_energy_args for the definition."""
    L = box_level(nodes, h, origin)
    nx, ny, nz = nodes
    ex, ey = nx - 1, ny - 1
    ne = ex * ey * ne_planes
    nn = nx * ny * nz
    T0 = np.asarray(T0, dtype=np.float64)
    T1 = np.asarray(T1, dtype=np.float64)
    Tb = 0.5 * (T0 + T1)
    S1 = (np.asarray(ph) & 1).astype(np.float64) if ph is not None else np.zeros(nn)
    _, _, k, _ = O.computeStateProperties(Tb, S1, props, substrate)
    inner = interior_mask(nodes, ne_planes)
    N, dNdx, wq = O.hex8_basis(O.getSampleCoords(L))
    wq = wq[0][0]
    NTN = N.T @ N
    BTB = sum(dNdx[:, :, d].T @ dNdx[:, :, d] for d in range(3))
    idx, _, _, _ = O.elem_nodes(ex, ey, nx, ny, np.arange(ne))
    kbar = k[idx].mean(axis=1)
    Ve = np.broadcast_to((NTN * wq).sum(axis=0)[None, :], idx.shape)
    V = np.bincount(idx.reshape(-1), Ve.reshape(-1), minlength=nn)[:nn]
    KT = np.bincount(idx.reshape(-1), ((Tb[idx] @ BTB.T) * (kbar * wq)[:, None]).reshape(-1), minlength=nn)[:nn]
    stored = float((V * (enthalpy(T1, props) - enthalpy(T0, props)))[inner].sum())
    conduct = float(-interval * KT[inner].sum())
    Fs = O.computeConvRadBC(L, Tb, ne, nn, props, np.zeros(nn))
    surface = float(interval * Fs[inner].sum())
    source = 0.0
    for r in np.asarray(rows, dtype=np.float64).reshape(-1, 7):
        F = O.computeSourcesL3(L, r, [0, ne, 0, 0, nn], props, r[6])
        source += float(r[5] * np.asarray(F)[:nn][inner].sum())
    return stored, source, surface, conduct


def enthalpy(T, p):
    """rho * integral of the phase model's c_p (computeStateProperties,
    :2567-2614) from 0 to T."""
    T = np.asarray(T, dtype=np.float64)
    Ts, Tl = p["T_solidus"], p["T_liquidus"]
    a0, a1, cm, cf = p["cp_solid_coeff_a0"], p["cp_solid_coeff_a1"], p["cp_mushy"], p["cp_fluid"]
    Hs = a0 * Ts + 0.5 * a1 * Ts * Ts
    H = np.where(T <= Ts, a0 * T + 0.5 * a1 * T * T,
                 np.where(T < Tl, Hs + cm * (T - Ts), Hs + cm * (Tl - Ts) + cf * (T - Tl)))
    return p["rho"] * H


def energy_residual(terms, rows, props):
    stored, source, surface, conduct = terms
    rows = np.asarray(rows, dtype=np.float64).reshape(-1, 7)
    e_in = props["laser_eta"] * float((rows[:, 5] * rows[:, 6]).sum())
    return abs(stored - source - surface - conduct) / e_in


def melt_pool(nodes, h, origin, T, iso):
    """(xmin, xmax, ymin, ymax, zmin, zmax, count) of the nodes with T >= iso,
    each extended to the linear isotherm crossing towards colder neighbours."""
    nx, ny, nz = nodes
    T = np.asarray(T, dtype=np.float64).reshape(nz, ny, nx)
    hot = T >= iso
    out = []
    for d, ax in ((0, 2), (1, 1), (2, 0)):  # x, y, z axes of the (z, y, x) array
        x = origin[d] + h[d] * np.arange(nodes[d])
        shape = [1, 1, 1]
        shape[ax] = -1
        X = np.broadcast_to(x.reshape(shape), T.shape)
        lo = np.where(hot, X, np.inf)
        hi = np.where(hot, X, -np.inf)
        Tm = np.roll(T, 1, axis=ax)  # neighbour at index - 1
        Tp = np.roll(T, -1, axis=ax)  # neighbour at index + 1
        idx = np.arange(nodes[d]).reshape(shape)
        has_m = np.broadcast_to(idx > 0, T.shape)
        has_p = np.broadcast_to(idx < nodes[d] - 1, T.shape)
        with np.errstate(divide="ignore", invalid="ignore"):
            cm = hot & has_m & (Tm < iso)
            cp = hot & has_p & (Tp < iso)
            lo = np.where(cm, X - h[d] * (T - iso) / (T - Tm), lo)
            hi = np.where(cp, X + h[d] * (T - iso) / (T - Tp), hi)
        out += [float(lo.min()), float(hi.max())]
    return tuple(out) + (float(hot.sum()),)


def field_error(a, b):
    d = np.asarray(a, dtype=np.float64) - np.asarray(b, dtype=np.float64)
    return float(np.abs(d).max()) if d.size else 0.0, float(np.sqrt((d * d).mean())) if d.size else 0.0
