"""The algebra of the separable coupling terms, restated on the CPU and
checked against the oracle's element reduction.  CPU only.

For constant k and rho*c the subgrid flux and mass terms of the coarse level
(computeCoarseTprimeTerm_jax / computeCoarseTprimeMassTerm_jax,
computeFunctions.py:1396-1565, and the Part-1/Part-2 functions that call
them) are tensor products of 1-D maps from the fine nodes of the window to
the coarse nodes of its box:
  V = k [cf0 (Dx Iy Iz) + cf1 (Ix Dy Iz) + cf2 (Ix Iy Dz)] T'
      - (wq / dt) rho c (Ix Iy Iz)(dTa - dTb),
  cf_d = -2 wq / (H_d h_d), wq = hx hy hz / 8,
with, per axis, D[N, i] the coarse gradient sign times the fine difference
over the fine elements assigned to coarse element N - A, and I[N, i] the
Gauss-side coarse weights times the fine linear shape functions.  The
per-axis tables come from the product's host geometry (geometry.couple_axis)
and the contraction follows couple_sep_x/y/z of gm_couple.cu.  Fine elements
are assigned to the coarse element of their first Gauss point while each
point keeps the weights of its own element, as the reference does; the
offset windows below make fine elements straddle coarse nodes.  The coarse
laser source (computeLevelSource, :2667-2730) factorises the same way and is
checked against the oracle's Gauss-point sum; the prolongation's per-axis
tables and validity rule are checked against interpolatePoints.
"""

import numpy as np
import pytest

import gomelt_oracle as O
from geometry import couple_axis

PQ, MQ = (1 + 1 / np.sqrt(3)) / 2, (1 - 1 / np.sqrt(3)) / 2


def level(lo, hi, n):
    coords, connect = O.createMesh3D((lo[0], hi[0], n[0]), (lo[1], hi[1], n[1]), (lo[2], hi[2], n[2]))
    return {"node_coords": coords, "connect": connect, "nn": n[0] * n[1] * n[2]}


def axis_maps(ax):
    """D and I of one axis over the box: (ncb + 1) coarse nodes x fine nodes."""
    ncb, flo, fhi, cw = ax["ncb"], ax["flo"], ax["fhi"], ax["cw"]
    f0 = int(flo[0])
    nfn = int(fhi[ncb - 1]) - f0 + 1
    D = np.zeros((ncb + 1, nfn))
    I = np.zeros((ncb + 1, nfn))
    for N in range(ncb + 1):
        for A in (1, 0):
            c = N - A
            if c < 0 or c >= ncb:
                continue
            sg = 1.0 if A else -1.0
            for e in range(flo[c], fhi[c]):
                a0 = cw[e, 0, A] * PQ + cw[e, 1, A] * MQ
                a1 = cw[e, 0, A] * MQ + cw[e, 1, A] * PQ
                i = e - f0
                D[N, i + 1] += sg
                D[N, i] -= sg
                I[N, i] += a0
                I[N, i + 1] += a1
    return D, I, f0, nfn


def separable_terms(fine, coarse, k, rc, dt, Tp, dT):
    axes = [couple_axis(fine["node_coords"][d], coarse["node_coords"][d]) for d in range(3)]
    maps = [axis_maps(a) for a in axes]
    h = [float(np.asarray(fine["node_coords"][d])[1] - np.asarray(fine["node_coords"][d])[0]) for d in range(3)]
    wq = h[0] * h[1] * h[2] / 8
    cf = [-2 * wq / (axes[d]["H"] * h[d]) for d in range(3)]
    nf = [np.asarray(fine["node_coords"][d]).size for d in range(3)]
    sl = tuple(slice(maps[d][2], maps[d][2] + maps[d][3]) for d in (2, 1, 0))
    (Dx, Ix, _, _), (Dy, Iy, _, _), (Dz, Iz, _, _) = maps
    F = Tp.reshape(nf[2], nf[1], nf[0])[sl]
    G = dT.reshape(nf[2], nf[1], nf[0])[sl]
    V = k * (cf[0] * np.einsum("ak,bj,ci,kji->abc", Iz, Iy, Dx, F)
             + cf[1] * np.einsum("ak,bj,ci,kji->abc", Iz, Dy, Ix, F)
             + cf[2] * np.einsum("ak,bj,ci,kji->abc", Dz, Iy, Ix, F))
    V -= (wq * rc / dt) * np.einsum("ak,bj,ci,kji->abc", Iz, Iy, Ix, G)
    return V, [a["lo"] for a in axes]


def element_terms(fine, coarse, k, rc, dt, Tp, dT):
    shape = O.computeCoarseFineShapeFunctions(coarse, fine)
    nn = fine["nn"]
    flux, wq = O._fine_flux(fine, Tp, np.full(nn, k))
    mass, w = O._fine_mass(fine, dT, np.full(nn, rc), dt)
    nnc = coarse["nn"]
    return O._flux_project(shape, flux, wq, nnc) + O._mass_project(shape, mass, w, nnc)


CASES = {
    # Level-3 window in a Level-2 level (ratio 4), grids aligned
    "l3_in_l2": (((0.6, 0.6, -0.2), (1.4, 1.4, 0.0), (41, 41, 11)),
                 ((0.8, 0.9, -0.06), (1.2, 1.1, 0.0), (81, 41, 13))),
    # Level-3 window in a Level-1 level (ratio 20 in x/y, 20 in z)
    "l3_in_l1": (((0.0, 0.0, -0.6), (2.0, 2.0, 0.0), (21, 21, 7)),
                 ((0.8, 0.9, -0.06), (1.2, 1.1, 0.0), (81, 41, 13))),
    # offset window: fine elements straddle coarse nodes along every axis
    "offset": (((0.6, 0.6, -0.2), (1.4, 1.4, 0.0), (41, 41, 11)),
               ((0.813, 0.907, -0.0613), (1.0, 1.003, -0.0013), (35, 19, 9))),
    # anisotropic fine spacing, ratio 3 / 5 / 2
    "aniso": (((0.0, 0.0, -0.3), (1.2, 0.9, 0.0), (13, 10, 7)),
              ((0.3, 0.2, -0.2), (0.6, 0.5, 0.0), (10, 16, 5))),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_separable_coupling_equals_element_reduction(case):
    (clo, chi, cn), (flo, fhi, fn) = CASES[case]
    coarse, fine = level(clo, chi, cn), level(flo, fhi, fn)
    rng = np.random.default_rng(len(case))
    nn = fine["nn"]
    Tp = 50 * rng.standard_normal(nn)
    dT = 20 * rng.standard_normal(nn)
    k, rc, dt = 0.022, 4.4e-6 * 700, 1.575e-5
    ref = element_terms(fine, coarse, k, rc, dt, Tp, dT).reshape(cn[2], cn[1], cn[0])
    V, lo = separable_terms(fine, coarse, k, rc, dt, Tp, dT)
    box = tuple(slice(lo[d], lo[d] + V.shape[2 - d]) for d in (2, 1, 0))
    scale = np.abs(ref).max()
    assert scale > 0
    np.testing.assert_allclose(V, ref[box], rtol=0, atol=1e-11 * scale)
    outside = ref.copy()
    outside[box] = 0
    assert np.abs(outside).max() <= 1e-12 * scale  # no term outside the box


def coarse_source_separable(fine, coarse, props, rows):
    """coarse_source_tables / coarse_source_assemble of gm_couple.cu: per
    position p and axis d the 1-D table S_d[p][t] = sum over the fine Gauss
    points assigned to coarse node t of their coarse weight times
    exp(-3 (x_q - v_p)^2 / s^2) (s = r in x, y; laser depth in z), the x
    table times cpre P_p; coarse node value = mean over p of Sx Sy Sz."""
    axes = [couple_axis(fine["node_coords"][d], coarse["node_coords"][d]) for d in range(3)]
    h = [float(np.asarray(fine["node_coords"][d])[1] - np.asarray(fine["node_coords"][d])[0]) for d in range(3)]
    r, dd = props["laser_radius"], props["laser_depth"]
    rc, dc = 1 / (r * np.sqrt(np.pi)), 1 / (dd * np.sqrt(np.pi))
    cpre = 6 * np.sqrt(3) * props["laser_eta"] * rc * rc * dc * (h[0] * h[1] * h[2] / 8)
    out = 0.0
    for row in rows:
        S = []
        for d in range(3):
            ax = axes[d]
            s2 = dd * dd if d == 2 else r * r
            t = np.zeros(ax["ncb"] + 1)
            for N in range(ax["ncb"] + 1):
                for A in (1, 0):
                    c = N - A
                    if c < 0 or c >= ax["ncb"]:
                        continue
                    for e in range(ax["flo"][c], ax["fhi"][c]):
                        for sd in (0, 1):
                            dx = ax["xq"][e, sd] - row[d]
                            t[N] += ax["cw"][e, sd, A] * np.exp(-3 * dx * dx / s2)
            S.append(t * (cpre * row[6]) if d == 0 else t)
        out = out + np.einsum("a,b,c->abc", S[2], S[1], S[0])
    return out / len(rows), [a["lo"] for a in axes]


@pytest.mark.parametrize("case", ["l3_in_l2", "offset", "aniso"])
def test_separable_coarse_source_equals_gauss_point_sum(case):
    """gm_coarse_source against computeLevelSource (:2667-2730): the Level-3
    Gauss-point source averaged over the coarse step's laser positions and
    projected onto the coarse nodes."""
    (clo, chi, cn), (flo, fhi, fn) = CASES[case]
    coarse, fine = level(clo, chi, cn), level(flo, fhi, fn)
    props = {"laser_eta": 0.35, "laser_radius": 0.05, "laser_depth": 0.03}
    c = [np.asarray(fine["node_coords"][d]) for d in range(3)]
    mid = [0.5 * (c[d][0] + c[d][-1]) for d in range(3)]
    rows = np.zeros((5, 7))
    for i in range(5):  # a short track across the window, the last position outside it
        rows[i, :3] = [mid[0] - 0.02 + 0.01 * i, mid[1] + 0.004 * i, c[2][-1]]
        rows[i, 6] = 150.0 + 10 * i
    rows[4, 0] = c[0][-1] + 0.08
    shape = O.computeCoarseFineShapeFunctions(coarse, fine)
    ref = O.computeLevelSource({3: fine}, None, rows, shape, props, rows[:, 6], coarse["nn"])
    ref = ref.reshape(cn[2], cn[1], cn[0])
    V, lo = coarse_source_separable(fine, coarse, props, rows)
    box = tuple(slice(lo[d], lo[d] + V.shape[2 - d]) for d in (2, 1, 0))
    scale = np.abs(ref).max()
    assert scale > 0
    np.testing.assert_allclose(V, ref[box], rtol=0, atol=1e-11 * scale)
    outside = ref.copy()
    outside[box] = 0
    assert np.abs(outside).max() <= 1e-12 * scale


def test_separable_prolongation_equals_reference():
    """The transfer kernels (interp_kernel, ring_kernel in gm_transfer.cu)
    interpolate through per-axis tables of the host (geometry.axis_map: the
    clipped-floor source element and the two linear weights per target
    coordinate): the eight weights are products of per-axis weights in the
    order (x0 y0 z0, x1 y0 z0, x1 y1 z0, x0 y1 z0, then z1), all eight in
    [-0.01, 1.01] or the point gets zero, clipped to [0, 1].  Reference:
    interpolatePoints (:1131-1210); targets here reach outside the source grid
    on every axis."""
    from geometry import axis_map

    src = level((0.6, 0.6, -0.2), (1.4, 1.4, 0.0), (41, 41, 11))
    rng = np.random.default_rng(3)
    u = 300 + 1500 * rng.random(src["nn"])
    tgt = [np.sort(rng.uniform(0.55, 1.45, 23)), np.sort(rng.uniform(0.58, 1.43, 17)),
           np.sort(rng.uniform(-0.23, 0.02, 9))]
    ref = O.interpolatePoints(src, u, tgt)
    m = [axis_map(src["node_coords"][d], tgt[d]) for d in range(3)]
    nx, ny = 41, 41
    got = np.zeros((tgt[2].size, tgt[1].size, tgt[0].size))
    for k in range(tgt[2].size):
        for j in range(tgt[1].size):
            for i in range(tgt[0].size):
                (x0, x1), (y0, y1), (z0, z1) = m[0].w[i], m[1].w[j], m[2].w[k]
                w8 = np.array([x0 * y0 * z0, x1 * y0 * z0, x1 * y1 * z0, x0 * y1 * z0,
                               x0 * y0 * z1, x1 * y0 * z1, x1 * y1 * z1, x0 * y1 * z1])
                ok = (w8 >= -1e-2).all() and (w8 <= 1 + 1e-2).all()
                w8 = np.clip(w8, 0, 1) if ok else np.zeros(8)
                b = m[0].elem[i] + m[1].elem[j] * nx + m[2].elem[k] * nx * ny
                sx, sy, sz = 1, nx, nx * ny
                corners = [b, b + sx, b + sx + sy, b + sy, b + sz, b + sx + sz, b + sx + sy + sz, b + sy + sz]
                got[k, j, i] = (w8 * u[corners]).sum()
    assert (ref == 0).any() and (ref != 0).any()  # both valid and rejected points
    np.testing.assert_allclose(got.reshape(-1), ref, rtol=1e-13, atol=1e-9)
