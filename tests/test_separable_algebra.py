"""The algebra of the separable level step, restated on the CPU and checked
against the oracle's element-by-element solveMatrixFreeFE.  CPU only.

For constant k and rho*c the element sum of solveMatrixFreeFE
(computeFunctions.py:582-642) is the assembled brick operator
k [Kx (x) My (x) Mz + Mx (x) Ky (x) Mz + Mx (x) My (x) Kz] T with the lumped
mass (rho c / dt)(hx hy hz / 8) times the element count of the node.  The
separable kernel (level_sep_kernel in gm_level.cu) evaluates it per node as
  Zm = Tm + Tp + 4 T0, Zk = 2 T0 - Tm - Tp   (one-sided on the top plane:
  Zm = Tm + 2 T0, Zk = T0 - Tm),
  u, w = y-neighbour sums of Zm, Zk,
  A = a1 (u + 4 Zm), B = b1 (2 Zm - u) + b2 (w + 4 Zk),
  K T = 2 A + 4 B + D(x-1) + D(x+1), D = B - A,
with a1, b1, b2 = k hy hz / (36 hx), k hx hz / (36 hy), k hx hy / (36 hz),
and T+ = T + (-K T) dt / (hx hy hz rho c) (twice that on the top plane).
This file restates exactly those formulas in NumPy and compares them with the
oracle on anisotropic grids, with all element planes active and with inactive
planes above the top.  It also checks the Hadamard-mode form of the element
matrix that the element-tile kernel applies (any material), the kernels'
separable laser-source factors and their top-surface flux assembly.
"""

import numpy as np
import pytest

import gomelt_oracle as O


def level(nx, ny, nz, h):
    coords, connect = O.createMesh3D((0.0, h[0] * (nx - 1), nx), (0.0, h[1] * (ny - 1), ny),
                                     (-h[2] * (nz - 1), 0.0, nz))
    return {"node_coords": coords, "connect": connect}


def separable_step(T, k, rc, dt, h, ntop):
    """New temperatures of the nodes off the x/y ring on node planes
    1..ntop, in the kernel's order of operations (no source, no flux)."""
    hx, hy, hz = h
    a1, b1, b2 = k * hy * hz / (36 * hx), k * hx * hz / (36 * hy), k * hx * hy / (36 * hz)
    minv = dt / (hx * hy * hz * rc)
    out = {}
    for p in range(1, ntop + 1):
        Tm, T0 = T[p - 1], T[p]
        if p < ntop:
            Tp = T[p + 1]
            s = Tm + Tp
            Zm, Zk, mi = s + 4 * T0, 2 * T0 - s, minv
        else:
            Zm, Zk, mi = Tm + 2 * T0, T0 - Tm, 2 * minv
        u = Zm[:-2] + Zm[2:]  # rows 1..ny-2
        w = Zk[:-2] + Zk[2:]
        A = a1 * (u + 4 * Zm[1:-1])
        B = b1 * (2 * Zm[1:-1] - u) + b2 * (w + 4 * Zk[1:-1])
        D = B - A
        KT = (2 * A[:, 1:-1] + 4 * B[:, 1:-1]) + (D[:, :-2] + D[:, 2:])
        out[p] = T0[1:-1, 1:-1] + (-KT) * mi
    return out


@pytest.mark.parametrize("dims,h,inactive", [
    ((13, 9, 8), (0.010, 0.015, 0.007), 0),
    ((7, 11, 5), (0.020, 0.005, 0.012), 0),
    ((10, 8, 9), (0.005, 0.005, 0.005), 3),  # the top three node planes inactive
    ((6, 6, 3), (0.004, 0.006, 0.005), 1),   # one active element plane
])
def test_separable_form_equals_element_sum(dims, h, inactive):
    nx, ny, nz = dims
    L = level(nx, ny, nz, h)
    hs = [float(np.asarray(L["node_coords"][d])[1] - np.asarray(L["node_coords"][d])[0]) for d in range(3)]
    ntop = nz - 1 - inactive  # top of the active element planes (node plane index)
    ne = (nx - 1) * (ny - 1) * ntop
    rng = np.random.default_rng(nx * 100 + ny * 10 + nz)
    nn = nx * ny * nz
    T = 300 + 1500 * rng.random(nn)
    k, rc, dt = 0.022, 4.4e-6 * 700, 1.5e-6
    with np.errstate(divide="ignore", invalid="ignore"):
        ref = O.solveMatrixFreeFE(L, nn, ne, np.full(nn, k), np.full(nn, rc), dt, T, np.zeros(nn), np.zeros(nn))
    ref = ref.reshape(nz, ny, nx)
    got = separable_step(T.reshape(nz, ny, nx), k, rc, dt, hs, ntop)
    T3 = T.reshape(nz, ny, nx)
    for p in range(1, ntop + 1):
        inc_ref = ref[p, 1:-1, 1:-1] - T3[p, 1:-1, 1:-1]
        inc_got = got[p] - T3[p, 1:-1, 1:-1]
        scale = np.abs(inc_ref).max()
        assert scale > 0
        np.testing.assert_allclose(inc_got, inc_ref, rtol=0, atol=1e-10 * scale)


def test_lumped_mass_counts():
    """The lumped mass of solveMatrixFreeFE is (rho c / dt)(h^3 / 8) times the
    node's element count: 8 inside, 4 on the top plane (the constants the
    kernel folds into dt / (hx hy hz rho c) and twice that on the top)."""
    nx, ny, nz = 6, 5, 4
    h = (0.01, 0.02, 0.005)
    L = level(nx, ny, nz, h)
    nn = nx * ny * nz
    ne = (nx - 1) * (ny - 1) * (nz - 1)
    rc, dt = 3.08e-3, 2e-6
    # with K T = 0 (uniform T) and F = 1 the update returns 1 + 1/M
    T = np.ones(nn)
    with np.errstate(divide="ignore", invalid="ignore"):
        out = O.solveMatrixFreeFE(L, nn, ne, np.full(nn, 0.02), np.full(nn, rc), dt, T, np.ones(nn), np.zeros(nn))
    M = 1.0 / (out - 1.0)
    M = M.reshape(nz, ny, nx)
    m8 = rc / dt * h[0] * h[1] * h[2]
    np.testing.assert_allclose(M[1:-1, 1:-1, 1:-1], m8, rtol=1e-12)
    np.testing.assert_allclose(M[-1, 1:-1, 1:-1], m8 / 2, rtol=1e-12)


# reference local node order of a hex8 element (convert2XYZ, :676-687): (x, y, z) corner bits
CORNERS = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]


@pytest.mark.parametrize("h", [(0.005, 0.005, 0.005), (0.01, 0.02, 0.005), (0.1, 0.02, 0.0025)])
def test_hadamard_stiffness_equals_element_matrix(h):
    """The element-tile kernel (level_body in gm_level.cu) applies the brick
    stiffness as a forward Hadamard butterfly of the 8 corner values, a
    scaling of modes 1..7 by lam_m k and the inverse butterfly, with
    lam_m = (Kx My Mz + Mx Ky Mz + Mx My Kz) / 8 from the 1-D eigenvalues
    (K: 0 or 2/h, M: h/2 or h/6 for the constant or the difference mode).
    That equals the reference's element matrix BTB * wq of
    solveMatrixFreeFE (2x2x2 Gauss); the lumped mass per corner is
    wq = hx hy hz / 8."""
    hx, hy, hz = h
    coords = np.array([[c[0] * hx, c[1] * hy, c[2] * hz] for c in CORNERS], dtype=float)
    N, dNdx, wq = O.hex8_basis(coords)
    BTB = sum(dNdx[:, :, d].T @ dNdx[:, :, d] for d in range(3))
    K_ref = BTB * wq[0][0]
    K_had = np.zeros((8, 8))
    for m in range(8):
        mx, my, mz = m & 1, (m >> 1) & 1, (m >> 2) & 1
        Mx, My, Mz = (hx / 6 if mx else hx / 2), (hy / 6 if my else hy / 2), (hz / 6 if mz else hz / 2)
        Kx, Ky, Kz = (2 / hx if mx else 0.0), (2 / hy if my else 0.0), (2 / hz if mz else 0.0)
        lam = (Kx * My * Mz + Mx * Ky * Mz + Mx * My * Kz) / 8.0
        v = np.array([np.prod([(1.0 if c[d] else -1.0) if (m >> d) & 1 else 1.0 for d in range(3)])
                      for c in CORNERS])
        K_had += lam * np.outer(v, v)
    np.testing.assert_allclose(K_had, K_ref, rtol=0, atol=1e-12 * np.abs(K_ref).max())
    # lumped mass: row sums of N^T N wq are the same for every corner
    np.testing.assert_allclose((N.T @ N * wq[0][0]).sum(axis=0), hx * hy * hz / 8, rtol=1e-13)


def src_factor(i, n, rel, h, inv_r2):
    """1-D laser factor of node i (src_factor in gm_common.cuh): the two
    elements e = i-1, i at their two Gauss points, weighted by node i's
    linear shape function there."""
    g0, g1 = (1 - 1 / np.sqrt(3)) / 2, (1 + 1 / np.sqrt(3)) / 2
    s = 0.0
    for e in (i - 1, i):
        if e < 0 or e >= n - 1:
            continue
        d0 = rel + h * (e + g0)
        d1 = rel + h * (e + g1)
        q0 = np.exp(-3 * d0 * d0 * inv_r2)
        q1 = np.exp(-3 * d1 * d1 * inv_r2)
        s += (g1 * q0 + g0 * q1) if i == e else (g0 * q0 + g1 * q1)
    return s


@pytest.mark.parametrize("laser", [(0.031, 0.052, -0.001), (0.0, 0.09, 0.0), (0.2, -0.05, -0.03)])
def test_separable_laser_source_equals_gauss_point_sum(laser):
    """The level kernels evaluate computeSourcesL3 (:2960-3012) as
    src_c P fx(i) fy(j) fz(k), src_c = 6 sqrt(3) eta rc^2 dc (hx hy hz / 8),
    rc = 1 / (r sqrt(pi)), dc = 1 / (d sqrt(pi)), with the 1-D factors above;
    the reference sums the 3-D Gaussian at the 8 Gauss points of every
    element.  The last laser position lies outside the window."""
    nx, ny, nz = 17, 12, 7
    h = (0.007, 0.011, 0.005)
    L = level(nx, ny, nz, h)
    props = {"laser_eta": 0.35, "laser_radius": 0.05, "laser_depth": 0.03}
    P = 200.0
    ne, nn = (nx - 1) * (ny - 1) * (nz - 1), nx * ny * nz
    ref = O.computeSourcesL3(L, np.asarray(laser), (0, ne, 0, 0, nn), props, P).reshape(nz, ny, nx)
    c = [np.asarray(L["node_coords"][d], dtype=float) for d in range(3)]
    r, dd = props["laser_radius"], props["laser_depth"]
    rc, dc = 1 / (r * np.sqrt(np.pi)), 1 / (dd * np.sqrt(np.pi))
    src_c = 6 * np.sqrt(3) * props["laser_eta"] * rc * rc * dc * (h[0] * h[1] * h[2] / 8)
    fx = np.array([src_factor(i, nx, c[0][0] - laser[0], h[0], 1 / r**2) for i in range(nx)])
    fy = np.array([src_factor(j, ny, c[1][0] - laser[1], h[1], 1 / r**2) for j in range(ny)])
    fz = np.array([src_factor(k, nz, c[2][0] - laser[2], h[2], 1 / dd**2) for k in range(nz)])
    got = src_c * P * fz[:, None, None] * fy[None, :, None] * fx[None, None, :]
    scale = np.abs(ref).max()
    assert scale > 0
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-11 * scale)


def surface_flux(gp, Tq):
    """surface_flux of gm_common.cuh on the product's gm_props [W/mm^2]."""
    Tq = np.minimum(Tq, gp.T_boiling + 1000)
    q = gp.h_conv * (gp.T_amb - Tq) + gp.sigma_sb * gp.emissivity * (gp.T_amb ** 4 - Tq ** 4)
    if gp.evc != 0:
        S = (gp.evc * gp.CP_coeff * np.exp(-gp.CT_coeff * (1 / Tq - 1 / gp.T_boiling)) * np.sqrt(gp.CM_coeff / Tq)
             * (gp.Lev + gp.cp_fluid * (Tq - gp.T_amb)))
        q = q - S
    return q * 1e-6


@pytest.mark.parametrize("evaporation", [0.0, 0.82])
def test_surface_flux_assembly_equals_reference(evaporation):
    """The top-surface flux of the level kernels (sep_surface in
    gm_level.cu): per top element the 2 x 2 Gauss points of its upper face
    with the bilinear weights (1 +- 1/sqrt3)/2, q(Tq) hx hy / 4, gathered to
    the four corners; the flux constants come from the product's gm_props
    (_native.props_struct).  Reference: computeConvRadBC (:2207-2301)."""
    import _native as N

    P = O.SetupProperties({
        "thermal_conductivity_powder": 0.4, "thermal_conductivity_bulk_a0": 4.23,
        "thermal_conductivity_bulk_a1": 0.016, "thermal_conductivity_fluid_a0": 29.0,
        "heat_capacity_solid_a0": 383.1, "heat_capacity_solid_a1": 0.174, "heat_capacity_mushy": 3235.0,
        "heat_capacity_fluid": 769.0, "density": 8e-06, "laser_radius": 0.04, "laser_depth": 0.03,
        "laser_power": 250.0, "laser_absorptivity": 0.45, "T_amb": 298.15, "T_solidus": 1533,
        "T_liquidus": 1609, "T_boiling": 3038.0, "h_conv": 1.5e-05, "emissivity": 0.3,
        "evaporation_coefficient": evaporation, "layer_height": 0.02})
    gp = N.props_struct(P)
    nx, ny, nz = 11, 9, 4
    hx, hy = 0.006, 0.009
    L = level(nx, ny, nz, (hx, hy, 0.005))
    nn, ne = nx * ny * nz, (nx - 1) * (ny - 1) * (nz - 1)
    rng = np.random.default_rng(5)
    T = 300 + 3500 * rng.random(nn)  # includes temperatures above T_boiling + 1000
    ref = O.computeConvRadBC(L, T, ne, nn, P, np.zeros(nn)).reshape(nz, ny, nx)
    Tt = T.reshape(nz, ny, nx)[-1]
    PQ, MQ = (1 + 1 / np.sqrt(3)) / 2, (1 - 1 / np.sqrt(3)) / 2
    w2 = hx * hy / 4
    F = np.zeros((ny, nx))
    for ey in range(ny - 1):
        for ex in range(nx - 1):
            t00, t10, t01, t11 = Tt[ey, ex], Tt[ey, ex + 1], Tt[ey + 1, ex], Tt[ey + 1, ex + 1]
            for qy in (0, 1):
                for qx in (0, 1):
                    px0, px1 = (MQ, PQ) if qx else (PQ, MQ)
                    py0, py1 = (MQ, PQ) if qy else (PQ, MQ)
                    Tq = px0 * py0 * t00 + px1 * py0 * t10 + px0 * py1 * t01 + px1 * py1 * t11
                    q = surface_flux(gp, Tq) * w2
                    F[ey, ex] += px0 * py0 * q
                    F[ey, ex + 1] += px1 * py0 * q
                    F[ey + 1, ex] += px0 * py1 * q
                    F[ey + 1, ex + 1] += px1 * py1 * q
    scale = np.abs(ref).max()
    assert scale > 0 and np.abs(ref[:-1]).max() == 0  # flux on the top plane only
    np.testing.assert_allclose(F, ref[-1], rtol=0, atol=1e-12 * scale)
