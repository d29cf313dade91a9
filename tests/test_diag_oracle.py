"""The energy-balance definition on plain explicit steps (CPU, oracle only):
N forward-Euler steps of a window with a fixed Dirichlet ring balance to
within the trapezoidal error of evaluating the flux terms at (T0 + TN)/2."""

import numpy as np

import diag_oracle as D
import gomelt_oracle as O

NODES = (21, 17, 9)
H = (0.005, 0.005, 0.005)
ORIGIN = (0.0, 0.0, -0.04)


def plain_steps(P, nsteps, dt, rows, T0, S1):
    L = D.box_level(NODES, H, ORIGIN)
    nn = int(np.prod(NODES))
    ne = (NODES[0] - 1) * (NODES[1] - 1) * (NODES[2] - 1)
    ring = ~D.interior_mask(NODES, NODES[2] - 1)
    T = T0.copy()
    for r in rows[:nsteps]:
        S1n, S2, k, rc = O.computeStateProperties(T, S1, P, 0)
        F = np.asarray(O.computeSourcesL3(L, r, [0, ne, 0, 0, nn], P, r[6]))
        F = O.computeConvRadBC(L, T, ne, nn, P, F)
        Tn = O.solveMatrixFreeFE(L, nn, ne, k, rc, dt, T, F, np.zeros(nn))
        Tn[ring] = T0[ring]
        T = Tn
    return T


def test_plain_steps_balance():
    """Constant-property material of the benchmark configurations, N3 = 10
    steps at 0.9 of the stability limit: the residual is well below the 1 %
    acceptance threshold (about 0.3 % here).  (With a mushy-zone heat
    capacity the explicit apparent-capacity step itself does not conserve
    enthalpy across the phase change, so no bound is asserted for it.)"""
    import workloads

    P = O.SetupProperties(dict(workloads.MATERIAL))
    nn = int(np.prod(NODES))
    T0 = np.full(nn, P["T_amb"])
    S1 = np.ones(nn)
    dt = 0.9 * H[0] ** 2 / (2 * workloads.ALPHA)
    n = 10
    rows = np.zeros((n, 7))
    rows[:, 0] = 0.05 + np.arange(n) * 1e-3
    rows[:, 1] = 0.04
    rows[:, 5] = dt
    rows[:, 6] = 200.0
    TN = plain_steps(P, n, dt, rows, T0, S1)
    terms = D.energy_balance(NODES, H, ORIGIN, NODES[2] - 1, T0, TN, np.ones(nn, np.uint8), 0, n * dt, rows, P)
    r = D.energy_residual(terms, rows, P)
    assert terms[0] > 0.5 * terms[1]  # most of the deposited heat is still stored
    assert r < 0.01, (terms, r)


def test_melt_pool_box():
    """A box-shaped hot region: extents are the interpolated crossings."""
    nx, ny, nz = NODES
    T = np.full((nz, ny, nx), 1000.0)
    T[5:9, 4:10, 6:15] = 3000.0
    ext = D.melt_pool(NODES, H, ORIGIN, T.reshape(-1), 2000.0)
    # crossing halfway between the hot node and its cold neighbour
    assert np.isclose(ext[0], ORIGIN[0] + H[0] * 5.5) and np.isclose(ext[1], ORIGIN[0] + H[0] * 14.5)
    assert np.isclose(ext[2], ORIGIN[1] + H[1] * 3.5) and np.isclose(ext[3], ORIGIN[1] + H[1] * 9.5)
    assert np.isclose(ext[4], ORIGIN[2] + H[2] * 4.5) and ext[5] == ORIGIN[2] + H[2] * 8
    assert ext[6] == 4 * 6 * 9
