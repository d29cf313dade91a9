"""GPU diagnostics (energy balance, melt pool, field error) against their
FP64 CPU definitions in oracle/diag_oracle.py."""

import numpy as np
import pytest
import torch

import diag_oracle as D_oracle
import gomelt_oracle as O
from test_gpu_level import PHASE_PROPS

pytestmark = pytest.mark.gpu

NODES = (23, 19, 11)
H = (0.01, 0.012, 0.008)
ORIGIN = (0.3, 0.45, -0.08)


def fields(seed=0):
    rng = np.random.default_rng(seed)
    nx, ny, nz = NODES
    x = ORIGIN[0] + H[0] * np.arange(nx)
    y = ORIGIN[1] + H[1] * np.arange(ny)
    z = ORIGIN[2] + H[2] * np.arange(nz)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    T0 = 298.15 + 2500 * np.exp(-((X - 0.41) ** 2 + (Y - 0.56) ** 2) / 0.002 + Z * 15)
    T1 = T0 + 40 * rng.standard_normal(T0.shape)
    ph = (rng.random(T0.shape) > 0.5).astype(np.uint8) | ((T0 > 1609) * 2).astype(np.uint8)
    rows = np.zeros((3, 7))
    rows[:, 0] = [0.40, 0.41, 0.42]
    rows[:, 1] = 0.56
    rows[:, 2] = 0.0
    rows[:, 5] = 1.2e-6
    rows[:, 6] = [250.0, 250.0, 200.0]
    return T0.reshape(-1), T1.reshape(-1), ph.reshape(-1), rows


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_energy_terms(dtype):
    import _native as N
    from diagnostics import Diagnostics

    P = O.SetupProperties(PHASE_PROPS)
    ps = N.props_struct(P)
    T0, T1, ph, rows = fields()
    if dtype == torch.float32:  # the oracle sees the same (rounded) inputs
        T0, T1 = T0.astype(np.float32).astype(np.float64), T1.astype(np.float32).astype(np.float64)
    ne_planes, substrate, interval = NODES[2] - 1, 2 * NODES[0] * NODES[1] + 5, 3.6e-6
    ref = D_oracle.energy_balance(NODES, H, ORIGIN, ne_planes, T0, T1, ph, substrate, interval, rows, P)
    dg = Diagnostics()
    got = dg.energy_terms(ps, nodes=NODES, h=H, origin=ORIGIN, ne_planes=ne_planes,
                          T0=torch.tensor(T0, dtype=dtype, device="cuda"),
                          T1=torch.tensor(T1, dtype=dtype, device="cuda"),
                          ph=torch.tensor(ph, device="cuda"), substrate=substrate, interval=interval, rows=rows)
    got = got.cpu().numpy()
    for g, r in zip(got, ref):
        assert abs(g - r) <= 1e-9 * max(abs(r), 1e-30), (got, ref)
    assert abs(dg.residual(got, rows, P["laser_eta"]) - D_oracle.energy_residual(ref, rows, P)) < 1e-9


def test_energy_partial_planes():
    """Inactive planes above ne_planes are outside the balance."""
    import _native as N
    from diagnostics import Diagnostics

    P = O.SetupProperties(PHASE_PROPS)
    ps = N.props_struct(P)
    T0, T1, ph, rows = fields(1)
    ne_planes = NODES[2] - 3
    ref = D_oracle.energy_balance(NODES, H, ORIGIN, ne_planes, T0, T1, ph, 0, 2e-6, rows, P)
    got = Diagnostics().energy_terms(ps, nodes=NODES, h=H, origin=ORIGIN, ne_planes=ne_planes,
                                     T0=torch.tensor(T0, device="cuda"), T1=torch.tensor(T1, device="cuda"),
                                     ph=torch.tensor(ph, device="cuda"), substrate=0, interval=2e-6,
                                     rows=rows).cpu().numpy()
    np.testing.assert_allclose(got, ref, rtol=1e-9)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("iso", [1609.0, 2000.0, 1e6])
def test_melt_pool(dtype, iso):
    from diagnostics import Diagnostics

    T0, _, _, _ = fields(2)
    T = T0.astype(np.float32).astype(np.float64) if dtype == torch.float32 else T0
    ref = D_oracle.melt_pool(NODES, H, ORIGIN, T, iso)
    got = Diagnostics().melt_pool(nodes=NODES, h=H, origin=ORIGIN, T=torch.tensor(T, dtype=dtype, device="cuda"),
                                  iso=iso)
    assert got["count"] == int(ref[6])
    if ref[6] == 0:
        assert got["length"] == 0.0 and got["depth"] == 0.0
    else:
        np.testing.assert_allclose(got["extents"], ref[:6], rtol=0, atol=1e-12)
        ztop = ORIGIN[2] + H[2] * (NODES[2] - 1)
        assert abs(got["depth"] - (ztop - ref[4])) < 1e-12


def test_field_error():
    from diagnostics import Diagnostics

    rng = np.random.default_rng(5)
    a = rng.standard_normal(100003) * 100 + 1000
    b = a + rng.standard_normal(a.size) * 1e-3
    dg = Diagnostics()
    m, r = dg.field_error(torch.tensor(a, dtype=torch.float32, device="cuda"), torch.tensor(b, device="cuda"))
    rm, rr = D_oracle.field_error(a.astype(np.float32), b)
    assert abs(m - rm) <= 1e-12 * max(rm, 1) and abs(r - rr) <= 1e-9 * rr


def test_energy_balance_closes_on_plain_steps():
    """On the plain multilevel path (single-track workload, constant
    properties) the Level-3 window's energy over each Level-2 step balances
    well inside the 1 % acceptance threshold of a predicted field once the
    window has warmed up."""
    import createPath
    import engine
    import levels
    import workloads
    from diagnostics import Diagnostics

    cfg = workloads.single_track()
    P = levels.setup_properties(cfg["properties"])
    nm = levels.setup_nonmesh(cfg["nonmesh"])
    rows = np.asarray(createPath.toolpath(nm, P, cfg["gcode"]), dtype=np.float64)
    vstart = np.asarray(cfg["properties"]["laser_center"], dtype=float)
    e = engine.Engine(cfg, P, 10, 10)
    e.set_layer(rows[0])
    dg = Diagnostics()
    res = []
    for k in range(6):
        c = rows[k * 100:(k + 1) * 100]
        e.move(c[0], vstart)
        T3s = e.T[3].clone()
        _, L3all, _ = e.subcycle(c, history=True)
        L3 = e.geo.L[3]
        for j in range(10):
            jr = c[j * 10:(j + 1) * 10]
            t = dg.energy_terms(e.ps, nodes=L3.nodes, h=L3.spacing(), origin=L3.origin(),
                                ne_planes=L3.nodes[2] - 1, T0=T3s if j == 0 else L3all[j - 1], T1=L3all[j],
                                ph=e.ph[3], substrate=e.substrate[3], interval=float(jr[:, 5].sum()), rows=jr)
            res.append((k, j, dg.residual(t, jr, P["laser_eta"])))
    # The trapezoidal flux terms are least accurate when the laser nears the
    # Dirichlet ring: on this 0.4 mm window that happens in the last Level-2
    # steps before each window move (measured up to ~1.5 %); while the laser
    # is well inside, the balance closes to ~0.1 %.
    inside = [r for k, j, r in res if k >= 1 and 1 <= j <= 6]
    assert max(inside) < 3e-3, res
    assert max(r for k, j, r in res) < 2e-2, res
