"""The reference-named call surface (go-melt_gb300/computeFunctions.py) on the
GPU against the reference's own per-function golden vectors.

Each test calls a function by its reference name and positional signature
(go_melt/computeFunctions.py of JLnorthwestern/GO-MELT) on the golden unit
state -- the windows moved to a non-trivial place, smooth non-trivial fields,
random Level-0 phases -- and compares with the vector the unmodified
reference computed on the same inputs (tests/golden/make_golden.py,
``unit_vectors``).  The level-solve wrappers with boundary handling
(computeL1Temperature, computeL2Temperature, computeSolutions_L3) have no
golden vector of their own; they are compared with the oracle's restatement,
which tests/test_oracle_golden.py pins to the reference.

Tolerances: FP64 1e-10 and FP32 1e-4 relative to the largest magnitude of
the reference vector (the FP32 bar: 1e-4 relative max temperature).
"""

import json

import numpy as np
import pytest
import torch

import gomelt_oracle as O
import stateio
from conftest import golden

pytestmark = pytest.mark.gpu

TOL = [(torch.float64, 1e-10), (torch.float32, 1e-4)]


def tup(g, key):
    return tuple(int(np.asarray(x)) for x in stateio.unflatten(g, key))


def host(t):
    return t.double().cpu().numpy() if torch.is_tensor(t) else np.asarray(t, dtype=float)


def rel(got, ref):
    got, ref = host(got).reshape(-1), np.asarray(ref, dtype=float).reshape(-1)
    assert got.shape == ref.shape, (got.shape, ref.shape)
    return float(np.max(np.abs(got - ref)) / max(float(np.max(np.abs(ref))), 1e-300))


def api_levels(g, dtype):
    """Levels of the GPU module on the golden unit state."""
    import computeFunctions as CF

    cfg = json.loads(str(g["cfg_json"]))
    P = stateio.unflatten(g, "properties")
    Levels = CF.SetupLevels(cfg, P, dtype=dtype)
    L = stateio.unflatten(g, "u.state")
    e = Levels.engine
    e.load_levels(L)
    e.tmp = tup(g, "u.tmp_ne_nn")
    e.substrate = tup(g, "u.substrate")
    return CF, Levels, L, P, cfg


@pytest.mark.parametrize("dtype,tol", TOL)
def test_computeStateProperties(case, dtype, tol):
    g = golden(case)
    CF, Levels, L, P, _ = api_levels(g, dtype)
    T = torch.as_tensor(g["u.props.T"], dtype=dtype, device="cuda")
    S1 = torch.as_tensor(g["u.props.S1"], dtype=dtype, device="cuda")
    S1o, S2o, k, rc = CF.computeStateProperties(T, S1, P, int(g["u.props.substrate"]))
    np.testing.assert_array_equal(host(S1o), g["u.props.out.S1"])
    np.testing.assert_array_equal(S2o.cpu().numpy(), np.asarray(g["u.props.out.S2"]).astype(bool))
    assert rel(k, g["u.props.out.k"]) < tol
    assert rel(rc, g["u.props.out.rhocp"]) < tol


@pytest.mark.parametrize("dtype,tol", TOL)
def test_computeSourcesL3_and_computeConvRadBC(case, dtype, tol):
    g = golden(case)
    CF, Levels, L, P, cfg = api_levels(g, dtype)
    ne_nn = tup(g, "u.ne_nn")
    tmp = tup(g, "u.tmp_ne_nn")
    Pw = float(cfg["properties"]["laser_power"])
    assert rel(CF.computeSourcesL3(Levels[3], g["u.move.in.v"], ne_nn, P, Pw), g["u.src3.out"]) < tol
    assert rel(CF.computeConvRadBC(Levels[3], Levels[3]["T0"], ne_nn[1], ne_nn[4], P, 0), g["u.conv3.out"]) < tol
    assert rel(CF.computeConvRadBC(Levels[1], Levels[1]["T0"], tmp[0], ne_nn[2], P, 0), g["u.conv1.out"]) < tol


@pytest.mark.parametrize("dtype,tol", TOL)
@pytest.mark.parametrize("lev", [3, 1])
def test_solveMatrixFreeFE(case, lev, dtype, tol):
    g = golden(case)
    CF, Levels, L, P, _ = api_levels(g, dtype)
    ne_nn = tup(g, "u.ne_nn")
    tmp = tup(g, "u.tmp_ne_nn")
    nn, ne = (ne_nn[4], ne_nn[1]) if lev == 3 else (ne_nn[2], tmp[0])
    pre = f"u.solve{lev}."
    out = CF.solveMatrixFreeFE(Levels[lev], nn, ne, g[pre + "k"], g[pre + "rhocp"], float(g[pre + "dt"]),
                               Levels[lev]["T0"], g[pre + "F"], g[pre + "Corr"])
    ref = np.asarray(g[pre + "out"], dtype=float)
    ok = np.isfinite(ref)  # the reference divides by zero above the active elements
    assert ok.sum() > 0
    assert rel(host(out)[ok], ref[ok]) < tol


def _oracle_solves(g, L, lev, rng):
    """Random positive properties and right-hand sides, the oracle's result."""
    P = stateio.unflatten(g, "properties")
    ne_nn = tup(g, "u.ne_nn")
    tmp = tup(g, "u.tmp_ne_nn")
    nn = int(np.asarray(L[lev]["nn"]))
    k = rng.uniform(0.005, 0.03, nn)
    rc = rng.uniform(0.002, 0.005, nn)
    F = rng.standard_normal(nn) * 1e-3
    V = rng.standard_normal(nn) * 1e-4
    dt = 3e-6
    if lev == 1:
        ref = O.computeL1Temperature(L, ne_nn, tmp, F, V, k, rc, dt, P)
    elif lev == 2:
        I12 = O.interpolatePointsMatrix(L[1], L[2]["node_coords"])
        ref = O.computeL2Temperature(L[1]["T0"], I12, L, ne_nn, L[2]["T0"], F, V, k, rc, dt)
    else:
        I23 = O.interpolatePointsMatrix(L[2], L[3]["node_coords"])
        ref = O.computeSolutions_L3(L[2]["T0"], I23, L, ne_nn, L[3]["T0"], F, k, rc, dt)
    return (k, rc, F, V, dt), np.asarray(ref, dtype=float)


@pytest.mark.parametrize("dtype,tol", TOL)
@pytest.mark.parametrize("lev", [1, 2, 3])
def test_level_temperature_surface(case, lev, dtype, tol):
    """computeL1Temperature / computeL2Temperature / computeSolutions_L3: the
    solve plus the level's boundary handling (Level-1 faces and inactive
    nodes, prolongated coarse ring for Levels 2 and 3)."""
    g = golden(case)
    CF, Levels, L, P, _ = api_levels(g, dtype)
    ne_nn = tup(g, "u.ne_nn")
    tmp = tup(g, "u.tmp_ne_nn")
    (k, rc, F, V, dt), ref = _oracle_solves(g, L, lev, np.random.default_rng(40 + lev))
    if lev == 1:
        out = CF.computeL1Temperature(Levels, ne_nn, tmp, F, V, k, rc, dt, P)
    elif lev == 2:
        I12 = CF.interpolatePointsMatrix(Levels[1], Levels[2]["node_coords"])
        out = CF.computeL2Temperature(Levels[1]["T0"], I12, Levels, ne_nn, Levels[2]["T0"], F, V, k, rc, dt)
    else:
        I23 = CF.interpolatePointsMatrix(Levels[2], Levels[3]["node_coords"])
        out = CF.computeSolutions_L3(Levels[2]["T0"], I23, Levels, ne_nn, Levels[3]["T0"], F, k, rc, dt)
    assert rel(out, ref) < tol


@pytest.mark.parametrize("dtype,tol", TOL)
def test_interpolation_surface(case, dtype, tol):
    """interpolatePointsMatrix / interpolate_w_matrix / interpolatePoints on
    points partly outside the source window (the reference's validity rule)."""
    g = golden(case)
    CF, Levels, L, P, _ = api_levels(g, dtype)
    n = g["u.interp.pts_len"]
    pts = np.split(np.asarray(g["u.interp.pts"], dtype=float), np.cumsum(n)[:2])
    M = CF.interpolatePointsMatrix(Levels[2], pts)
    Nc, node = M[0], M[1]
    assert rel(Nc, g["u.interp.Nc"]) < (1e-12 if dtype == torch.float64 else 1e-6)
    np.testing.assert_array_equal(node.cpu().numpy(), np.asarray(g["u.interp.node"]))
    assert rel(CF.interpolate_w_matrix(M, Levels[2]["T0"]), g["u.interp.out"]) < tol
    assert rel(CF.interpolatePoints(Levels[2], Levels[2]["T0"], pts), g["u.interp.out"]) < tol


@pytest.mark.parametrize("dtype,tol", TOL)
@pytest.mark.parametrize("materialised", [False, True])
def test_getNewTprime(case, materialised, dtype, tol):
    """Restriction of the fine field onto the coarse overlap nodes and the new
    T' = T_f - I(T_c), with the separable map or the materialised matrix."""
    g = golden(case)
    CF, Levels, L, P, _ = api_levels(g, dtype)
    C2F = CF.interpolatePointsMatrix(Levels[2], Levels[3]["node_coords"])
    if materialised:
        C2F = [C2F[0], C2F[1]]  # a plain [Nc, node] pair, no separable map
    Tp, Tc = CF.getNewTprime(Levels[3], Levels[3]["T0"], Levels[2]["T0"], Levels[2], C2F)
    scale = float(np.max(np.abs(g["u.tprime.Tc"])))
    assert rel(Tc, g["u.tprime.Tc"]) < tol
    assert float(np.max(np.abs(host(Tp) - np.asarray(g["u.tprime.Tp"])))) / scale < tol


@pytest.mark.parametrize("dtype,tol", TOL)
def test_coarse_source_and_tprime_terms(case, dtype, tol):
    """computeLevelSource onto Levels 1 and 2, and the subgrid flux (Part 1)
    and mass (Part 2) terms of both coarse levels."""
    g = golden(case)
    CF, Levels, L, P, _ = api_levels(g, dtype)
    ne_nn = tup(g, "u.ne_nn")
    sub = tup(g, "u.substrate")
    Shapes = [CF.computeCoarseFineShapeFunctions(Levels[1], Levels[2]),
              CF.computeCoarseFineShapeFunctions(Levels[1], Levels[3]),
              CF.computeCoarseFineShapeFunctions(Levels[2], Levels[3])]
    assert rel(CF.computeLevelSource(Levels, ne_nn, g["u.lsrc.lp"], Shapes[1], P, g["u.lsrc.lP"]),
               g["u.lsrc.out1"]) < tol
    assert rel(CF.computeLevelSource(Levels, ne_nn, g["u.lsrc.lp"], Shapes[2], P, g["u.lsrc.lP"]),
               g["u.lsrc.out2"]) < tol
    _, _, k3, rc3 = CF.computeStateProperties(Levels[3]["T0"], Levels[3]["S1"], P, sub[3])
    _, _, k2, rc2 = CF.computeStateProperties(Levels[2]["T0"], Levels[2]["S1"], P, sub[2])
    assert rel(CF.computeL1TprimeTerms_Part1(Levels, ne_nn, k3, Shapes, k2), g["u.tp1.L1"]) < tol
    assert rel(CF.computeL2TprimeTerms_Part1(Levels, ne_nn, Levels[3]["Tprime0"], k3, Shapes), g["u.tp1.L2"]) < tol
    nn1, nn2 = int(np.asarray(L[1]["nn"])), int(np.asarray(L[2]["nn"]))
    assert rel(CF.computeL1TprimeTerms_Part2(Levels, ne_nn, g["u.tp2.Tp3n"], g["u.tp2.Tp2n"], rc3, rc2, 2e-5,
                                             Shapes, np.zeros(nn1)), g["u.tp2.L1"]) < tol
    assert rel(CF.computeL2TprimeTerms_Part2(Levels, ne_nn, g["u.tp2.Tp3n"], Levels[3]["Tprime0"], rc3, 2e-5,
                                             Shapes, np.zeros(nn2)), g["u.tp2.L2"]) < tol
