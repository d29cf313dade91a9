"""Pin the NumPy oracle to the reference: golden vectors from the unmodified
GO-MELT sources (run by tests/golden/make_golden.py) must be reproduced."""

import copy
import json

import numpy as np
import pytest

import gomelt_oracle as O
import stateio
from conftest import golden

RT = 1e-9


def close(a, b, rtol=RT, atol=1e-9):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    assert a.shape == b.shape, (a.shape, b.shape)
    np.testing.assert_allclose(a, b, rtol=rtol, atol=atol)


def tup(g, key):
    return tuple(int(np.asarray(x)) for x in stateio.unflatten(g, key))


def props_of(g):
    return stateio.unflatten(g, "properties")


def shapes_and_interp(L):
    shapes = [O.computeCoarseFineShapeFunctions(L[1], L[2]), O.computeCoarseFineShapeFunctions(L[1], L[3]),
              O.computeCoarseFineShapeFunctions(L[2], L[3])]
    interp = [O.interpolatePointsMatrix(L[1], L[2]["node_coords"]),
              O.interpolatePointsMatrix(L[2], L[3]["node_coords"])]
    return shapes, interp


def compare_levels(Lo, Lr, keys=("T0", "Tprime0", "S1", "S2")):
    for lev in range(4):
        for k in keys:
            if k in Lr[lev]:
                close(Lo[lev][k], Lr[lev][k], atol=1e-8)


def test_setup_levels(case):
    g = golden(case)
    cfg = json.loads(str(g["cfg_json"]))
    P = O.SetupProperties(cfg["properties"])
    Pr = props_of(g)
    for k in ("h_conv", "CM_coeff", "CT_coeff", "CP_coeff", "k_powder", "rho", "T_amb", "laser_eta"):
        close(P[k], Pr[k], rtol=1e-14)
    L = O.SetupLevels(cfg, P)
    Lr = stateio.unflatten(g, "u.move.in.Levels")  # set-up geometry before any move
    for lev in range(4):
        for k in ("nodes", "elements", "h", "ne", "nn"):
            if k in Lr[lev]:
                close(np.asarray(L[lev][k], dtype=float), np.asarray(Lr[lev][k], dtype=float), rtol=1e-14)
        for k in ("connect", "BC", "orig_overlap_nodes", "orig_overlap_coors", "orig_overlap_nodes_L2",
                  "init_node_coors", "node_coords"):
            if k in Lr[lev]:
                for a, b in zip(L[lev][k], Lr[lev][k]):
                    close(a, b, rtol=1e-14, atol=1e-14)
    close(L[0]["idx"], Lr[0]["idx"])
    close(L[0]["idx_L2"], Lr[0]["idx_L2"])
    for lev in (2, 3):
        for ax in ("ix", "iy", "iz"):
            close(L[lev]["bounds"][ax], Lr[lev]["bounds"][ax], rtol=1e-14)


def test_props(case):
    g = golden(case)
    P = props_of(g)
    out = O.computeStateProperties(g["u.props.T"], g["u.props.S1"], P, int(g["u.props.substrate"]))
    for k, o in zip(("S1", "S2", "k", "rhocp"), out):
        close(o, g[f"u.props.out.{k}"], rtol=1e-14, atol=0)


def test_fine_source_and_surface(case):
    g = golden(case)
    P = props_of(g)
    L = stateio.unflatten(g, "u.state")
    ne_nn = tuple(int(x) for x in g["u.ne_nn"])
    tmp = tuple(int(x) for x in g["u.tmp_ne_nn"])
    v = g["u.move.in.v"]
    Pw = float(json.loads(str(g["cfg_json"]))["properties"]["laser_power"])
    close(O.computeSourcesL3(L[3], v, ne_nn, P, Pw), g["u.src3.out"], atol=1e-12)
    close(O.computeConvRadBC(L[3], L[3]["T0"], ne_nn[1], ne_nn[4], P, 0), g["u.conv3.out"], atol=1e-15)
    close(O.computeConvRadBC(L[1], L[1]["T0"], tmp[0], ne_nn[2], P, 0), g["u.conv1.out"], atol=1e-15)


def test_level_solves(case):
    g = golden(case)
    L = stateio.unflatten(g, "u.state")
    ne_nn = tuple(int(x) for x in g["u.ne_nn"])
    tmp = tuple(int(x) for x in g["u.tmp_ne_nn"])
    for lev, nn, ne in ((3, ne_nn[4], ne_nn[1]), (1, ne_nn[2], tmp[0])):
        pre = f"u.solve{lev}."
        out = O.solveMatrixFreeFE(L[lev], nn, ne, g[pre + "k"], g[pre + "rhocp"], float(g[pre + "dt"]),
                                  L[lev]["T0"], g[pre + "F"], g[pre + "Corr"])
        ref = g[pre + "out"]
        ok = np.isfinite(ref)
        assert ok.sum() > 0
        np.testing.assert_array_equal(np.isfinite(out), ok)
        close(out[ok], ref[ok])


def test_interpolation(case):
    g = golden(case)
    L = stateio.unflatten(g, "u.state")
    n = g["u.interp.pts_len"]
    pts = np.split(g["u.interp.pts"], np.cumsum(n)[:2])
    Nc, node = O.interpolatePointsMatrix(L[2], pts)
    close(Nc, g["u.interp.Nc"], rtol=1e-12, atol=1e-14)
    np.testing.assert_array_equal(node, g["u.interp.node"])
    close(O.interpolatePoints(L[2], L[2]["T0"], pts), g["u.interp.out"])


def test_restriction_tprime(case):
    g = golden(case)
    L = stateio.unflatten(g, "u.state")
    C2F = O.interpolatePointsMatrix(L[2], L[3]["node_coords"])
    Tp, Tc = O.getNewTprime(L[3], L[3]["T0"], L[2]["T0"], L[2], C2F)
    close(Tp, g["u.tprime.Tp"], atol=1e-9)
    close(Tc, g["u.tprime.Tc"])


def test_coarse_coupling_terms(case):
    g = golden(case)
    P = props_of(g)
    L = stateio.unflatten(g, "u.state")
    ne_nn = tuple(int(x) for x in g["u.ne_nn"])
    sub = tuple(int(x) for x in g["u.substrate"])
    shapes, _ = shapes_and_interp(L)
    for i in range(3):
        close(shapes[i][0], g[f"u.move.out.Shapes#{i}#0"], atol=1e-13)
        for d in range(3):
            close(shapes[i][1][d], g[f"u.move.out.Shapes#{i}#1#{d}"], atol=1e-9)
        np.testing.assert_array_equal(shapes[i][2].reshape(-1), g[f"u.move.out.Shapes#{i}.bcoo"][:, 0])
    nn1, nn2 = int(L[1]["nn"]), int(L[2]["nn"])
    close(O.computeLevelSource(L, ne_nn, g["u.lsrc.lp"], shapes[1], P, g["u.lsrc.lP"], nn1), g["u.lsrc.out1"],
          atol=1e-12)
    close(O.computeLevelSource(L, ne_nn, g["u.lsrc.lp"], shapes[2], P, g["u.lsrc.lP"], nn2), g["u.lsrc.out2"],
          atol=1e-12)
    _, _, k3, rc3 = O.computeStateProperties(L[3]["T0"], L[3]["S1"], P, sub[3])
    _, _, k2, rc2 = O.computeStateProperties(L[2]["T0"], L[2]["S1"], P, sub[2])
    close(O.computeL1TprimeTerms_Part1(L, ne_nn, k3, shapes, k2), g["u.tp1.L1"], atol=1e-12)
    close(O.computeL2TprimeTerms_Part1(L, ne_nn, L[3]["Tprime0"], k3, shapes), g["u.tp1.L2"], atol=1e-12)
    close(O.computeL1TprimeTerms_Part2(L, ne_nn, g["u.tp2.Tp3n"], g["u.tp2.Tp2n"], rc3, rc2, 2e-5, shapes,
                                       np.zeros(nn1)), g["u.tp2.L1"], atol=1e-12)
    close(O.computeL2TprimeTerms_Part2(L, ne_nn, g["u.tp2.Tp3n"], L[3]["Tprime0"], rc3, 2e-5, shapes,
                                       np.zeros(nn2)), g["u.tp2.L2"], atol=1e-12)


def _move_check(g, pre, has_shapes=True):
    Lin = stateio.unflatten(g, pre + ".in.Levels")
    v = g[pre + ".in.v"]
    vstart = g[pre + ".in.vstart"]
    if pre + ".in.L1L2Eratio@list" in g:
        r12 = [int(x) for x in stateio.unflatten(g, pre + ".in.L1L2Eratio")]
        r23 = [int(x) for x in stateio.unflatten(g, pre + ".in.L2L3Eratio")]
        height = float(g[pre + ".in.height"])
        mv = stateio.unflatten(g, pre + ".in.move_v")
    else:  # unit case
        P = props_of(g)
        r12 = [int(np.round(float(Lin[1]["h"][i]) / float(Lin[2]["h"][i]))) for i in range(2)] + [
            int(np.round(float(P["layer_height"]) / float(Lin[2]["h"][2])))]
        r23 = [int(np.round(float(Lin[2]["h"][i]) / float(Lin[3]["h"][i]))) for i in range(3)]
        height = float(P["layer_height"])
        mv = [0, 0, 0]
    Lo, shapes, interp, mvo = O.moveEverything(v, vstart, copy.deepcopy(Lin), mv, [None, None], r12, r23, height)
    Lr = stateio.unflatten(g, pre + ".out.Levels")
    compare_levels(Lo, Lr)
    for lev in (2, 3):
        for k in ("node_coords", "overlapNodes", "overlapCoords"):
            for a, b in zip(Lo[lev][k], Lr[lev][k]):
                close(a, b, rtol=1e-14, atol=1e-14)
    for k in ("idx", "idx_L2"):
        np.testing.assert_array_equal(Lo[0][k], Lr[0][k])
    np.testing.assert_array_equal(np.asarray(mvo), np.asarray(stateio.unflatten(g, pre + ".out.move_v")))
    Ir = stateio.unflatten(g, pre + ".out.LInterp")
    for i in range(2):
        close(interp[i][0], Ir[i][0], rtol=1e-12, atol=1e-14)
        np.testing.assert_array_equal(interp[i][1], Ir[i][1])
    if has_shapes:
        for i in range(3):
            close(shapes[i][0], g[f"{pre}.out.Shapes#{i}#0"], atol=1e-13)


def test_move_unit(case):
    _move_check(golden(case), "u.move")


@pytest.mark.parametrize("n", [0, 1])
def test_move_driver(case, n):
    g = golden(case)
    if f"move{n}.in.v" not in g:
        pytest.skip("no such call")
    _move_check(g, f"move{n}")


@pytest.mark.parametrize("n", [0, 1])
def test_subcycle(case, n):
    g = golden(case)
    pre = f"sub{n}"
    if pre + ".in.laser_position" not in g:
        pytest.skip("no such call")
    P = props_of(g)
    L = stateio.unflatten(g, pre + ".in.Levels")
    shapes, interp = shapes_and_interp(L)
    args = [tup(g, pre + f".in.{k}") for k in ("ne_nn", "substrate", "tmp_ne_nn")]
    sc = stateio.unflatten(g, pre + ".in.subcycle")
    sc = (int(sc[0]), int(sc[1]), int(sc[2]), float(sc[3]), float(sc[4]), float(sc[5]))
    Lo, L2all, L3all, L3pall, macc, acc = O.subcycleGOMELT(
        L, args[0], shapes, args[1], interp, args[2], g[pre + ".in.laser_position"], P, g[pre + ".in.laserP"], sc,
        g[pre + ".in.max_accum_L3"], g[pre + ".in.accum_L3"])
    Lr = stateio.unflatten(g, pre + ".out.Levels")
    compare_levels(Lo, Lr)
    close(L2all, g[pre + ".out.L2all"], atol=1e-8)
    close(L3all, g[pre + ".out.L3all"], atol=1e-8)
    close(L3pall, g[pre + ".out.L3pall"], atol=1e-8)
    close(macc, g[pre + ".out.max_accum"], atol=1e-15)
    close(acc, g[pre + ".out.accum"], atol=1e-15)


@pytest.mark.parametrize("n", [0, 1])
def test_single_step(case, n):
    g = golden(case)
    pre = f"step{n}"
    if pre + ".in.v" not in g:
        pytest.skip("no such call")
    P = props_of(g)
    L = stateio.unflatten(g, pre + ".in.Levels")
    shapes, interp = shapes_and_interp(L)
    ne_nn, tmp, sub = (tup(g, pre + f".in.{k}") for k in ("ne_nn", "tmp_ne_nn", "substrate"))
    Lo, reset = O.stepGOMELT(L, ne_nn, tmp, shapes, interp, g[pre + ".in.v"], P, float(g[pre + ".in.dt"]),
                             float(g[pre + ".in.laserP"]), sub)
    compare_levels(Lo, stateio.unflatten(g, pre + ".out.Levels"))
    np.testing.assert_array_equal(reset, g[pre + ".out.resetmask"])


def test_dwell(case):
    g = golden(case)
    pre = "dwell0"
    if pre + ".in.dt" not in g:
        pytest.skip("no dwell step")
    P = props_of(g)
    L = stateio.unflatten(g, pre + ".in.Levels")
    tmp, ne_nn, sub = (tup(g, pre + f".in.{k}") for k in ("tmp_ne_nn", "ne_nn", "substrate"))
    Lo = O.stepGOMELTDwellTime(L, tmp, ne_nn, P, float(g[pre + ".in.dt"]), sub)
    close(Lo[1]["T0"], stateio.unflatten(g, pre + ".out.Levels")[1]["T0"])
