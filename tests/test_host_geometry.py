"""The product's host-side geometry (set-up, window moves, overlap index sets)
against the reference's golden vectors.  CPU only."""

import json

import numpy as np
import pytest

import stateio
from conftest import golden


def geometry(g):
    from levels import Geometry, setup_properties

    cfg = json.loads(str(g["cfg_json"]))
    P = setup_properties(cfg["properties"])
    return Geometry(cfg, P), P


def test_setup(case):
    g = golden(case)
    geo, P = geometry(g)
    Pr = stateio.unflatten(g, "properties")
    for k in ("h_conv", "CM_coeff", "CT_coeff", "CP_coeff", "k_powder", "rho", "laser_eta", "T_amb"):
        assert np.isclose(P[k], float(Pr[k]), rtol=1e-15)
    Lr = stateio.unflatten(g, "u.move.in.Levels")
    for lev in (1, 2, 3):
        L = geo.L[lev]
        assert L.nodes == [int(x) for x in Lr[lev]["nodes"]]
        for d in range(3):
            np.testing.assert_array_equal(L.coords[d], Lr[lev]["node_coords"][d])
            assert L.h[d] == float(Lr[lev]["h"][d])
    for lev in (2, 3):
        for d in range(3):
            np.testing.assert_array_equal(geo.L[lev].orig_overlap_nodes[d], Lr[lev]["orig_overlap_nodes"][d])
            np.testing.assert_array_equal(geo.L[lev].orig_overlap_coors[d], Lr[lev]["orig_overlap_coors"][d])
            lim = Lr[lev]["bounds"][("ix", "iy", "iz")[d]]
            assert list(geo.L[lev].limits[d]) == [float(x) for x in lim]
    assert geo.L0_nodes == [int(x) for x in Lr[0]["nodes"]]
    for d in range(3):
        np.testing.assert_array_equal(geo.L0_orig_overlap[d], Lr[0]["orig_overlap_nodes"][d])
        np.testing.assert_array_equal(geo.L0_orig_overlap_L2[d], Lr[0]["orig_overlap_nodes_L2"][d])
    assert geo.layer_idx_delta == int(Lr[0]["layer_idx_delta"])
    assert geo.ne_nn() == tuple(int(x) for x in g["u.ne_nn"])


@pytest.mark.parametrize("pre", ["u.move", "move0", "move1"])
def test_move(case, pre):
    g = golden(case)
    if pre + ".in.v" not in g:
        pytest.skip("no such call")
    geo, P = geometry(g)
    Lin = stateio.unflatten(g, pre + ".in.Levels")
    for lev in (1, 2, 3):
        geo.L[lev].coords = [np.asarray(c, dtype=float) for c in Lin[lev]["node_coords"]]
    new3, new2, mv = geo.move(g[pre + ".in.v"], g[pre + ".in.vstart"])
    Lr = stateio.unflatten(g, pre + ".out.Levels")
    for d in range(3):
        np.testing.assert_array_equal(new3[d], Lr[3]["node_coords"][d])
        np.testing.assert_array_equal(new2[d], Lr[2]["node_coords"][d])
        for lev in (2, 3):
            np.testing.assert_array_equal(geo.L[lev].overlap_nodes[d], Lr[lev]["overlapNodes"][d])
            np.testing.assert_allclose(geo.L[lev].overlap_coords[d], Lr[lev]["overlapCoords"][d], rtol=0,
                                       atol=1e-15)
        np.testing.assert_array_equal(geo.L0_overlap[d], Lr[0]["overlapNodes"][d])
        np.testing.assert_array_equal(geo.L0_overlap_L2[d], Lr[0]["overlapNodes_L2"][d])
    np.testing.assert_array_equal(mv, np.asarray(stateio.unflatten(g, pre + ".out.move_v")))


def test_static_counts(case):
    g = golden(case)
    geo, P = geometry(g)
    pre = "sub0" if "sub0.in.laser_position" in g else "step0"
    Lin = stateio.unflatten(g, pre + ".in.Levels")
    for lev in (1, 2, 3):
        geo.L[lev].coords = [np.asarray(c, dtype=float) for c in Lin[lev]["node_coords"]]
    geo.L0_coords = [np.asarray(c, dtype=float) for c in Lin[0]["node_coords"]]
    v = g[pre + ".in.laser_position"][0] if pre == "sub0" else g[pre + ".in.v"]
    assert geo.tmp_ne_nn(v) == tuple(int(np.asarray(x)) for x in stateio.unflatten(g, pre + ".in.tmp_ne_nn"))
    assert geo.substrate() == tuple(int(np.asarray(x)) for x in stateio.unflatten(g, pre + ".in.substrate"))
