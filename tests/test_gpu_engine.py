"""GPU engine vs the reference's golden vectors: moveEverything and
subcycleGOMELT on the states recorded from reference runs (FP64 and FP32)."""

import json

import numpy as np
import pytest
import torch

import stateio
from conftest import golden

pytestmark = pytest.mark.gpu


def tup(g, key):
    return tuple(int(np.asarray(x)) for x in stateio.unflatten(g, key))


def make_engine(g, Lin, dtype, N2=1, N3=1):
    from engine import Engine

    cfg = json.loads(str(g["cfg_json"]))
    P = stateio.unflatten(g, "properties")
    eng = Engine(cfg, P, N2, N3, dtype=dtype)
    eng.load_levels(Lin)
    return eng


def relT(a, b):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1.0))


def absdiff(a, b, scale):
    return float(np.max(np.abs(np.asarray(a, dtype=float) - np.asarray(b, dtype=float))) / scale)


TOL = [(torch.float64, 1e-10), (torch.float32, 1e-4)]


@pytest.mark.parametrize("dtype,tol", TOL)
@pytest.mark.parametrize("n", [0, 1])
def test_subcycle_golden(case, n, dtype, tol):
    g = golden(case)
    pre = f"sub{n}"
    if pre + ".in.laser_position" not in g:
        pytest.skip("no such call")
    Lin = stateio.unflatten(g, pre + ".in.Levels")
    sc = stateio.unflatten(g, pre + ".in.subcycle")
    eng = make_engine(g, Lin, dtype, int(sc[0]), int(sc[1]))
    eng.tmp = tup(g, pre + ".in.tmp_ne_nn")
    eng.substrate = tup(g, pre + ".in.substrate")
    eng.macc3 = torch.as_tensor(g[pre + ".in.max_accum_L3"], dtype=dtype, device="cuda").contiguous()
    eng.acc3 = torch.as_tensor(g[pre + ".in.accum_L3"], dtype=dtype, device="cuda").contiguous()
    hist = eng.subcycle(g[pre + ".in.laser_position"], history=True)
    torch.cuda.synchronize()
    out = eng.fields_numpy()
    Lr = stateio.unflatten(g, pre + ".out.Levels")
    Tscale = max(float(np.max(Lr[lev]["T0"])) for lev in (1, 2, 3))
    for lev in (1, 2, 3):
        assert relT(out[lev]["T0"], Lr[lev]["T0"]) < tol, lev
        np.testing.assert_array_equal(out[lev]["S1"], np.asarray(Lr[lev]["S1"]) > 0.499)
    for lev in (2, 3):
        assert absdiff(out[lev]["Tprime0"], Lr[lev]["Tprime0"], Tscale) < tol, lev
    np.testing.assert_array_equal(out[3]["S2"], np.asarray(Lr[3]["S2"]).astype(bool))
    np.testing.assert_array_equal(out[0]["S1"], np.asarray(Lr[0]["S1"]) > 0.499)
    assert relT(hist[0].cpu().numpy(), g[pre + ".out.L2all"]) < tol
    assert relT(hist[1].cpu().numpy(), g[pre + ".out.L3all"]) < tol
    assert absdiff(hist[2].cpu().numpy(), g[pre + ".out.L3pall"], Tscale) < tol
    np.testing.assert_allclose(eng.acc3.double().cpu().numpy(), g[pre + ".out.accum"], rtol=1e-5, atol=1e-10)
    np.testing.assert_allclose(eng.macc3.double().cpu().numpy(), g[pre + ".out.max_accum"], rtol=1e-5,
                               atol=1e-10)


def _move(g, pre, dtype, tol):
    Lin = stateio.unflatten(g, pre + ".in.Levels")
    eng = make_engine(g, Lin, dtype)
    mv = eng.move(g[pre + ".in.v"], g[pre + ".in.vstart"])
    torch.cuda.synchronize()
    Lr = stateio.unflatten(g, pre + ".out.Levels")
    out = eng.fields_numpy()
    Tscale = max(float(np.max(Lr[lev]["T0"])) for lev in (1, 2, 3))
    for lev in (2, 3):
        assert relT(out[lev]["T0"], Lr[lev]["T0"]) < tol, lev
        assert absdiff(out[lev]["Tprime0"], Lr[lev]["Tprime0"], Tscale) < tol, lev
        np.testing.assert_array_equal(out[lev]["S1"], np.asarray(Lr[lev]["S1"]) > 0.499)
        for d in range(3):
            np.testing.assert_allclose(eng.geo.L[lev].coords[d], Lr[lev]["node_coords"][d], rtol=0, atol=1e-14)
            np.testing.assert_array_equal(eng.geo.L[lev].overlap_nodes[d], Lr[lev]["overlapNodes"][d])
    np.testing.assert_array_equal(out[3]["S2"], np.asarray(Lr[3]["S2"]).astype(bool))
    for d in range(3):
        np.testing.assert_array_equal(eng.geo.L0_overlap[d], Lr[0]["overlapNodes"][d])
        np.testing.assert_array_equal(eng.geo.L0_overlap_L2[d], Lr[0]["overlapNodes_L2"][d])
    if pre + ".out.move_v@list" in g:
        np.testing.assert_array_equal(np.asarray(mv), np.asarray(stateio.unflatten(g, pre + ".out.move_v")))


@pytest.mark.parametrize("dtype,tol", TOL)
@pytest.mark.parametrize("n", [0, 1])
def test_move_golden(case, n, dtype, tol):
    g = golden(case)
    pre = f"move{n}"
    if pre + ".in.v" not in g:
        pytest.skip("no such call")
    _move(g, pre, dtype, tol)


@pytest.mark.parametrize("dtype,tol", TOL)
@pytest.mark.parametrize("n", [0, 1])
def test_step_golden(case, n, dtype, tol):
    g = golden(case)
    pre = f"step{n}"
    if pre + ".in.v" not in g:
        pytest.skip("no such call")
    Lin = stateio.unflatten(g, pre + ".in.Levels")
    eng = make_engine(g, Lin, dtype)
    eng.tmp = tup(g, pre + ".in.tmp_ne_nn")
    eng.substrate = tup(g, pre + ".in.substrate")
    v = np.array(g[pre + ".in.v"], dtype=float)
    v[5] = float(g[pre + ".in.dt"])
    v[6] = float(g[pre + ".in.laserP"])
    reset = eng.step(v)
    torch.cuda.synchronize()
    Lr = stateio.unflatten(g, pre + ".out.Levels")
    out = eng.fields_numpy()
    Tscale = max(float(np.max(Lr[lev]["T0"])) for lev in (1, 2, 3))
    for lev in (1, 2, 3):
        assert relT(out[lev]["T0"], Lr[lev]["T0"]) < tol, lev
        np.testing.assert_array_equal(out[lev]["S1"], np.asarray(Lr[lev]["S1"]) > 0.499)
    for lev in (2, 3):
        assert absdiff(out[lev]["Tprime0"], Lr[lev]["Tprime0"], Tscale) < tol, lev
    np.testing.assert_array_equal(out[3]["S2"], np.asarray(Lr[3]["S2"]).astype(bool))
    np.testing.assert_array_equal(out[0]["S1"], np.asarray(Lr[0]["S1"]) > 0.499)
    np.testing.assert_array_equal(reset.cpu().numpy(), g[pre + ".out.resetmask"])


@pytest.mark.parametrize("dtype,tol", TOL)
def test_dwell_golden(case, dtype, tol):
    g = golden(case)
    pre = "dwell0"
    if pre + ".in.dt" not in g:
        pytest.skip("no dwell step")
    Lin = stateio.unflatten(g, pre + ".in.Levels")
    eng = make_engine(g, Lin, dtype)
    eng.tmp = tup(g, pre + ".in.tmp_ne_nn")
    eng.substrate = tup(g, pre + ".in.substrate")
    eng.dwell(float(g[pre + ".in.dt"]))
    torch.cuda.synchronize()
    Lr = stateio.unflatten(g, pre + ".out.Levels")
    assert relT(eng.T[1].double().cpu().numpy(), Lr[1]["T0"]) < tol
