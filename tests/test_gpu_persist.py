"""The persistent Level-3 kernel (gm_level3_persist): N3 fine steps in one
launch against N3 launches of the one-step separable kernel, bit for bit;
the subcycle with and without it; its device status word.

The one-step kernel is itself checked against the oracle
(tests/test_gpu_separable.py), so equality here carries that parity over.
"""

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

CONST_MAT = {"thermal_conductivity_powder": 22.0, "thermal_conductivity_bulk_a0": 22.0,
             "thermal_conductivity_bulk_a1": 0.0, "thermal_conductivity_fluid_a0": 22.0,
             "heat_capacity_solid_a0": 700.0, "heat_capacity_solid_a1": 0.0, "heat_capacity_mushy": 700.0,
             "heat_capacity_fluid": 700.0, "density": 4.4e-06, "laser_radius": 0.05, "laser_depth": 0.05,
             "laser_power": 200.0, "laser_absorptivity": 0.35, "T_amb": 300.0, "T_solidus": 1878.0,
             "T_liquidus": 1900.0, "h_conv": 1e-5, "emissivity": 0.3, "evaporation_coefficient": 0.0,
             "layer_height": 0.05}
EVAP_MAT = dict(CONST_MAT, evaporation_coefficient=0.82)

# (Level-3 elements, bounds) of the windows: the single-track and part-scale
# windows, and an odd one (x-tiles of uneven width, a partial last y-tile)
WINDOWS = {
    "single_track": ([80, 80, 20], {"x": [0.3, 0.7], "y": [2.3, 2.7], "z": [-0.1, 0.0]}),
    "part_scale": ([160, 160, 40], {"x": [1.6, 2.4], "y": [1.6, 2.4], "z": [-0.2, 0.0]}),
    "odd": ([93, 37, 9], {"x": [0.3, 0.765], "y": [2.3, 2.485], "z": [-0.045, 0.0]}),
}


def _cfg(window, mat=CONST_MAT):
    e3, b3 = WINDOWS[window]
    return {
        "Level1": {"elements": [40, 40, 10], "bounds": {"x": [0.0, 4.0], "y": [0.0, 4.0], "z": [-1.0, 0.0]},
                   "conditions": {"x": [300, 300], "y": [300, 300], "z": [300, 300]}},
        "Level2": {"elements": [100, 100, 15], "bounds": {"x": [0.0, 2.0] if window != "part_scale" else [1.0, 3.0],
                                                          "y": [1.5, 3.5] if window != "part_scale" else [1.0, 3.0],
                                                          "z": [-0.3, 0.0]}},
        "Level3": {"elements": e3, "bounds": b3},
        "properties": dict(mat, laser_center=[sum(b3["x"]) / 2, sum(b3["y"]) / 2, 0.0, 0, 0, 0, 0]),
    }


def _case(window, dtype, N3, mat=CONST_MAT, seed=3):
    """An engine on the window with a hot random field, ring arrays, the step
    rows and their laser factor table."""
    import _native as N
    from engine import Engine
    from levels import setup_properties

    cfg = _cfg(window, mat)
    P = setup_properties(cfg["properties"])
    eng = Engine(cfg, P, 1, N3, dtype=dtype)
    L3 = eng.geo.L[3]
    nn = L3.nn
    rng = np.random.default_rng(seed)
    x, y, z = (np.asarray(c) for c in L3.coords)
    X = np.tile(x, len(y) * len(z))
    Y = np.repeat(np.tile(y, len(z)), len(x))
    Z = np.repeat(z, len(x) * len(y))
    cx, cy = np.mean(x), np.mean(y)
    T = 300 + 2600 * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / 0.004 + Z * 30) + 3 * rng.standard_normal(nn)
    dev = "cuda"
    eng.T[3].copy_(torch.as_tensor(T, dtype=dtype))
    ph = (rng.random(nn) > 0.5).astype(np.uint8) | ((T >= 1900).astype(np.uint8) << 1)
    eng.ph[3].copy_(torch.as_tensor(ph))
    ringA = torch.as_tensor(300 + 600 * rng.random(nn), dtype=dtype, device=dev)
    ringB = torch.as_tensor(300 + 600 * rng.random(nn), dtype=dtype, device=dev)
    dt3 = 1.575e-6
    rows = np.zeros((N3, 7))
    rows[:, 0] = cx - 0.01 + 1e3 * dt3 * np.arange(N3)
    rows[:, 1] = cy + 0.003
    rows[:, 3] = rows[:, 4] = 1
    rows[:, 5] = dt3 * (1 + 0.01 * np.arange(N3))
    rows[:, 6] = 200.0
    rows_d = torch.as_tensor(rows, device=dev)
    Lw = int(sum(L3.nodes))
    tab = torch.empty(N3 * Lw, dtype=dtype, device=dev)
    N.call("gm_fine_source_tables", kern_code(dtype), (C.c_int * 3)(*L3.nodes), (C.c_double * 3)(*L3.origin()),
           (C.c_double * 3)(*L3.spacing()), rows_d.data_ptr(), N3, C.byref(eng.ps), tab.data_ptr(), None)
    acc = torch.as_tensor(rng.uniform(0, 1e-4, nn), dtype=dtype, device=dev)
    macc = torch.as_tensor(rng.uniform(0, 1e-4, nn), dtype=dtype, device=dev)
    return eng, ringA, ringB, rows_d, tab, acc, macc


def kern_code(dtype):
    import _native as N

    return N.GM_F32 if dtype == torch.float32 else N.GM_F64


def per_step(eng, ringA, ringB, rows_d, tab, acc, macc, N3, shape):
    """N3 launches of the one-step separable kernel (bc_mode 3, factor table)."""
    import kern

    L3 = eng.geo.L[3]
    Lw = int(sum(L3.nodes))
    Ta, pa = eng.T[3].clone(), eng.ph[3].clone()
    Tb, pb = torch.empty_like(Ta), torch.empty_like(pa)
    kw_acc = dict(accum=acc, max_accum=macc) if acc is not None else {}
    for s in range(N3):
        kw = eng.level_kwargs(3, Ta, Tb, rows_d[s, 5:6], pa, pb, laser=rows_d[s], ring=(ringA, ringB),
                              alpha=(s + 1) / N3)
        kw.update(kw_acc)
        kw["src_tab"] = tab[s * Lw:(s + 1) * Lw]
        kern.level_step_shape(eng.ps, kernel=1, rows=shape[0], tile_y=shape[1], zchunk=shape[2], **kw)
        Ta, Tb, pa, pb = Tb, Ta, pb, pa
    torch.cuda.synchronize()
    return Ta, pa


def persist(eng, ringA, ringB, rows_d, tab, acc, macc, N3, base=0, flags=None, hold=0, T_in=None):
    import _native as N

    L3 = eng.geo.L[3]
    nn = L3.nn
    nf = int(N.lib().gm_level3_persist_flags((C.c_int * 3)(*L3.nodes)))
    assert nf > 0
    if flags is None:
        flags = torch.zeros(nf, dtype=torch.int32, device="cuda")
    xb = [torch.full((nn,), float("nan"), dtype=eng.dtype, device="cuda") for _ in range(2)]
    Tout = torch.full((nn,), -1.0, dtype=eng.dtype, device="cuda")
    pout = torch.full((nn,), 255, dtype=torch.uint8, device="cuda")
    Tin = eng.T[3] if T_in is None else T_in
    a = N.gm_persist_args()
    a.dtype = kern_code(eng.dtype)
    for d in range(3):
        a.nodes[d] = L3.nodes[d]
        a.h[d] = L3.spacing()[d]
    a.nsteps, a.nsub = N3, N3
    a.T_in, a.T_out = Tin.data_ptr(), Tout.data_ptr()
    a.ph_in, a.ph_out = eng.ph[3].data_ptr(), pout.data_ptr()
    a.substrate = eng.substrate[3]
    a.ring_new, a.ring_old = ringA.data_ptr(), ringB.data_ptr()
    a.src_tab, a.rows = tab.data_ptr(), rows_d.data_ptr()
    if acc is not None:
        a.accum, a.max_accum = acc.data_ptr(), macc.data_ptr()
    a.xbuf[0], a.xbuf[1] = xb[0].data_ptr(), xb[1].data_ptr()
    a.flags, a.flags_cap, a.base = flags.data_ptr(), nf, base
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    a.status = status.data_ptr()
    a.hold = hold
    rc = N.lib().gm_level3_persist(C.byref(a), C.byref(eng.ps), None)
    torch.cuda.synchronize()
    return rc, Tout, pout, int(status.item()), flags


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("accum", [False, True])
@pytest.mark.parametrize("window,N3", [("single_track", 10), ("part_scale", 10), ("odd", 7), ("odd", 1)])
def test_persist_equals_per_step(window, N3, dtype, accum):
    import _native as N

    eng, rA, rB, rows_d, tab, acc, macc = _case(window, dtype, N3)
    if eng.persist_shape() is None:
        pytest.skip("no persistent shape for this window and dtype on this device")
    acc2, macc2 = (acc.clone(), macc.clone()) if accum else (None, None)
    Tref, pref = per_step(eng, rA, rB, rows_d, tab, acc2, macc2, N3, (2, 4, 6))
    acc1, macc1 = (acc.clone(), macc.clone()) if accum else (None, None)
    rc, Tout, pout, status, flags = persist(eng, rA, rB, rows_d, tab, acc1, macc1, N3)
    assert rc == N.GM_OK and status == 0
    assert float(Tref.max()) > 1900.0  # melting nodes exercise the phase and melt-time paths
    torch.testing.assert_close(Tout, Tref, rtol=0, atol=0)
    assert torch.equal(pout, pref)
    if accum:
        torch.testing.assert_close(acc1, acc2, rtol=0, atol=0)
        torch.testing.assert_close(macc1, macc2, rtol=0, atol=0)
    assert torch.all(flags == N3)  # every counter ends at base + nsteps


def test_persist_evaporation_and_chained_launches():
    """Evaporation in the surface flux; two launches in a row with base = N3."""
    import _native as N

    N3 = 5
    eng, rA, rB, rows_d, tab, acc, macc = _case("odd", torch.float32, N3, mat=EVAP_MAT, seed=9)
    Tref, _ = per_step(eng, rA, rB, rows_d, tab, None, None, N3, (1, 2, 3))
    rc, T1, p1, st, flags = persist(eng, rA, rB, rows_d, tab, None, None, N3)
    assert rc == N.GM_OK and st == 0
    torch.testing.assert_close(T1, Tref, rtol=0, atol=0)
    rc, T2, _, st, flags = persist(eng, rA, rB, rows_d, tab, None, None, N3, base=N3, flags=flags, T_in=T1)
    assert rc == N.GM_OK and st == 0
    eng.T[3].copy_(T1)
    eng.ph[3].copy_(p1)
    Tref2, _ = per_step(eng, rA, rB, rows_d, tab, None, None, N3, (1, 2, 3))
    torch.testing.assert_close(T2, Tref2, rtol=0, atol=0)
    assert torch.all(flags == 2 * N3)


def test_persist_wait_timeout_sets_status():
    """A tile that never publishes its counters: its neighbours' waits run out
    after about a second, the launch ends with GM_PERSIST_TIMEOUT in the
    status word, and the context stays usable for the next launch."""
    import _native as N

    N3 = 4
    eng, rA, rB, rows_d, tab, acc, macc = _case("single_track", torch.float32, N3)
    shape = eng.persist_shape()
    assert shape is not None and shape[0] > 4
    rc, _, _, status, _ = persist(eng, rA, rB, rows_d, tab, None, None, N3, hold=shape[0] // 2 + 1)
    assert rc == N.GM_OK
    assert status & N.GM_PERSIST_TIMEOUT
    # fresh counters: the next launch completes normally
    Tref, _ = per_step(eng, rA, rB, rows_d, tab, None, None, N3, (2, 4, 6))
    rc, Tout, _, status, _ = persist(eng, rA, rB, rows_d, tab, None, None, N3)
    assert rc == N.GM_OK and status == 0
    torch.testing.assert_close(Tout, Tref, rtol=0, atol=0)


def test_persist_flags_out_of_range_field():
    """An infinite temperature in the window is reported in the status word."""
    import _native as N

    N3 = 2
    eng, rA, rB, rows_d, tab, acc, macc = _case("odd", torch.float32, N3)
    T = eng.T[3].clone()
    T[T.numel() // 2] = float("inf")
    rc, _, _, status, _ = persist(eng, rA, rB, rows_d, tab, None, None, N3, T_in=T)
    assert rc == N.GM_OK
    assert status & N.GM_PERSIST_BAD_T


def test_persist_rejects_bad_arguments():
    import _native as N

    eng, rA, rB, rows_d, tab, acc, macc = _case("odd", torch.float32, 2)
    a = N.gm_persist_args()
    assert N.lib().gm_level3_persist(C.byref(a), C.byref(eng.ps), None) == N.GM_ERR_ARG
    assert N.lib().gm_level3_persist(None, C.byref(eng.ps), None) == N.GM_ERR_ARG


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_subcycle_persist_on_off(graph, dtype, mode):
    """Three move + subcycle calls of the single-track workload with the
    N3 Level-3 steps of a Level-2 step as one launch (mode 1: window in shared
    memory, mode 2: one-step body with grid barriers) and with one launch a
    step: identical fields."""
    import copy

    import workloads
    from engine import Engine
    from levels import setup_properties
    from test_gpu_parity_scale import _rows

    cfg = workloads.single_track()
    rows = _rows(cfg)
    P = setup_properties(cfg["properties"])
    vstart = np.asarray(cfg["properties"]["laser_center"], dtype=float)
    out = {}
    for persist_on in (0, mode):
        stream = torch.cuda.Stream()
        with torch.cuda.stream(stream):
            eng = Engine(copy.deepcopy(cfg), P, 10, 10, dtype=dtype, stream=stream)
            eng.use_persist = persist_on
            eng.use_graph = graph
            eng.set_layer(rows[0])
            for c in range(3):
                ch = rows[c * 100:(c + 1) * 100]
                eng.move(ch[0], vstart)
                eng.subcycle(ch)
            stream.synchronize()
        eng.check_status()
        out[persist_on] = eng
    a, b = out[0], out[mode]
    assert mode == 2 or b.persist_shape() is not None
    for lev in (1, 2, 3):
        torch.testing.assert_close(b.T[lev], a.T[lev], rtol=0, atol=0)
        assert torch.equal(b.ph[lev], a.ph[lev])
    for lev in (2, 3):
        torch.testing.assert_close(b.Tp[lev], a.Tp[lev], rtol=0, atol=0)
    torch.testing.assert_close(b.acc3, a.acc3, rtol=0, atol=0)
    torch.testing.assert_close(b.macc3, a.macc3, rtol=0, atol=0)
    assert float(a.T[3].max()) > 2000.0


def steps_launch(eng, ringA, ringB, rows_d, tab, acc, macc, N3, base=0, counter=None):
    """gm_level3_steps: the N3 steps in one launch with grid barriers."""
    import _native as N
    import kern

    L3 = eng.geo.L[3]
    nn = L3.nn
    Tout = torch.full((nn,), -1.0, dtype=eng.dtype, device="cuda")
    pout = torch.full((nn,), 255, dtype=torch.uint8, device="cuda")
    tb = [torch.full((nn,), float("nan"), dtype=eng.dtype, device="cuda") for _ in range(2)]
    kw = eng.level_kwargs(3, eng.T[3], Tout, rows_d[0, 5:6], eng.ph[3], pout, laser=rows_d[0], ring=(ringA, ringB),
                          alpha=1.0 / N3)
    if acc is not None:
        kw.update(accum=acc, max_accum=macc)
    kw["src_tab"] = tab
    a = N.gm_steps_args()
    a.level = kern.level_args(**kw)
    a.nsteps, a.nsub = N3, N3
    a.rows, a.src_tab = rows_d.data_ptr(), tab.data_ptr()
    a.tbuf[0], a.tbuf[1] = tb[0].data_ptr(), tb[1].data_ptr()
    if counter is None:
        counter = torch.zeros(1, dtype=torch.int32, device="cuda")
    a.counter, a.base = counter.data_ptr(), base
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    a.status = status.data_ptr()
    rc = N.lib().gm_level3_steps(C.byref(a), C.byref(eng.ps), None)
    torch.cuda.synchronize()
    return rc, Tout, pout, int(status.item())


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("accum", [False, True])
@pytest.mark.parametrize("window,N3", [("single_track", 10), ("part_scale", 10), ("odd", 7), ("odd", 1)])
def test_grid_steps_equal_per_step(window, N3, dtype, accum):
    """gm_level3_steps runs the one-step kernel's body: the same bits as N3
    launches of the one-step kernel with the same launch shape."""
    import _native as N

    eng, rA, rB, rows_d, tab, acc, macc = _case(window, dtype, N3)
    acc2, macc2 = (acc.clone(), macc.clone()) if accum else (None, None)
    Tref, pref = per_step(eng, rA, rB, rows_d, tab, acc2, macc2, N3, (2, 4, 6))
    acc1, macc1 = (acc.clone(), macc.clone()) if accum else (None, None)
    rc, Tout, pout, status = steps_launch(eng, rA, rB, rows_d, tab, acc1, macc1, N3)
    assert rc == N.GM_OK and status == 0
    assert float(Tref.max()) > 1900.0
    torch.testing.assert_close(Tout, Tref, rtol=0, atol=0)
    assert torch.equal(pout, pref)
    if accum:
        torch.testing.assert_close(acc1, acc2, rtol=0, atol=0)
        torch.testing.assert_close(macc1, macc2, rtol=0, atol=0)

