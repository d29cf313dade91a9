"""Two Level-3 fine steps in one launch (gm_level_step2) against two launches
of the one-step separable kernel, bit for bit: windows of several shapes
(the single-track and part-scale windows, an odd window, shallow ones),
launch shapes, FP32 and FP64, with and without the melt-time update, and
the device status word.  The one-step kernel is itself checked against the
oracle (tests/test_gpu_separable.py), so equality carries that parity over;
the subcycle that takes its Level-3 steps two at a time is compared with the
one that takes them one at a time in tests/test_gpu_persist.py and against
the oracle in tests/test_gpu_parity_scale.py."""


import pytest
import torch

from test_gpu_persist import WINDOWS, _case, per_step

pytestmark = pytest.mark.gpu

WINDOWS.setdefault("shallow", ([37, 23, 2], {"x": [0.3, 0.485], "y": [2.3, 2.415], "z": [-0.01, 0.0]}))
WINDOWS.setdefault("shallow3", ([31, 29, 3], {"x": [0.3, 0.455], "y": [2.3, 2.445], "z": [-0.015, 0.0]}))


def two_step(eng, ringA, ringB, rows_d, tab, acc, macc, N3, shape=None):
    """The N3 steps as N3 // 2 two-step launches (and one one-step launch if
    N3 is odd)."""
    import kern

    L3 = eng.geo.L[3]
    Lw = int(sum(L3.nodes))
    Ta, pa = eng.T[3].clone(), eng.ph[3].clone()
    Tb, pb = torch.full_like(Ta, -1.0), torch.full_like(pa, 255)
    kw_acc = dict(accum=acc, max_accum=macc) if acc is not None else {}
    s = 0
    while s < N3:
        kw = eng.level_kwargs(3, Ta, Tb, rows_d[s, 5:6], pa, pb, laser=rows_d[s], ring=(ringA, ringB),
                              alpha=(s + 1) / N3)
        kw.update(kw_acc)
        kw["src_tab"] = tab[s * Lw:(s + 1) * Lw]
        if s + 1 < N3:
            a2 = (s + 2) / N3
            kern.level_step2(eng.ps, shape=shape, dt2=rows_d[s + 1, 5:6], src_tab2=tab[(s + 1) * Lw:(s + 2) * Lw],
                             bc_alpha2=a2, bc_beta2=1.0 - a2, **kw)
            s += 2
        else:
            kern.level_step(eng.ps, **kw)
            s += 1
        Ta, Tb, pa, pb = Tb, Ta, pb, pa
    torch.cuda.synchronize()
    return Ta, pa


def _same(a, b):
    assert torch.equal(a, b), f"max |diff| {float((a.double() - b.double()).abs().max())}"


ONE_STEP = (4, 4, 6)  # one-step separable shape of the comparison runs


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("accum", [False, True])
@pytest.mark.parametrize("window", ["single_track", "odd", "shallow", "shallow3"])
def test_two_steps_equal_two_launches(window, accum, dtype):
    N3 = 5  # two pairs and a single step
    eng, rA, rB, rows, tab, acc, macc = _case(window, dtype, N3)
    acc2, macc2 = (acc.clone(), macc.clone()) if accum else (None, None)
    T1, p1 = per_step(eng, rA, rB, rows, tab, acc if accum else None, macc if accum else None, N3, ONE_STEP)
    T2, p2 = two_step(eng, rA, rB, rows, tab, acc2, macc2, N3)
    _same(T1, T2)
    _same(p1, p2)
    if accum:
        _same(acc, acc2)
        _same(macc, macc2)


# (rows, warps a CTA, z-chunk): every row count and CTA size, z-chunks of one
# plane, uneven splits and the largest
SHAPES2 = [(1, 2, 1), (1, 8, 7), (2, 4, 4), (2, 2, 13), (4, 4, 6), (4, 1, 30), (2, 8, 38), (4, 2, 3)]


@pytest.mark.parametrize("shape", SHAPES2)
def test_two_steps_launch_shapes(shape):
    N3 = 4
    eng, rA, rB, rows, tab, acc, macc = _case("single_track", torch.float32, N3)
    acc2, macc2 = acc.clone(), macc.clone()
    T1, p1 = per_step(eng, rA, rB, rows, tab, acc, macc, N3, ONE_STEP)
    if shape[2] > 30:
        with pytest.raises(Exception):
            two_step(eng, rA, rB, rows, tab, acc2, macc2, N3, shape=shape)
        return
    T2, p2 = two_step(eng, rA, rB, rows, tab, acc2, macc2, N3, shape=shape)
    _same(T1, T2)
    _same(p1, p2)
    _same(acc, acc2)
    _same(macc, macc2)


@pytest.mark.parametrize("accum", [False, True])
def test_two_steps_part_scale_window(accum):
    """The 161 x 161 x 41 Level-3 window of the part-scale workload, with the
    shape the two-step autotuner picks on it."""
    import kern

    N3 = 10
    eng, rA, rB, rows, tab, acc, macc = _case("part_scale", torch.float32, N3)
    L3 = eng.geo.L[3]
    Lw = int(sum(L3.nodes))
    Ts, ps_ = torch.empty_like(eng.T[3]), torch.empty_like(eng.ph[3])
    kw = eng.level_kwargs(3, eng.T[3], Ts, rows[0, 5:6], eng.ph[3], ps_, laser=rows[0], ring=(rA, rB), alpha=0.1)
    if accum:
        kw.update(accum=acc.clone(), max_accum=macc.clone())
    kw["src_tab"] = tab[:Lw]
    tuned = kern.level_autotune2(eng.ps, reps=2, dt2=rows[1, 5:6], src_tab2=tab[Lw:2 * Lw], bc_alpha2=0.2,
                                 bc_beta2=0.8, **kw)
    assert tuned.kernel == 2 and tuned.us > 0
    acc2, macc2 = acc.clone(), macc.clone()
    T1, p1 = per_step(eng, rA, rB, rows, tab, acc if accum else None, macc if accum else None, N3, ONE_STEP)
    T2, p2 = two_step(eng, rA, rB, rows, tab, acc2 if accum else None, macc2 if accum else None, N3)
    _same(T1, T2)
    _same(p1, p2)
    if accum:
        _same(acc, acc2)
        _same(macc, macc2)


def test_two_steps_report_bad_values():
    """A node driven above 1e5 K in the first step sets GM_STATUS_BAD_T."""
    import _native as N
    import kern

    eng, rA, rB, rows, tab, acc, macc = _case("odd", torch.float32, 2)
    L3 = eng.geo.L[3]
    Lw = int(sum(L3.nodes))
    nx, ny, nz = L3.nodes
    T = eng.T[3].clone()
    T[(nz // 2) * nx * ny + (ny // 2) * nx + nx // 2] = 1e9  # an interior node
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    To, po = torch.empty_like(T), torch.empty_like(eng.ph[3])
    kw = eng.level_kwargs(3, T, To, rows[0, 5:6], eng.ph[3], po, laser=rows[0], ring=(rA, rB), alpha=0.5)
    kw.update(src_tab=tab[:Lw], status=status)
    kern.level_step2(eng.ps, dt2=rows[1, 5:6], src_tab2=tab[Lw:2 * Lw], bc_alpha2=1.0, bc_beta2=0.0, **kw)
    torch.cuda.synchronize()
    assert int(status.item()) & N.GM_STATUS_BAD_T


def test_two_steps_unsupported_calls():
    """Calls outside the served feature set are refused, not mis-computed."""
    import _native as N
    import kern

    eng, rA, rB, rows, tab, acc, macc = _case("odd", torch.float32, 2)
    L3 = eng.geo.L[3]
    Lw = int(sum(L3.nodes))
    To, po = torch.empty_like(eng.T[3]), torch.empty_like(eng.ph[3])
    kw = eng.level_kwargs(3, eng.T[3], To, rows[0, 5:6], eng.ph[3], po, laser=rows[0], ring=(rA, rB), alpha=0.5)
    kw["src_tab"] = tab[:Lw]
    two = dict(dt2=rows[1, 5:6], src_tab2=tab[Lw:2 * Lw], bc_alpha2=1.0, bc_beta2=0.0)
    with pytest.raises(N.GomeltError, match="unsupported"):
        kern.level_step2(eng.ps, **two, **dict(kw, src_tab=None))  # no first-step factor table
    with pytest.raises(N.GomeltError, match="unsupported"):
        kern.level_step2(eng.ps, **two, **dict(kw, ne_planes=kw["ne_planes"] - 1))  # nodes above the top plane
    with pytest.raises(N.GomeltError, match="invalid argument"):
        kern.level_step2(eng.ps, **two, **dict(kw, bc_mode=1))  # the ring arrays are required


@pytest.mark.parametrize("N2,N3", [(10, 10), (3, 7)])
@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_subcycle_pairs_on_off(dtype, graph, N2, N3):
    """Three move + subcycle calls of the single-track workload with the
    Level-3 steps two at a time and one at a time: identical fields (an odd
    N3 ends each Level-2 step with a single step)."""
    import copy

    import numpy as np

    import workloads
    from engine import Engine
    from levels import setup_properties
    from test_gpu_parity_scale import _rows

    cfg = workloads.single_track()
    rows = _rows(cfg)
    P = setup_properties(cfg["properties"])
    vstart = np.asarray(cfg["properties"]["laser_center"], dtype=float)
    n23 = N2 * N3
    out = {}
    for pairs in (False, True):
        stream = torch.cuda.Stream()
        with torch.cuda.stream(stream):
            eng = Engine(copy.deepcopy(cfg), P, N2, N3, dtype=dtype, stream=stream)
            eng.use_pairs = pairs
            eng.use_graph = graph
            eng.set_layer(rows[0])
            for c in range(3):
                ch = rows[c * n23:(c + 1) * n23]
                eng.move(ch[0], vstart)
                eng.subcycle(ch)
            stream.synchronize()
        eng.check_status()
        out[pairs] = eng
    a, b = out[False], out[True]
    for lev in (1, 2, 3):
        _same(a.T[lev], b.T[lev])
        _same(a.ph[lev], b.ph[lev])
    for lev in (2, 3):
        _same(a.Tp[lev], b.Tp[lev])
    _same(a.acc3, b.acc3)
    _same(a.macc3, b.macc3)
    assert float(a.T[3].max()) > 2000.0
