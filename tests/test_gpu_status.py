"""The device status word of the level steps: a new value that is non-finite
or above 1e5 K (the bound of the reference's printLevelMaxMin,
go_melt/computeFunctions.py:3635-3664, which ends the run) sets
GM_STATUS_BAD_T; ordinary steps leave it clear.  Through the subcycle the
engine raises GomeltError, and among many batched instances the bad one is
named with one device-to-host read.  The failure is made by the input (an
infinite or huge temperature at one interior node), not by a fault."""

import numpy as np
import pytest
import torch

from test_gpu_separable import CFG, level3_case, run

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [(1, 4, 4, 6), (1, 2, 2, 3), (0, 0, 0, 5)])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_level_step_status(shape, dtype):
    import _native as N

    ps, nn3, kw, ref, _, _ = level3_case(CFG, 5, dtype, False)
    kw["ph_out"] = torch.empty(nn3, dtype=torch.uint8, device="cuda")  # the subcycle's Level-3 feature set
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = run(ps, shape, nn3, dtype, status=status, **kw)
    assert int(status.item()) == 0
    assert np.all(np.isfinite(out))
    nx, ny, nz = kw["nodes"]
    mid = nx // 2 + (ny // 2) * nx + (nz // 2) * nx * ny  # an interior node of the marching planes
    for bad in (float("inf"), 5e7):
        status.zero_()
        T = kw["T_in"].clone()
        T[mid] = bad
        run(ps, shape, nn3, dtype, status=status, **dict(kw, T_in=T))
        assert int(status.item()) & N.GM_STATUS_BAD_T, bad


def _track_engine(dtype, stream):
    import copy

    import workloads
    from engine import Engine
    from levels import setup_properties
    from test_gpu_parity_scale import _rows

    cfg = workloads.single_track()
    rows = _rows(cfg)
    P = setup_properties(cfg["properties"])
    vstart = np.asarray(cfg["properties"]["laser_center"], dtype=float)
    eng = Engine(copy.deepcopy(cfg), P, 10, 10, dtype=dtype, stream=stream)
    eng.set_layer(rows[0])
    eng.move(rows[0], vstart)
    return eng, rows


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_subcycle_status_raises(dtype):
    import _native as N

    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        eng, rows = _track_engine(dtype, stream)
        eng.subcycle(rows[:100])
        stream.synchronize()
        eng.check_status()  # a normal call: clear
        n3 = eng.geo.L[3].nodes
        eng.T[3][n3[0] // 2 + (n3[1] // 2) * n3[0] + (n3[2] // 2) * n3[0] * n3[1]] = float("inf")
        eng.subcycle(rows[100:200])
        stream.synchronize()
    with pytest.raises(N.GomeltError, match="non-finite or out-of-range"):
        eng.check_status()
    eng.check_status()  # the word was cleared by the read


def test_batched_instances_name_the_bad_one():
    import engine
    import workloads
    from test_gpu_batched_subcycle import _engines

    inst = workloads.batched_instances(n=3, seed=7)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        engs, rows, vst = _engines(inst, stream, torch.float32)
        for e, r, v in zip(engs, rows, vst):
            e.move(r[0], v)
        engine.subcycle_batched(engs, [r[:100] for r in rows])
        assert engine.failed_instances(engs) == []
        for e, r, v in zip(engs, rows, vst):
            e.move(r[100], v)
        n3 = engs[1].geo.L[3].nodes
        engs[1].T[3][n3[0] // 2 + (n3[1] // 2) * n3[0] + (n3[2] // 2) * n3[0] * n3[1]] = 1e9
        engine.subcycle_batched(engs, [r[100:200] for r in rows])
        assert engine.failed_instances(engs) == [1]
        assert engine.failed_instances(engs) == []
