"""Toolpath rows generated on the device (gm_toolpath_rows, FP64 position and
time accumulation) against the host generator createPath.toolpath: bit for
bit, chunk by chunk, as the subcycle consumes them."""

import json

import numpy as np
import pytest
import torch

from conftest import golden

pytestmark = pytest.mark.gpu


def _device_chunks(runs, n23, N2, nchunks):
    from engine import DeviceToolpath

    tp = DeviceToolpath(runs, "cuda")
    rows = torch.empty(nchunks * n23 * 7, dtype=torch.float64, device="cuda")
    dts = torch.empty(nchunks * (N2 + 1), dtype=torch.float64, device="cuda")
    for c in range(nchunks):
        tp.next(n23, N2, rows[c * n23 * 7:(c + 1) * n23 * 7], dts[c * (N2 + 1):(c + 1) * (N2 + 1)])
    torch.cuda.synchronize()
    return tp, rows.cpu().numpy().reshape(-1, 7), dts.cpu().numpy().reshape(nchunks, N2 + 1)


def _check(nm, P, text, N2, N3, nchunks=None):
    import createPath
    from engine import step_dts

    rows = np.asarray(createPath.toolpath(nm, P, text), dtype=np.float64)
    runs = createPath.toolpath_runs(nm, P, text)
    n23 = N2 * N3
    nchunks = nchunks or -(-len(rows) // n23)
    tp, got, dts = _device_chunks(runs, n23, N2, nchunks)
    n = min(len(rows), nchunks * n23)
    np.testing.assert_array_equal(got[:n].view(np.uint64), rows[:n].view(np.uint64))
    assert np.all(got[n:] == 0)  # past the end of the path
    padded = np.zeros((nchunks * n23, 7))
    padded[:n] = rows[:n]
    for c in range(nchunks):
        np.testing.assert_array_equal(dts[c].view(np.uint64),
                                      step_dts(padded[c * n23:(c + 1) * n23], N2).view(np.uint64))
    t = 0.0
    for v in padded[:, 5]:
        t += v
    run, k, emitted, x, y, tt = tp.state_host()
    assert emitted == nchunks * n23 and tt == t
    return len(rows)


def test_device_rows_golden_gcodes(case):
    from levels import setup_nonmesh, setup_properties

    g = golden(case)
    cfg = json.loads(str(g["cfg_json"]))
    nm = setup_nonmesh(cfg["nonmesh"])
    n = _check(nm, setup_properties(cfg["properties"]), str(g["gcode"]), nm["subcycle_num_L2"],
               nm["subcycle_num_L3"])
    assert n > 0


def test_device_rows_single_track():
    import workloads
    from levels import setup_nonmesh, setup_properties

    cfg = workloads.single_track()
    assert _check(setup_nonmesh(cfg["nonmesh"]), setup_properties(cfg["properties"]), cfg["gcode"], 10, 10) > 2500


@pytest.mark.parametrize("layers,ntracks,nchunks", [(1, 40, 120), (3, 4, None)])
def test_device_rows_serpentine_raster(layers, ntracks, nchunks):
    from test_toolpath import _raster_inputs

    nm, P, text = _raster_inputs(layers, ntracks)
    _check(nm, P, text, 10, 10, nchunks)
