"""gm_subcycle as one CUDA graph per call (captured, updated in place) gives
the same fields, bit for bit, as the directly issued launches, over several
moving-window steps of the part-scale workload's Level-1/2/3 geometry at a
reduced size."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def run(use_graph, nsteps=4):
    import createPath
    import engine
    import levels
    import workloads

    cfg = workloads.single_track()
    P = levels.setup_properties(cfg["properties"])
    nm = levels.setup_nonmesh(cfg["nonmesh"])
    rows = np.asarray(createPath.toolpath(nm, P, cfg["gcode"]), dtype=np.float64)
    st = torch.cuda.Stream()
    vstart = np.asarray(cfg["properties"]["laser_center"], dtype=float)
    with torch.cuda.stream(st):
        e = engine.Engine(cfg, P, 10, 10, stream=st)
        e.use_graph = use_graph
        e.set_layer(rows[0])
        for k in range(nsteps):
            e.move(rows[k * 100], vstart)
            e.subcycle(rows[k * 100:(k + 1) * 100])
    st.synchronize()
    return e


def test_graph_mode_matches_direct():
    a = run(False)
    b = run(True)
    for lev in (1, 2, 3):
        assert torch.equal(a.T[lev], b.T[lev]), lev
        assert torch.equal(a.ph[lev], b.ph[lev]), lev
    for lev in (2, 3):
        assert torch.equal(a.Tp[lev], b.Tp[lev]), lev
    assert torch.equal(a.acc3, b.acc3) and torch.equal(a.macc3, b.macc3)
    assert torch.equal(a.L0, b.L0)
