"""Whole subcycle calls of several scan instances of uneven mesh sizes as one
CUDA graph of parallel branches (gm_subcycle_batched) against the same
instances run one at a time: identical fields, phases and melt time after
three move + subcycle steps (the first batched call issues directly, the
later ones replay an updated graph)."""

import copy

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _engines(inst, stream, dtype):
    from engine import Engine
    import surrogate_run as SR

    engs, rows, vst = [], [], []
    for cfg in inst:
        P, nm, r = SR._instance_rows(copy.deepcopy(cfg))
        e = Engine(copy.deepcopy(cfg), P, nm["subcycle_num_L2"], nm["subcycle_num_L3"], dtype=dtype, stream=stream)
        e.use_persist = False
        e.set_layer(r[0])
        engs.append(e)
        rows.append(r)
        vst.append(np.asarray(cfg["properties"]["laser_center"], dtype=float))
    return engs, rows, vst


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_batched_subcycles_equal_single_runs(dtype):
    import engine
    import workloads

    inst = workloads.batched_instances(n=4, seed=7)
    assert len({tuple(c["Level1"]["elements"]) for c in inst}) > 1  # uneven Level-1 meshes
    out = {}
    for mode in ("single", "batched"):
        stream = torch.cuda.Stream()
        with torch.cuda.stream(stream):
            engs, rows, vst = _engines(inst, stream, dtype)
            for k in range(3):
                for e, r, v in zip(engs, rows, vst):
                    e.move(r[k * 100], v)
                if mode == "batched":
                    engine.subcycle_batched(engs, [r[k * 100:(k + 1) * 100] for r in rows])
                else:
                    for e, r in zip(engs, rows):
                        e.subcycle(r[k * 100:(k + 1) * 100])
            stream.synchronize()
        out[mode] = engs
    hot = 0
    for a, b in zip(out["single"], out["batched"]):
        for lev in (1, 2, 3):
            torch.testing.assert_close(b.T[lev], a.T[lev], rtol=0, atol=0)
            assert torch.equal(b.ph[lev], a.ph[lev])
        for lev in (2, 3):
            torch.testing.assert_close(b.Tp[lev], a.Tp[lev], rtol=0, atol=0)
        torch.testing.assert_close(b.acc3, a.acc3, rtol=0, atol=0)
        torch.testing.assert_close(b.macc3, a.macc3, rtol=0, atol=0)
        assert torch.equal(b.L0, a.L0)
        hot += float(a.T[3].max()) > 1000.0
    assert hot == len(inst)


def test_batched_subcycle_rejects_shared_default_stream():
    import _native as N
    import engine
    import workloads

    inst = workloads.batched_instances(n=2, seed=7)
    engs, rows, vst = _engines(inst, None, torch.float32)
    for e, r, v in zip(engs, rows, vst):
        e.move(r[0], v)
    with pytest.raises(N.GomeltError):
        engine.subcycle_batched(engs, [r[:100] for r in rows])
