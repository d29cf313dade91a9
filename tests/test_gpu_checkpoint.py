"""Checkpoint and restart through the JSON driver (go_melt.py:115-129 load with
a toolpath seek, :390-411 save at a layer change): a run stopped at a layer's
checkpoint and restarted from it ends with the same fields, bit for bit, as
the run that never stopped.

The workload is the golden two-layer case's mesh and material with a
three-layer G-code, so the restart at layer 1 also carries the Level-1 S1
layer store through the checkpoint into the next layer change, and a second
restart at layer 2 checks a checkpoint written by a restarted run."""

import copy
import json
import os

import numpy as np
import pytest
import torch

from conftest import golden

pytestmark = pytest.mark.gpu

GCODE3 = ("G0 X0.44 Y0.5 Z0.05\nG1 X0.52 Y0.5 Z0.05\n"
          "G0 X0.52 Y0.48 Z0.1\nG1 X0.44 Y0.48 Z0.1\n"
          "G0 X0.44 Y0.52 Z0.15\nG1 X0.52 Y0.52 Z0.15\n")


def _cfg(tmp, name, layer_num, restart_layer_num):
    g = golden("two_layers")
    cfg = json.loads(str(g["cfg_json"]))
    d = tmp / name
    (d / "out").mkdir(parents=True, exist_ok=True)
    (d / "path.gcode").write_text(GCODE3)
    cfg["nonmesh"].update(gcode=str(d / "path.gcode"), save_path=str(d / "out") + "/",
                          toolpath=str(d / "toolpath.txt"), layer_num=layer_num,
                          restart_layer_num=restart_layer_num)
    return cfg


def _final(d):
    f = np.load(str(d / "out" / "FinalTemperatureFields.npz"))
    return {k: f[k] for k in ("L1T", "L2T", "L3T")}


def _copy_checkpoints(src, dst):
    s, t = src / "out" / "checkpoint", dst / "out" / "checkpoint"
    t.mkdir(parents=True, exist_ok=True)
    for f in os.listdir(s):
        (t / f).write_bytes((s / f).read_bytes())


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_restart_matches_uninterrupted_run(tmp_path, dtype):
    import go_melt

    # uninterrupted: layer checkpoints are written on the way
    full = _cfg(tmp_path, "full", 0, 10000)
    go_melt.go_melt(copy.deepcopy(full), dtype=dtype)
    ref = _final(tmp_path / "full")
    ck = tmp_path / "full" / "out" / "checkpoint"
    assert sorted(os.listdir(ck)) == ["Checkpoint0001.pkl", "Checkpoint0002.pkl"]
    assert max(float(np.max(v)) for v in ref.values()) > 800.0  # the laser melted something

    # stop at the layer-1 checkpoint
    stop = _cfg(tmp_path, "stop", 0, 1)
    go_melt.go_melt(copy.deepcopy(stop), dtype=dtype)
    assert not (tmp_path / "stop" / "out" / "FinalTemperatureFields.npz").exists()
    assert sorted(os.listdir(tmp_path / "stop" / "out" / "checkpoint")) == ["Checkpoint0001.pkl"]

    # restart from it (a fresh engine in this process) and run to the end
    rest = _cfg(tmp_path, "restart", 1, 10000)
    _copy_checkpoints(tmp_path / "stop", tmp_path / "restart")
    go_melt.go_melt(copy.deepcopy(rest), dtype=dtype)
    got = _final(tmp_path / "restart")
    for k in ref:
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
    for name in ("accum_time0002.npz",):
        a = np.load(str(tmp_path / "full" / "out" / name))["accum_time"]
        b = np.load(str(tmp_path / "restart" / "out" / name))["accum_time"]
        np.testing.assert_array_equal(b, a)

    # restart from the layer-2 checkpoint the restarted run wrote
    rest2 = _cfg(tmp_path, "restart2", 2, 10000)
    _copy_checkpoints(tmp_path / "restart", tmp_path / "restart2")
    go_melt.go_melt(copy.deepcopy(rest2), dtype=dtype)
    got2 = _final(tmp_path / "restart2")
    for k in ref:
        np.testing.assert_array_equal(got2[k], ref[k], err_msg=k)
