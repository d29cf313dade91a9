"""The JSON driver end to end on the GPU against the reference driver's final
outputs (FinalTemperatureFields and accum_time) for the golden cases."""

import json
import os

import numpy as np
import pytest
import torch

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-9), (torch.float32, 1e-4)])
def test_driver_final_fields(case, dtype, tol, tmp_path):
    import go_melt

    g = golden(case)
    cfg = json.loads(str(g["cfg_json"]))
    gpath = tmp_path / "path.gcode"
    gpath.write_text(str(g["gcode"]))
    cfg["nonmesh"]["gcode"] = str(gpath)
    cfg["nonmesh"]["save_path"] = str(tmp_path / "out") + "/"
    cfg["nonmesh"]["toolpath"] = str(tmp_path / "toolpath.txt")
    go_melt.go_melt(cfg, dtype=dtype)
    assert (tmp_path / "toolpath.txt").read_text() == str(g["toolpath_txt"])
    fin = np.load(str(tmp_path / "out" / "FinalTemperatureFields.npz"))
    for k in ("L1T", "L2T", "L3T"):
        ref = g[f"final.{k}"]
        err = np.max(np.abs(fin[k] - ref)) / np.max(np.abs(ref))
        assert err < tol, (k, err)
    # the final Level-0 state file the reference always writes (go_melt.py:501)
    assert any(f.startswith("Level0_") and f.endswith(".vtr") for f in os.listdir(tmp_path / "out"))
    for f in sorted(os.listdir(tmp_path / "out")):
        if f.startswith("accum_time"):
            ref = g[f"final.{f[:-4]}"]
            got = np.load(str(tmp_path / "out" / f))["accum_time"]
            np.testing.assert_allclose(got, ref, rtol=1e-4, atol=1e-9 if dtype == torch.float64 else 1e-7)
