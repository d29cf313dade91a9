"""The product's G-code -> toolpath generator reproduces the reference's
toolpath files byte for byte (CPU only)."""

import io
import json

import numpy as np

from conftest import golden


def test_toolpath_text(case):
    from createPath import toolpath
    from levels import setup_nonmesh, setup_properties

    g = golden(case)
    cfg = json.loads(str(g["cfg_json"]))
    nm = setup_nonmesh(cfg["nonmesh"])
    P = setup_properties(cfg["properties"])
    buf = io.StringIO()
    rows = toolpath(nm, P, str(g["gcode"]), buf)
    ref = str(g["toolpath_txt"])
    assert buf.getvalue() == ref
    assert len(rows) == ref.count("\n")


def test_serpentine_shape():
    from createPath import gcode_points, serpentine_gcode

    pts = gcode_points(serpentine_gcode(1.0, 2.0, 4.0, 0.1, 3, layers=2))
    assert len(pts) == 12
    assert pts[0][3] == 1.0 and pts[1][3] == 0.0
    assert np.isclose(pts[3][0], 1.0) and np.isclose(pts[6][2], 0.05)


def _raster_inputs(layers=1, ntracks=40):
    import createPath
    import levels
    import workloads

    cfg = workloads.part_scale_raster()
    r = cfg["raster"]
    P = levels.setup_properties(cfg["properties"])
    nm = levels.setup_nonmesh(cfg["nonmesh"])
    return nm, P, createPath.serpentine_gcode(r["x0"], r["y0"], r["length"], r["hatch"], ntracks, layers=layers)


def test_run_table_expands_to_the_rows(case):
    """The run table the device generator expands reproduces the toolpath rows
    bit for bit (golden G-codes, the single track, a three-layer raster)."""
    import createPath
    import workloads
    from levels import setup_nonmesh, setup_properties

    g = golden(case)
    cfg = json.loads(str(g["cfg_json"]))
    inputs = [(setup_nonmesh(cfg["nonmesh"]), setup_properties(cfg["properties"]), str(g["gcode"]))]
    st = workloads.single_track()
    inputs.append((setup_nonmesh(st["nonmesh"]), setup_properties(st["properties"]), st["gcode"]))
    inputs.append(_raster_inputs(layers=3, ntracks=3))
    for nm, P, text in inputs:
        rows = np.asarray(createPath.toolpath(nm, P, text), dtype=np.float64)
        runs = createPath.toolpath_runs(nm, P, text)
        assert createPath.run_rows(runs) == len(rows)
        ex = createPath.expand_runs(runs)
        np.testing.assert_array_equal(ex.view(np.uint64), rows.view(np.uint64))
        part = createPath.expand_runs(runs, 5, 11)
        np.testing.assert_array_equal(part.view(np.uint64), rows[5:16].view(np.uint64))
        assert len(runs) < len(rows)


def test_step_dts_are_row_order_sums():
    from engine import step_dts

    rows = np.zeros((6, 7))
    rows[:, 5] = [1e-5, 2e-5, 3e-5, 1e-16, 1.0, 1e-5]
    d = step_dts(rows, 2)
    acc = 0.0
    for v in rows[:, 5]:
        acc += v
    assert d[0] == acc
    assert d[1] == (1e-5 + 2e-5) + 3e-5 and d[2] == (1e-16 + 1.0) + 1e-5
