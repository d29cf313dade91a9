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
