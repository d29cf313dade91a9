"""The VTK rectilinear-grid writer: round trip of coordinates and point data
(x fastest), and the file header."""

import numpy as np

import vtk


def test_vtr_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    x, y, z = np.linspace(0, 1, 5), np.linspace(-1, 0, 4), np.linspace(2, 3, 3)
    T = rng.random(60).astype(np.float32)
    S = (rng.random(60) > 0.5).astype(np.float64)
    ph = rng.integers(0, 2, 60).astype(np.uint8)
    f = vtk.write_vtr(tmp_path / "Level3_00000001", x, y, z - 1e-3,
                      {"Temperature (K)": T, "State (Powder/Solid)": S, "phase": ph})
    assert f.endswith("Level3_00000001.vtr")
    head = open(f, "rb").read(400).decode("ascii", "replace")
    assert 'type="RectilinearGrid"' in head and 'WholeExtent="0 4 0 3 0 2"' in head
    xr, yr, zr, pd = vtk.read_vtr(f)
    assert np.array_equal(xr, x) and np.array_equal(yr, y) and np.array_equal(zr, z - 1e-3)
    assert np.array_equal(pd["Temperature (K)"], T) and pd["Temperature (K)"].dtype == np.float32
    assert np.array_equal(pd["State (Powder/Solid)"], S) and np.array_equal(pd["phase"], ph)
