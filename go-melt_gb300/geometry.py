"""Host-side (FP64) geometry of GO-MELT's structured levels.

The device kernels never see coordinate arrays.  Everything they need about
where one grid sits inside another is reduced here to small per-axis tables
(``AxisMap``) computed in double precision with the reference's own rules:

* coarse element of a point: ``clip(floor((x - x0)/h), 0, ne-1)`` with
  ``h = x[1] - x[0]`` (interpolatePointsMatrix, go_melt/computeFunctions.py
  :1068-1076);
* the two linear weights ``((x_{e+1} - x)/h, (x - x_e)/h)`` whose products
  are the trilinear weights of compute3DN (:1361-1393).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

INV_SQ3 = 1.0 / np.sqrt(3.0)


@dataclass
class AxisMap:
    elem: np.ndarray  # int32 (n,)
    w: np.ndarray     # float64 (n, 2)


def axis_map(src_coords, tgt_coords) -> AxisMap:
    """Map target coordinates along one axis onto a source node axis."""
    c = np.asarray(src_coords, dtype=np.float64)
    t = np.asarray(tgt_coords, dtype=np.float64)
    h = c[1] - c[0]
    ne = c.size - 1
    e = np.clip(np.floor((t - c[0]) / h).astype(np.int64), 0, ne - 1)
    w0 = (c[e + 1] - t) / h
    w1 = (t - c[e]) / h
    return AxisMap(e.astype(np.int32), np.stack([w0, w1], axis=1))


def quad_points_1d(coords):
    """Gauss-point coordinates of the elements along one axis: (ne, 2).

    Side 0 is the point at xi = -1/sqrt(3), side 1 at +1/sqrt(3), i.e. the
    reference's quadrature points 0 and 1 (getQuadratureCoords, :3151-3166).
    """
    c = np.asarray(coords, dtype=np.float64)
    a, b = c[:-1], c[1:]
    lo = 0.5 * (1 + INV_SQ3) * a + 0.5 * (1 - INV_SQ3) * b
    hi = 0.5 * (1 - INV_SQ3) * a + 0.5 * (1 + INV_SQ3) * b
    return np.stack([lo, hi], axis=1)


def grid_origin_spacing(coords):
    c = np.asarray(coords, dtype=np.float64)
    return float(c[0]), float(c[1] - c[0])
