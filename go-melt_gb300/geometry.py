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


class _Cache:
    """Bounded memo of per-axis tables keyed by the exact coordinate bytes.

    Between two window moves most axes do not change (a raster track moves
    the windows along one axis; Level 1 never moves within a layer), so most
    tables of a move are found here.  Cached arrays are read-only."""

    def __init__(self, cap=1024):
        self.cap = cap
        self.d = {}

    def get(self, key):
        return self.d.get(key)

    def put(self, key, val):
        if len(self.d) >= self.cap:
            self.d.pop(next(iter(self.d)))
        self.d[key] = val
        return val


_AXIS_MAPS = _Cache()


def _frozen(*arrays):
    for a in arrays:
        a.setflags(write=False)


def axis_map(src_coords, tgt_coords) -> AxisMap:
    """Map target coordinates along one axis onto a source node axis."""
    c = np.asarray(src_coords, dtype=np.float64)
    t = np.asarray(tgt_coords, dtype=np.float64)
    key = (c.tobytes(), t.tobytes())
    m = _AXIS_MAPS.get(key)
    if m is not None:
        return m
    h = c[1] - c[0]
    ne = c.size - 1
    e = np.clip(np.floor((t - c[0]) / h).astype(np.int64), 0, ne - 1)
    w = np.empty((t.size, 2), dtype=np.float64)
    w[:, 0] = (c[e + 1] - t) / h
    w[:, 1] = (t - c[e]) / h
    m = AxisMap(e.astype(np.int32), w)
    _frozen(m.elem, m.w)
    return _AXIS_MAPS.put(key, m)


_COUPLE_AXES = _Cache()


def couple_axis(fine_coords, coarse_coords):
    """Per-axis geometry of a fine level inside a coarse level for the
    coupling terms (computeCoarseFineShapeFunctions, :1213-1358, restated per
    axis): Gauss-point coordinates xq (nfe, 2), the coarse element I of each
    Gauss point (clipped floor), the two 1-D coarse weights cw (nfe, 2, 2),
    node0 = the coarse element of Gauss side 0 (the element whose nodes the
    reference assigns the fine element's terms to), and for each coarse
    element lo + j, j < ncb, the range [flo[j], fhi[j]) of fine elements
    assigned to it.  Returns a dict; arrays are read-only."""
    f = np.asarray(fine_coords, dtype=np.float64)
    c = np.asarray(coarse_coords, dtype=np.float64)
    key = (f.tobytes(), c.tobytes())
    r = _COUPLE_AXES.get(key)
    if r is not None:
        return r
    xq = quad_points_1d(f)
    H = c[1] - c[0]
    nce = c.size - 1
    I = np.clip(np.floor((xq - c[0]) / H).astype(np.int64), 0, nce - 1)
    cw = np.empty(xq.shape + (2,), dtype=np.float64)
    cw[..., 0] = (c[I + 1] - xq) / H
    cw[..., 1] = (xq - c[I]) / H
    node0 = I[:, 0]
    lo = int(node0.min())
    ncb = int(node0.max()) - lo + 1
    cells = lo + np.arange(ncb)
    flo = np.searchsorted(node0, cells, side="left")
    fhi = np.searchsorted(node0, cells, side="right")
    r = dict(xq=xq, cw=cw, node0=node0.astype(np.int32), flo=flo.astype(np.int32), fhi=fhi.astype(np.int32),
             lo=lo, ncb=ncb, rmax=int((fhi - flo).max()), H=float(H))
    _frozen(r["xq"], r["cw"], r["node0"], r["flo"], r["fhi"])
    return _COUPLE_AXES.put(key, r)


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
