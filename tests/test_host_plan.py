"""Host planning of window moves without a GPU: the per-window tables that
Engine.plan_move stages for one upload are the same bytes whether the
per-axis memos (axis maps, coupling axes, injection tables) are warm or cold,
along a raster that moves the windows along x, then y.  The device pointers
in the tables are the staging buffer's base plus these offsets, so equal
bytes and offsets are equal uploads."""

import numpy as np


class _StagingBuffer:
    """The table arena's host half (TableArena without the device buffer)."""

    ALIGN = 256

    def __init__(self, nbytes):
        self.buf = np.zeros(nbytes, np.uint8)
        self.off = 0
        self.open = False

    def begin(self):
        self.off = 0
        self.open = True

    def put(self, arr, dtype=None):
        a = np.ascontiguousarray(arr if dtype is None else np.asarray(arr, dtype=dtype))
        b = a.reshape(-1).view(np.uint8)
        off = (self.off + self.ALIGN - 1) // self.ALIGN * self.ALIGN
        assert off + b.size <= self.buf.size
        self.buf[off:off + b.size] = b
        self.off = off + b.size
        return 1 << 40 | off

    def upload(self, stream):
        self.open = False


def _planner(cfg, P):
    import engine as E

    eng = E.Engine.__new__(E.Engine)  # the host half only: no device state
    eng.geo = E.Geometry(cfg, P)
    eng.np_dtype = np.float32
    eng._pending = None
    g = eng.geo
    axes = sum(sum(g.L[lv].nodes) for lv in (1, 2, 3)) + sum(g.L0_nodes)
    eng.arena = _StagingBuffer(1 << 20 | (256 * axes + 64 * 1024))
    eng._buf = lambda *a, **k: None
    return eng


def test_plan_move_tables_do_not_depend_on_the_memos():
    import engine as E
    import geometry as G
    import levels
    import workloads

    cfg = workloads.single_track()
    P = levels.setup_properties(cfg["properties"])
    warm, cold = _planner(cfg, P), _planner(cfg, P)
    vstart = np.asarray(cfg["properties"]["laser_center"], dtype=float)
    # along x, then a turn along y (each move shifts the windows by whole coarse cells)
    path = [vstart + [0.02 * i, 0.0, 0.0, 0, 0, 0, 0] for i in range(12)]
    path += [path[-1] + [0.0, 0.02 * i, 0.0, 0, 0, 0, 0] for i in range(1, 8)]
    for v in path:
        warm.plan_move(v, vstart)
        warm._pending = None
        for memo in (G._AXIS_MAPS, G._COUPLE_AXES, E._INJECT_AXES):
            memo.d.clear()
        cold.plan_move(v, vstart)
        cold._pending = None
        assert warm.arena.off == cold.arena.off
        assert np.array_equal(warm.arena.buf[:warm.arena.off], cold.arena.buf[:cold.arena.off])
        for lev in (2, 3):
            for d in range(3):
                assert np.array_equal(warm.geo.L[lev].coords[d], cold.geo.L[lev].coords[d])

