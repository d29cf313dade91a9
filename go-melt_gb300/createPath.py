"""G-code -> laser toolpath rows (the reference's createPath.py interface).

``parsingGcode(Nonmesh, Properties, L2h)`` reads the G-code named by
``Nonmesh["gcode"]`` and writes ``Nonmesh["toolpath"]``: one line per fine
time step, ``x,y,z,Ljump,Ldwell,dt,P`` (x, y, z right-justified ``%.8e`` in 15
columns, flags as integers, dt and P as ``%.8e``), the format the driver reads
back (go_melt/createPath.py:6-188).  It returns the number of lines.

Semantics kept from the reference:
* G1 moves are followed at ``laser_velocity`` in steps of ``timestep_L3``; a
  segment's remainder becomes one short step; ``P = Ljump*laser_power``.
* a segment that ends at a G0 (travel) move has Ljump = 0 (laser off);
* a change of z inserts, at the old position with P = 0, up to ``wait_time``
  steps of ``timestep_L3`` (not beyond ``dwell_time``), then dwell steps of
  ``timestep_L3 * dwell_time_multiplier * N2 * N3`` and a remainder step;
  the segment that jumps to the new layer is not traversed;
* the path ends with the same wait/dwell sequence.
"""

from __future__ import annotations

import re

import numpy as np

_PATTERN = re.compile(r"(?:G(\d+)\s*X(-?\d+\.\d+|-?\d+)\s*Y(-?\d+\.\d+|-?\d+)(?:\s*Z(-?\d+\.\d+|-?\d+))?)")


def format_fixed(val, width=15, precision=8):
    return f"{val:.{precision}e}".rjust(width)


def count_lines(file_path):
    with open(file_path, "r") as f:
        return sum(1 for _ in f)


def gcode_points(text):
    """(x, y, z, is_travel) per G-code move; z persists between moves."""
    pts = []
    z = None
    for g, x, y, zz in _PATTERN.findall(text):
        if zz:
            z = float(zz)
        pts.append((float(x), float(y), z, 0.0 if g == "1" else 1.0))
    return pts


class _Writer:
    def __init__(self, fh=None):
        self.fh = fh
        self.rows = []

    def add(self, x, y, z, jump, dwell, dt, P):
        if self.fh is not None:
            self.fh.write(f"{format_fixed(x)},{format_fixed(y)},{format_fixed(z)},{jump:d},{dwell:d},"
                          f"{dt:.8e},{P:.8e}\n")
        self.rows.append((x, y, z, jump, dwell, dt, P))


def _dwell_block(w, x, y, z, jump, nm, dwell_t, coef, initial_wait=True):
    dt3 = nm["timestep_L3"]
    if initial_wait:
        for k in range(int(nm["wait_time"])):
            if (k + 1) * dt3 > nm["dwell_time"]:
                break
            w.add(x, y, z, jump, 0, dt3, 0)
    if dwell_t > 0:
        rest = max(0, dwell_t - nm["wait_time"] * dt3)
        n = int(rest / dt3 / coef)
        for _ in range(n):
            w.add(x, y, z, jump, 0, dt3 * coef, 0)
        small = rest - n * dt3 * coef
        if small > 0:
            w.add(x, y, z, jump, 0, small, 0)


def toolpath(nm, props, gcode_text, fh=None):
    """Generate the toolpath rows; write them to ``fh`` if given."""
    coef = float(nm["dwell_time_multiplier"] * nm["subcycle_num_L2"] * nm["subcycle_num_L3"])
    dwell_t = max(nm["dwell_time"] - nm["wait_time"] * nm["timestep_L3"], nm["dwell_time"])
    pts = gcode_points(gcode_text)
    w = _Writer(fh)
    dt3 = nm["timestep_L3"]
    vel = nm["laser_velocity"]
    dx = vel * dt3
    x = y = None
    z = pts[0][2]
    jump = 1
    for i in range(len(pts) - 1):
        jump = 1
        a, b = pts[i], pts[i + 1]
        if a[2] != b[2]:
            _dwell_block(w, a[0], a[1], z, jump, nm, dwell_t, coef)
            x, y = a[0], a[1]
            continue
        if b[3] == 1:
            jump = 0
        dist = np.linalg.norm(np.array([b[0] - a[0], b[1] - a[1]]))  # np.float64: 0/0 -> nan, as the reference
        nsteps = int(dist // dx)
        short = (dist % dx) / dx * dt3
        x, y = a[0], a[1]
        ux = vel * (b[0] - a[0]) / dist
        uy = vel * (b[1] - a[1]) / dist
        z = a[2]
        P = jump * props["laser_power"]
        for _ in range(nsteps):
            x += ux * dt3
            y += uy * dt3
            w.add(x, y, z, jump, 1, dt3, P)
        if short > 0:
            x += ux * short
            y += uy * short
            w.add(x, y, z, jump, 1, short, P)
    # closing wait and dwell (the reference writes these with the last flags)
    for k in range(int(int(nm["wait_time"]))):
        if (k + 1) * dt3 > nm["dwell_time"]:
            break
        w.add(x, y, z, jump, 0, dt3, 0)
    _dwell_block(w, x, y, z, jump, nm, dwell_t, coef, initial_wait=False)
    return w.rows


# ---------------------------------------------------------------------------
# Run table of a toolpath (for generating its rows on the device)
# ---------------------------------------------------------------------------
RUN_MOVE, RUN_HOLD = 0, 1


def toolpath_runs(nm, props, gcode_text):
    """The rows of ``toolpath`` as a table of runs, each a float64 record
    (kind, count, x, y, z, jump, ux, uy, dt, P, short):

    * RUN_MOVE: the position is set to (x, y), then ``count`` rows follow, each
      after ``x += ux * dt; y += uy * dt`` (dwell flag 1, time step dt, power
      P), then, if ``short`` > 0, one row after ``x += ux * short; y += uy *
      short`` with time step ``short``;
    * RUN_HOLD: ``count`` rows at (x, y) with dwell flag 0, time step dt and
      power 0.

    Expanding the runs in order with float64 arithmetic (products rounded
    before the sums, no fused multiply-add) gives ``toolpath``'s rows bit for
    bit; the device generator (gm_toolpath_rows) does exactly that."""
    coef = float(nm["dwell_time_multiplier"] * nm["subcycle_num_L2"] * nm["subcycle_num_L3"])
    dwell_t = max(nm["dwell_time"] - nm["wait_time"] * nm["timestep_L3"], nm["dwell_time"])
    pts = gcode_points(gcode_text)
    dt3 = nm["timestep_L3"]
    vel = nm["laser_velocity"]
    dx = vel * dt3
    runs = []

    def hold(x, y, z, jump, n, dt):
        if n > 0:
            if runs and runs[-1][0] == RUN_HOLD and runs[-1][2:6] == [x, y, z, jump] and runs[-1][8] == dt:
                runs[-1][1] += n
            else:
                runs.append([RUN_HOLD, n, x, y, z, jump, 0.0, 0.0, dt, 0.0, 0.0])

    def dwell_block(x, y, z, jump, initial_wait=True):
        if initial_wait:
            n = 0
            for k in range(int(nm["wait_time"])):
                if (k + 1) * dt3 > nm["dwell_time"]:
                    break
                n += 1
            hold(x, y, z, jump, n, dt3)
        if dwell_t > 0:
            rest = max(0, dwell_t - nm["wait_time"] * dt3)
            n = int(rest / dt3 / coef)
            hold(x, y, z, jump, n, dt3 * coef)
            small = rest - n * dt3 * coef
            if small > 0:
                hold(x, y, z, jump, 1, small)

    x = y = None
    z = pts[0][2]
    jump = 1
    for i in range(len(pts) - 1):
        jump = 1
        a, b = pts[i], pts[i + 1]
        if a[2] != b[2]:
            dwell_block(a[0], a[1], z, jump)
            x, y = a[0], a[1]
            continue
        if b[3] == 1:
            jump = 0
        dist = np.linalg.norm(np.array([b[0] - a[0], b[1] - a[1]]))
        nsteps = int(dist // dx)
        short = (dist % dx) / dx * dt3
        ux = vel * (b[0] - a[0]) / dist
        uy = vel * (b[1] - a[1]) / dist
        z = a[2]
        runs.append([RUN_MOVE, nsteps, a[0], a[1], z, jump, ux, uy, dt3, jump * props["laser_power"],
                     short if short > 0 else 0.0])
        # the position after the run, as toolpath() carries it
        x, y = a[0], a[1]
        for _ in range(nsteps):
            x += ux * dt3
            y += uy * dt3
        if short > 0:
            x += ux * short
            y += uy * short
    n = 0
    for k in range(int(int(nm["wait_time"]))):
        if (k + 1) * dt3 > nm["dwell_time"]:
            break
        n += 1
    hold(x, y, z, jump, n, dt3)
    dwell_block(x, y, z, jump, initial_wait=False)
    return np.asarray(runs, dtype=np.float64).reshape(-1, 11)


def run_rows(runs):
    """Number of rows a run table expands to."""
    return int(runs[:, 1].sum()) + int(np.count_nonzero((runs[:, 0] == RUN_MOVE) & (runs[:, 10] > 0)))


def expand_runs(runs, start=0, count=None):
    """Rows [start, start + count) of a run table (the algorithm of the
    device generator, for checking it)."""
    out = []
    total = run_rows(runs)
    count = total - start if count is None else count
    k = 0
    for r in runs:
        kind, n, x, y, z, jump, ux, uy, dt, P, short = r
        n = int(n)
        if kind == RUN_MOVE:
            x, y = float(x), float(y)
            for _ in range(n):
                x += ux * dt
                y += uy * dt
                if start <= k < start + count:
                    out.append((x, y, z, jump, 1.0, dt, P))
                k += 1
            if short > 0:
                x += ux * short
                y += uy * short
                if start <= k < start + count:
                    out.append((x, y, z, jump, 1.0, short, P))
                k += 1
        else:
            for _ in range(n):
                if start <= k < start + count:
                    out.append((x, y, z, jump, 0.0, dt, 0.0))
                k += 1
    return np.asarray(out, dtype=np.float64).reshape(-1, 7)


def parsingGcode(Nonmesh, Properties, L2h):
    with open(Nonmesh["gcode"], "r") as f:
        text = f.read()
    with open(Nonmesh["toolpath"], "w") as fh:
        rows = toolpath(Nonmesh, Properties, text, fh)
    return len(rows)


def serpentine_gcode(x0, y0, length, hatch, ntracks, z=0.0, layers=1, layer_height=0.05):
    """Raster G-code: alternating-direction tracks along x, `hatch` apart in y,
    repeated for `layers` layers (a travel move starts every track)."""
    lines = []
    for L in range(layers):
        zz = z + L * layer_height
        for t in range(ntracks):
            y = y0 + t * hatch
            xa, xb = (x0, x0 + length) if t % 2 == 0 else (x0 + length, x0)
            lines.append(f"G0 X{xa:.4f} Y{y:.4f} Z{zz:.4f}")
            lines.append(f"G1 X{xb:.4f} Y{y:.4f} Z{zz:.4f}")
    return "\n".join(lines) + "\n"
