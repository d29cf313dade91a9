"""Multilevel engine: device state of Levels 0-3 and the hot-path sequences.

``Engine.move`` is moveEverything (go_melt/computeFunctions.py:2400-2510),
``Engine.subcycle`` is subcycleGOMELT (:3224-3632), ``Engine.step`` is
stepGOMELT (:2304-2397) and ``Engine.dwell`` is stepGOMELTDwellTime
(:2617-2664), each issued as a sequence of libgomelt kernels on one CUDA
stream.  Host work per call is limited to FP64 index arithmetic and small
per-axis tables; fields stay on the device.

Device layout (per level, node-major, x fastest): T (float32 or float64),
T' (Levels 2, 3), phase byte (bit0 S1, bit1 S2).  Level 0 keeps one byte
(S1) per node of the part footprint at Level-3 resolution; its S2, which the
reference stores only inside the last written window (:2390-2392), is taken
from Level 3's phase at gather time.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

import _native as N
import kern
from geometry import _Cache, axis_map, couple_axis
from levels import Geometry

PH_S1, PH_S2 = 1, 2


def l0_words(nodes):
    """32-bit words of the bit-packed Level-0 S1 store of a node grid (each
    (y, z) row of nodes[0] bits padded to whole words)."""
    return ((int(nodes[0]) + 31) // 32) * int(nodes[1]) * int(nodes[2])


def l0_pack(s1, nodes):
    """Bit-pack a Level-0 S1 array (nodes[0]*nodes[1]*nodes[2] values, set
    where > 0.499) into the store's int32 words (torch, on s1's device; one
    byte of work space per node)."""
    t = torch.as_tensor(s1)
    nx, ny, nz = (int(v) for v in nodes)
    wpr = (nx + 31) // 32
    rows = nz * ny
    pad = torch.zeros(rows, wpr * 32, dtype=torch.uint8, device=t.device)
    pad[:, :nx] = (t.reshape(rows, nx) > 0.499).to(torch.uint8)
    sh = torch.arange(8, dtype=torch.uint8, device=t.device)
    byt = (pad.reshape(rows, wpr * 4, 8) << sh).sum(dim=2, dtype=torch.uint8)  # little-endian bytes of the words
    return byt.reshape(-1).view(torch.int32).clone()


def l0_unpack(words, nodes):
    """Level-0 S1 (uint8 0/1 per node, node-major) from the store's words."""
    nx, ny, nz = (int(v) for v in nodes)
    wpr = (nx + 31) // 32
    rows = nz * ny
    byt = words.contiguous().view(torch.uint8).reshape(rows, wpr * 4)
    sh = torch.arange(8, dtype=torch.uint8, device=words.device)
    bits = (byt[:, :, None] >> sh) & 1
    return bits.reshape(rows, wpr * 32)[:, :nx].reshape(-1).contiguous()


class TableArena:
    """Per-window tables of one move packed into a pinned host buffer and copied
    to a device buffer with one non-blocking H2D copy.  Two pinned buffers
    alternate so the host can fill the next move's tables while the previous
    copy is in flight; the device buffer is rewritten in stream order."""

    ALIGN = 256

    def __init__(self, nbytes, device):
        self.nbytes = int(nbytes)
        self.dev = torch.empty(self.nbytes, dtype=torch.uint8, device=device)
        self.host = [torch.empty(self.nbytes, dtype=torch.uint8, pin_memory=True) for _ in range(2)]
        self.hview = [h.numpy() for h in self.host]
        self.evt = [None, None]
        self.cur = 0
        self.off = 0
        self.open = False

    def begin(self):
        self.cur ^= 1
        if self.evt[self.cur] is not None:
            self.evt[self.cur].synchronize()
        self.off = 0
        self.open = True

    def put(self, arr, dtype=None):
        """Stage an array; returns its device address (valid after upload)."""
        a = np.ascontiguousarray(arr if dtype is None else np.asarray(arr, dtype=dtype))
        b = a.reshape(-1).view(np.uint8)
        off = (self.off + self.ALIGN - 1) // self.ALIGN * self.ALIGN
        if off + b.size > self.nbytes:
            raise N.GomeltError(f"table arena too small ({off + b.size} > {self.nbytes} bytes)")
        self.hview[self.cur][off:off + b.size] = b
        self.off = off + b.size
        return self.dev.data_ptr() + off

    def upload(self, stream):
        n = self.off
        s = stream if stream is not None else torch.cuda.current_stream()
        with torch.cuda.stream(s):
            self.dev[:n].copy_(self.host[self.cur][:n], non_blocking=True)
        e = torch.cuda.Event()
        e.record(s)
        self.evt[self.cur] = e
        self.open = False


class ArenaMap3:
    """gm_map3 whose per-axis tables live in the table arena."""

    def __init__(self, arena, maps, src_nodes, np_dtype):
        s = N.gm_map3()
        self.n = [int(m.elem.size) for m in maps]
        for d, m in enumerate(maps):
            s.n[d] = self.n[d]
            s.elem[d] = arena.put(m.elem, np.int32)
            s.w[d] = arena.put(m.w.reshape(-1), np_dtype)
        s.src_nx, s.src_ny = int(src_nodes[0]), int(src_nodes[1])
        self.struct = s


class CoupleGeom:
    """Per-axis tables of a fine level inside a coarse level (gm_couple_geom),
    staged in the table arena."""

    def __init__(self, fine_coords, coarse_coords, np_dtype, arena):
        self.axes = []
        g = N.gm_couple_geom()
        for d in range(3):
            r = couple_axis(fine_coords[d], coarse_coords[d])
            a = g.ax[d]
            a.nfe = r["xq"].shape[0]
            a.cw = arena.put(r["cw"].reshape(-1), np_dtype)
            a.node0 = C.cast(arena.put(r["node0"]), C.POINTER(C.c_int))
            a.cb_lo = r["lo"]
            a.ncb = r["ncb"]
            a.flo = C.cast(arena.put(r["flo"]), C.POINTER(C.c_int))
            a.fhi = C.cast(arena.put(r["fhi"]), C.POINTER(C.c_int))
            a.rmax = r["rmax"]
            a.H = r["H"]
            self.axes.append(dict(lo=r["lo"], ncb=r["ncb"], xq=arena.put(r["xq"].reshape(-1))))
        self.struct = g
        self.box_lo = [ax["lo"] for ax in self.axes]
        self.box_n = [ax["ncb"] + 1 for ax in self.axes]
        self.partials = int(N.lib().gm_couple_partials_size(C.byref(g)))


def step_dts(rows, N2):
    """dt of the Level-1 step and of each of the N2 Level-2 steps of a chunk of
    toolpath rows: sums of the rows' dt in row order (the order the device
    toolpath generator, gm_toolpath_rows, sums them in)."""
    dt = [float(v) for v in np.asarray(rows, dtype=np.float64)[:, 5]]
    per = len(dt) // N2
    out = [0.0] * (N2 + 1)
    for i, v in enumerate(dt):
        out[0] += v
        out[1 + i // per] += v
    return np.asarray(out, dtype=np.float64)


class DeviceToolpath:
    """Toolpath rows generated on the device (gm_toolpath_rows): the run table
    of createPath.toolpath_runs is uploaded once; each ``next`` call expands
    the next chunk into device rows and step dts, with the position and the
    elapsed time accumulated in FP64 in a device-resident state."""

    def __init__(self, runs, device, stream=None):
        import createPath

        runs = np.ascontiguousarray(np.asarray(runs, dtype=np.float64).reshape(-1, 11))
        self.nruns = runs.shape[0]
        self.total = createPath.run_rows(runs)
        self.dev = torch.device(device)
        self.stream = stream
        self.runs = torch.as_tensor(runs.reshape(-1), device=self.dev)
        self.state = torch.zeros(C.sizeof(N.gm_toolpath_state) // 8, dtype=torch.int64, device=self.dev)
        self.emitted = 0

    def next(self, nrows, ngroups, rows_out, dts_out):
        """Expand rows [emitted, emitted + nrows) into rows_out (nrows x 7
        float64) and their dts (ngroups + 1 float64) on the stream."""
        if rows_out.dtype != torch.float64 or dts_out.dtype != torch.float64:
            raise N.GomeltError("toolpath rows and dts are float64")
        if rows_out.numel() < 7 * nrows or dts_out.numel() < ngroups + 1:
            raise N.GomeltError("toolpath output buffers too small")
        N.call("gm_toolpath_rows", self.runs.data_ptr(), self.nruns, self.state.data_ptr(), int(nrows), int(ngroups),
               kern.ptr(rows_out), kern.ptr(dts_out), kern.stream_ptr(self.stream))
        self.emitted += int(nrows)

    def state_host(self):
        """(run, k, rows emitted, x, y, elapsed time) of the device state."""
        raw = self.state.cpu().numpy()
        f = raw.view(np.float64)
        return int(raw[0]), int(raw[1]), int(raw[2]), float(f[3]), float(f[4]), float(f[5])


_INJECT_AXES = _Cache()


def _inject_axis(fine_c, fine_n, overlap_c, overlap_i, coarse_c):
    """One axis of Engine._inject: (cf0, cf1, c_of_f) as int32 arrays, or
    False when the overlap coordinates do not all coincide with fine nodes.
    Memoised on the exact inputs (a raster move changes one axis); the cached
    arrays are read-only."""
    fc = np.asarray(fine_c, dtype=np.float64)
    oc = np.asarray(overlap_c, dtype=np.float64)
    ci = np.asarray(overlap_i, dtype=np.int64)
    cc = np.asarray(coarse_c, dtype=np.float64)
    key = (fc.tobytes(), oc.tobytes(), ci.tobytes(), cc.tobytes(), int(fine_n))
    hit = _INJECT_AXES.get(key)
    if hit is not None:
        return hit
    m = axis_map(fc, oc)
    e = np.asarray(m.elem, dtype=np.int64)
    w = np.asarray(m.w)
    at0, at1 = np.abs(w[:, 1]) <= 1e-9, np.abs(w[:, 0]) <= 1e-9
    nc = len(cc)
    r = False
    if np.all(at0 | at1):
        f = np.where(at0, e, e + 1)
        if not (f.min() < 0 or f.max() >= fine_n or ci.min() < 0 or ci.max() >= nc):
            foc = np.full(nc, -1, dtype=np.int64)  # coarse index -> coinciding fine index
            foc[ci] = f
            b = np.full(int(fine_n), -1, dtype=np.int32)
            b[f] = ci
            ce = np.asarray(axis_map(cc, fc).elem, dtype=np.int64)  # as cmap
            r = (foc[ce].astype(np.int32), foc[ce + 1].astype(np.int32), b)
            for x in r:
                x.setflags(write=False)
    return _INJECT_AXES.put(key, r)


class MovePlan:
    """Host half of one window move (see Engine.plan_move)."""

    __slots__ = ("v", "move_v", "m3", "m2", "tables", "table_bytes")

    def __init__(self, v, move_v, m3, m2, tables, table_bytes):
        self.v, self.move_v, self.m3, self.m2, self.tables, self.table_bytes = v, move_v, m3, m2, tables, table_bytes


class Engine:
    def __init__(self, solver_input: dict, props: dict, N2: int, N3: int, dtype=torch.float32, device="cuda",
                 stream=None):
        self.geo = Geometry(solver_input, props)
        self.P = props
        self.ps = N.props_struct(props)
        self.dtype = dtype
        self.dev = torch.device(device)
        self.N2, self.N3 = int(N2), int(N3)
        self.stream = stream
        g = self.geo
        Tamb = float(props["T_amb"])
        f = dict(dtype=dtype, device=self.dev)
        self.T = {lv: torch.full((g.L[lv].nn,), Tamb, **f) for lv in (1, 2, 3)}
        self.Tp = {lv: torch.zeros(g.L[lv].nn, **f) for lv in (2, 3)}
        self.ph = {lv: torch.zeros(g.L[lv].nn, dtype=torch.uint8, device=self.dev) for lv in (1, 2, 3)}
        self.L0 = torch.zeros(l0_words(g.L0_nodes), dtype=torch.int32, device=self.dev)  # bit-packed S1
        self.acc3 = torch.zeros(g.L[3].nn, **f)
        self.macc3 = torch.zeros(g.L[3].nn, **f)
        self.s2_prev_lo = None  # Level-0 start of the window last written (S2 snapshot)
        self._pending = None  # MovePlan made by plan_move and not yet applied
        self.use_graph = False  # run gm_subcycle as one CUDA graph per call
        self.use_pdl = True  # level steps as programmatic dependent launches
        # a Level-2 step's N3 Level-3 steps as one launch: 0 one launch a step, 1 the window in shared memory
        # (gm_level3_persist, where the window has a shape), 2 the one-step kernel's body with grid barriers
        # (gm_level3_steps); constant-property materials only
        self.use_persist = 0
        # with one launch a step: the Level-3 steps two at a time (gm_level_step2; constant-property
        # materials); autotune() turns it on where the pair measures faster than two single steps
        self.use_pairs = False
        self.status = torch.zeros(1, dtype=torch.int32, device=self.dev)  # GM_PERSIST_* bits of the device kernels
        self.last_table_bytes = 0  # bytes of the last move's table upload
        self.substrate = g.substrate()
        self.tmp = None
        self._work = None
        self.tables = None
        self.np_dtype = np.float32 if dtype == torch.float32 else np.float64
        axes = sum(sum(g.L[lv].nodes) for lv in (1, 2, 3)) + sum(g.L0_nodes)
        self.arena = TableArena(1 << 20 | (256 * axes + 64 * 1024), self.dev)
        self.rarena = TableArena(8 * 8 * (self.N2 * self.N3 * 7 + self.N2 + 1) + 4096, self.dev)

    # ------------------------------------------------------------------
    # helpers
    # ------------------------------------------------------------------
    def _buf(self, name, n, dtype=None):
        if self._work is None:
            self._work = {}
        t = self._work.get(name)
        dt = dtype or self.dtype
        if t is None or t.numel() < n or t.dtype != dt:
            t = torch.empty(n, dtype=dt, device=self.dev)
            self._work[name] = t
        return t[:n]

    def _map(self, src_level_coords, src_nodes, tgt_coords):
        return ArenaMap3(self.arena, [axis_map(src_level_coords[d], tgt_coords[d]) for d in range(3)], src_nodes,
                         self.np_dtype)

    def _interp(self, terms, n, out, base=None, out_term=None, which=0):
        a = N.gm_interp_args()
        a.dtype = kern.dtype_code(out)
        for d in range(3):
            a.n[d] = int(n[d])
        a.nterms = len(terms)
        for q, (m, src, coef) in enumerate(terms):
            a.map[q] = m.struct
            a.src[q] = kern.ptr(src)
            a.coef[q] = float(coef)
        a.base = kern.ptr(base)
        a.out = kern.ptr(out)
        a.out_term = kern.ptr(out_term)
        a.which_term = int(which)
        N.call("gm_interp", C.byref(a), kern.stream_ptr(self.stream))

    def _inject(self, fine_coords, fine_nodes, overlap_coords, overlap_idx, coarse_coords):
        """Tables of gm_tprime_inject (cf0[3], cf1[3], c_of_f[3]) when the
        restriction of the fine level at the coarse overlap nodes is an
        injection (each overlap coordinate coincides with a fine node: weights
        0 / 1 within 1e-9), else None."""
        axes = [_inject_axis(fine_coords[d], fine_nodes[d], overlap_coords[d], overlap_idx[d], coarse_coords[d])
                for d in range(3)]
        if any(r is False for r in axes):
            return None
        cf0, cf1, cof = ([r[q] for r in axes] for q in range(3))
        return [C.cast(self.arena.put(x, np.int32), C.POINTER(C.c_int)) for x in cf0 + cf1 + cof]

    def _idx_tensor(self, arrs, nodes, what):
        """Stage per-axis node-index arrays (device int pointers) after checking
        they address the grid."""
        for d in range(3):
            a = np.asarray(arrs[d])
            if a.size == 0 or a.min() < 0 or a.max() >= nodes[d]:
                raise N.GomeltError(f"{what}: axis {d} indices [{a.min() if a.size else '-'}, "
                                    f"{a.max() if a.size else '-'}] outside [0, {nodes[d]})")
        return [C.cast(self.arena.put(a, np.int32), C.POINTER(C.c_int)) for a in arrs]

    # ------------------------------------------------------------------
    # per-window tables (rebuilt after every move)
    # ------------------------------------------------------------------
    def build_tables(self, assign=True):
        own = not self.arena.open
        if own:
            self.arena.begin()
        g = self.geo
        L1, L2, L3 = g.L[1], g.L[2], g.L[3]
        t = {}
        t["bc12"] = self._map(L1.coords, L1.nodes, L2.coords)  # Level 1 -> Level 2 nodes (LInterp[0])
        t["bc23"] = self._map(L2.coords, L2.nodes, L3.coords)  # Level 2 -> Level 3 nodes (LInterp[1])
        t["r32"] = self._map(L3.coords, L3.nodes, L3.overlap_coords)  # Level 3 at Level-2 overlap nodes
        t["r21"] = self._map(L2.coords, L2.nodes, L2.overlap_coords)  # Level 2 at Level-1 overlap nodes
        t["r32_idx"] = self._idx_tensor(L3.overlap_nodes, L2.nodes, "Level-3 overlap in Level 2")
        t["r21_idx"] = self._idx_tensor(L2.overlap_nodes, L1.nodes, "Level-2 overlap in Level 1")
        t["inj32"] = self._inject(L3.coords, L3.nodes, L3.overlap_coords, L3.overlap_nodes, L2.coords)
        t["inj21"] = self._inject(L2.coords, L2.nodes, L2.overlap_coords, L2.overlap_nodes, L1.coords)
        t["c32"] = CoupleGeom(L3.coords, L2.coords, self.np_dtype, self.arena)
        t["c31"] = CoupleGeom(L3.coords, L1.coords, self.np_dtype, self.arena)
        t["c21"] = CoupleGeom(L2.coords, L1.coords, self.np_dtype, self.arena)
        t["l0_3"] = self._idx_tensor(g.L0_overlap, g.L0_nodes, "Level-3 window in Level 0")
        t["l0_2"] = self._idx_tensor(g.L0_overlap_L2, g.L0_nodes, "Level-2 window in Level 0")
        c31, c21 = t["c31"], t["c21"]
        for d in range(3):
            if c31.box_lo[d] < c21.box_lo[d] or c31.box_lo[d] + c31.box_n[d] > c21.box_lo[d] + c21.box_n[d]:
                raise N.GomeltError("Level-3 window reaches outside Level 2's footprint in Level 1")
        if assign:
            self.tables = t
        nmax = max(t["c32"].partials, t["c31"].partials, t["c21"].partials)
        self._buf("partials", nmax)
        if own:
            self.arena.upload(self.stream)
        return t

    # ------------------------------------------------------------------
    # moveEverything (:2400-2510)
    # ------------------------------------------------------------------
    def plan_move(self, v, vstart):
        """Host half of move(): the new window positions, the remap maps and
        the per-window tables, staged in the table arena's next pinned buffer.
        It needs no device state, so a driver can plan move i+1 while move i
        and its subcycle run on the device, then apply it with
        ``move(v, vstart, plan)``.  Plan only after the previous move's
        subcycle (or step) has been issued: planning moves the host geometry.
        At most one plan is outstanding."""
        if self._pending is not None:
            raise N.GomeltError("a planned move is still pending")
        g = self.geo
        L1, L2, L3 = g.L[1], g.L[2], g.L[3]
        old3 = [c.copy() for c in L3.coords]
        old2 = [c.copy() for c in L2.coords]
        new3, new2, move_v = g.move(v, vstart)
        self.arena.begin()
        m3 = [self._map(L1.coords, L1.nodes, new3), self._map(old2, L2.nodes, new3), self._map(old3, L3.nodes, new3)]
        m2 = [self._map(L1.coords, L1.nodes, new2), self._map(old2, L2.nodes, new2)]
        L3.coords = new3
        L2.coords = new2
        t = self.build_tables(assign=False)
        self._pending = MovePlan(np.array(v, dtype=np.float64), move_v, m3, m2, t, self.arena.off)
        return self._pending

    def move(self, v, vstart, plan=None):
        """moveEverything: apply ``plan`` (from plan_move for the same v), or
        plan and apply now.  Enqueues one table upload and the remap kernels."""
        if plan is None:
            plan = self.plan_move(v, vstart)
        elif plan is not self._pending or not np.array_equal(plan.v, np.asarray(v, dtype=np.float64)):
            raise N.GomeltError("move(): plan is not the pending plan for this laser position")
        self._pending = None
        g = self.geo
        L2, L3 = g.L[2], g.L[3]
        n3, n2 = L3.nodes, L2.nodes
        m3, m2, t, move_v = plan.m3, plan.m2, plan.tables, plan.move_v
        self.tables = t
        self.last_table_bytes = plan.table_bytes
        self.arena.upload(self.stream)
        # Level 3: T = I_L1(T1) + I_L2(T'2) + I_L3old(T'3); T'3 = I_L3old(T'3)
        T3n = self._buf("mvT3", L3.nn)
        Tp3n = self._buf("mvTp3", L3.nn)
        self._interp([(m3[0], self.T[1], 1.0), (m3[1], self.Tp[2], 1.0), (m3[2], self.Tp[3], 1.0)], n3, T3n,
                     out_term=Tp3n, which=2)
        # Level 2: T'2 = I_L2old(T'2); T = I_L1(T1) + T'2
        T2n = self._buf("mvT2", L2.nn)
        Tp2n = self._buf("mvTp2", L2.nn)
        self._interp([(m2[0], self.T[1], 1.0), (m2[1], self.Tp[2], 1.0)], n2, T2n, out_term=Tp2n, which=1)
        self.T[3], T3n = T3n, self.T[3]
        self.Tp[3], Tp3n = Tp3n, self.Tp[3]
        self.T[2], T2n = T2n, self.T[2]
        self.Tp[2], Tp2n = Tp2n, self.Tp[2]
        self._work["mvT3"], self._work["mvTp3"], self._work["mvT2"], self._work["mvTp2"] = T3n, Tp3n, T2n, Tp2n
        # Level-0 gather of the window phases (:2500-2502)
        ph3n = self._buf("mvph3", L3.nn, torch.uint8)
        self._l0_gather(t["l0_3"], n3, ph3n, self.ph[3] if self.s2_prev_lo is not None else None, self.s2_prev_lo,
                        n3)
        self.ph[3], self._work["mvph3"] = ph3n, self.ph[3]
        self._l0_gather(t["l0_2"], n2, self.ph[2], None, None, None)
        return move_v

    def autotune(self, row, reps=5):
        """Measure the launch shape (kernel, tile, z-chunk) of the Level-3,
        Level-2 and Level-1 steps as the subcycle issues them
        (gm_level_autotune); later level steps of the same shapes use the
        fastest.  Needs the tables of a move; writes only scratch outputs;
        synchronises the stream.  Returns {level: kern.TunedShape}, the
        Level-3 step with the melt-time update under "3acc" and, for a
        constant-property material, the two-step kernel (gm_level_step2)
        under "3pair" / "3pair_acc"; the subcycle then takes its Level-3 steps
        two at a time if that measured faster per step (use_pairs)."""
        g = self.geo
        t = self.tables
        if t is None:
            raise N.GomeltError("autotune needs a move first")
        rowd = torch.as_tensor(np.asarray(row, dtype=np.float64), device=self.dev)
        out = {}
        for lev in (3, 2, 1):
            L = g.L[lev]
            To = self._buf(f"tuneT{lev}", L.nn)
            Po = self._buf(f"tunePh{lev}", L.nn, torch.uint8)
            if lev == 3:
                kw = self.level_kwargs(3, self.T[3], To, rowd[5:6], self.ph[3], Po, laser=rowd,
                                       ring=self._ring(3, self.T[2], self.T[2]), alpha=0.5)
                tab = None
                if N.props_constant(self.ps):  # the subcycle's Level-3 steps read tabulated laser factors
                    nl = int(sum(L.nodes))
                    tab = self._buf("tuneTab", 2 * nl)
                    rows2 = torch.stack([rowd, rowd])
                    N.call("gm_fine_source_tables", kern.dtype_code(self.T[3]), (C.c_int * 3)(*L.nodes),
                           (C.c_double * 3)(*L.origin()), (C.c_double * 3)(*L.spacing()), rows2.data_ptr(), 2,
                           C.byref(self.ps), tab.data_ptr(), kern.stream_ptr(self.stream))
                    kw["src_tab"] = tab[:nl]
            else:
                cg = t["c32"] if lev == 2 else t["c21"]
                box = [v for d in range(3) for v in (cg.box_lo[d], cg.box_lo[d] + cg.box_n[d])]
                rhs = self._buf("rhs2" if lev == 2 else "rhs1", int(np.prod(cg.box_n)))
                extra = dict(ring=self._ring(2, self.T[1], self.T[1]), alpha=0.5) if lev == 2 else {}
                # the subcycle's Level-1 steps keep the phase (no phase output)
                kw = self.level_kwargs(lev, self.T[lev], To, rowd[5:6], self.ph[lev], Po if lev == 2 else None,
                                       rhs=rhs, box=box, **extra)
            out[lev] = kern.level_autotune(self.ps, reps=reps, stream=self.stream, **kw)
            if lev == 3:  # the corrector's step with the melt-time update, on scratch accumulators
                acc = self._buf("tuneAcc", L.nn)
                macc = self._buf("tuneMacc", L.nn)
                with torch.cuda.stream(self.stream):
                    acc.zero_()
                    macc.zero_()
                kw.update(accum=acc, max_accum=macc)
                out["3acc"] = kern.level_autotune(self.ps, reps=reps, stream=self.stream, **kw)
                if tab is not None and L.nodes[2] >= 3:
                    # the two-step kernel (the subcycle's paired steps), with and without melt time
                    kw2 = dict(kw)
                    two = dict(dt2=rowd[5:6], src_tab2=tab[nl:], bc_alpha2=0.6, bc_beta2=0.4)
                    out["3pair_acc"] = kern.level_autotune2(self.ps, reps=reps, stream=self.stream, **two, **kw2)
                    kw2.pop("accum")
                    kw2.pop("max_accum")
                    out["3pair"] = kern.level_autotune2(self.ps, reps=reps, stream=self.stream, **two, **kw2)
                    self.use_pairs = out["3pair"].us + out["3pair_acc"].us < 2.0 * (out[3].us + out["3acc"].us)
        return out

    def _l0_gather(self, idx, n, ph_out, prev_ph, prev_lo, prev_n):
        a = N.gm_l0_args()
        for d in range(3):
            a.n[d] = int(n[d])
            a.idx[d] = idx[d]
        a.l0_nx, a.l0_ny = self.geo.L0_nodes[0], self.geo.L0_nodes[1]
        a.l0_bits = self.L0.data_ptr()
        a.ph = C.cast(ph_out.data_ptr(), C.POINTER(C.c_uint8))
        if prev_ph is not None:
            a.prev_ph = C.cast(prev_ph.data_ptr(), C.POINTER(C.c_uint8))
            for d in range(3):
                a.prev_lo[d] = int(prev_lo[d])
                a.prev_n[d] = int(prev_n[d])
        N.call("gm_l0_gather", C.byref(a), kern.stream_ptr(self.stream))

    def l0_scatter(self):
        g = self.geo
        idx = self.tables["l0_3"]
        a = N.gm_l0_args()
        for d in range(3):
            a.n[d] = g.L[3].nodes[d]
            a.idx[d] = idx[d]
        a.l0_nx, a.l0_ny = g.L0_nodes[0], g.L0_nodes[1]
        a.l0_bits = self.L0.data_ptr()
        a.ph = C.cast(self.ph[3].data_ptr(), C.POINTER(C.c_uint8))
        N.call("gm_l0_scatter", C.byref(a), kern.stream_ptr(self.stream))
        self.s2_prev_lo = [int(np.asarray(g.L0_overlap[d])[0]) for d in range(3)]

    # ------------------------------------------------------------------
    # building blocks
    # ------------------------------------------------------------------
    def _ring(self, lev, A, B):
        """Prolongate the coarse fields A and B onto the Dirichlet ring of
        level `lev` (gm_ring_prolong); returns the two ring arrays that a
        `_level(..., ring=...)` call blends."""
        L = self.geo.L[lev]
        outA, outB = self._buf(f"ring{lev}a", L.nn), self._buf(f"ring{lev}b", L.nn)
        a = N.gm_ring_args()
        a.dtype = kern.dtype_code(A)
        for d in range(3):
            a.nodes[d] = L.nodes[d]
        a.map = (self.tables["bc12"] if lev == 2 else self.tables["bc23"]).struct
        a.srcA, a.srcB = kern.ptr(A), kern.ptr(B)
        a.outA, a.outB = kern.ptr(outA), kern.ptr(outB)
        N.call("gm_ring_prolong", C.byref(a), kern.stream_ptr(self.stream))
        return outA, outB

    def _level(self, lev, T_in, T_out, dt, ph_in, ph_out, **kw):
        kern.level_step(self.ps, stream=self.stream, **self.level_kwargs(lev, T_in, T_out, dt, ph_in, ph_out, **kw))

    def level_kwargs(self, lev, T_in, T_out, dt, ph_in, ph_out, *, rhs=None, box=None, laser=None, bc_new=None,
                     bc_old=None, alpha=0.0, accum=False, clamp=True, ring=None):
        """Arguments of kern.level_args for one level step of level `lev`."""
        g = self.geo
        L = g.L[lev]
        kw = {}
        if lev == 1:
            ne_planes = self.tmp[0] // (L.elements[0] * L.elements[1])
            c = g.conditions
            kw.update(bc_mode=1, face=[c["x"][0], c["x"][1], c["y"][0], c["y"][1], c["z"][0]], inactive_amb=1)
        elif ring is not None:
            ne_planes = L.elements[2]
            kw.update(bc_mode=3, bc_new=ring[0], bc_old=ring[1], bc_alpha=alpha, bc_beta=1.0 - alpha)
        else:
            ne_planes = L.elements[2]
            m = self.tables["bc12"] if lev == 2 else self.tables["bc23"]
            kw.update(bc_mode=2, bc_new=bc_new, bc_old=bc_old, bc_alpha=alpha, bc_beta=1.0 - alpha, bc_map=m)
        if accum:
            kw.update(accum=self.acc3, max_accum=self.macc3)
        return dict(T_in=T_in, T_out=T_out, nodes=L.nodes, h=L.spacing(), origin=L.origin(), ne_planes=ne_planes,
                    dt=dt, ph_in=ph_in, ph_out=ph_out, substrate=self.substrate[lev], rhs_box=rhs, box=box,
                    laser=laser, surface=1, clamp=1 if clamp else 0, **kw)

    def _couple(self, cg, fine_lev, out, out_lo, out_n, *, T, ph, Tp=None, dTa=None, dTb=None, dt=None):
        g = self.geo
        L = g.L[fine_lev]
        a = N.gm_couple_args()
        a.dtype = kern.dtype_code(out)
        a.geom = cg.struct
        for d in range(3):
            a.fine_nodes[d] = L.nodes[d]
            a.fine_h[d] = L.spacing()[d]
            a.out_lo[d] = int(out_lo[d])
            a.out_n[d] = int(out_n[d])
        a.T = kern.ptr(T)
        a.ph = C.cast(ph.data_ptr(), C.POINTER(C.c_uint8))
        a.substrate = self.substrate[fine_lev]
        a.Tp = kern.ptr(Tp)
        a.dTa, a.dTb = kern.ptr(dTa), kern.ptr(dTb)
        a.dt = kern.ptr(dt)
        a.out = kern.ptr(out)
        a.scale = 1.0
        part = self._work["partials"]
        a.partials = part.data_ptr()
        a.partials_cap = part.numel()
        N.call("gm_couple", C.byref(a), C.byref(self.ps), kern.stream_ptr(self.stream))

    def _coarse_source(self, cg, rows, npos, out, out_lo, out_n):
        L3 = self.geo.L[3]
        a = N.gm_coarse_source_args()
        a.dtype = kern.dtype_code(out)
        a.geom = cg.struct
        a.npos = int(npos)
        a.rows = kern.ptr(rows)
        for d in range(3):
            a.xq[d] = C.cast(cg.axes[d]["xq"], C.POINTER(C.c_double))
            a.out_lo[d] = int(out_lo[d])
            a.out_n[d] = int(out_n[d])
        h = L3.spacing()
        a.fine_wq = h[0] * h[1] * h[2] / 8.0
        a.out = kern.ptr(out)
        per = sum(cg.box_n)
        scr = self._buf("srcscratch", npos * per)
        a.scratch = scr.data_ptr()
        a.scratch_cap = scr.numel()
        N.call("gm_coarse_source", C.byref(a), C.byref(self.ps), kern.stream_ptr(self.stream))

    def _restrict(self, rmap, idx, coarse_nodes, fine_T, coarse_T):
        a = N.gm_restrict_args()
        a.dtype = kern.dtype_code(fine_T)
        for d in range(3):
            a.n[d] = rmap.n[d]
            a.cidx[d] = idx[d]
        a.map = rmap.struct
        a.cnx, a.cny = coarse_nodes[0], coarse_nodes[1]
        a.fine = kern.ptr(fine_T)
        a.coarse = kern.ptr(coarse_T)
        N.call("gm_restrict", C.byref(a), kern.stream_ptr(self.stream))

    def _new_tprime(self, fine_lev, fine_T, coarse_T, out_Tp, fused=True):
        """getNewTprime (:2060-2099): restrict into coarse_T, then T' = T_f - I(T_c)
        (one gm_tprime_inject launch where the restriction is an injection,
        unless fused is False)."""
        g = self.geo
        if fine_lev == 3:
            rmap, idx, cmap, cn = self.tables["r32"], self.tables["r32_idx"], self.tables["bc23"], g.L[2].nodes
            inj = self.tables.get("inj32")
        else:
            rmap, idx, cmap, cn = self.tables["r21"], self.tables["r21_idx"], self.tables["bc12"], g.L[1].nodes
            inj = self.tables.get("inj21")
        if fused and inj is not None:
            a = N.gm_tprime_args()
            a.dtype = kern.dtype_code(fine_T)
            for d in range(3):
                a.n[d] = int(g.L[fine_lev].nodes[d])
                a.cf0[d], a.cf1[d], a.c_of_f[d] = inj[d], inj[3 + d], inj[6 + d]
            a.cmap = cmap.struct
            a.cnx, a.cny = int(cn[0]), int(cn[1])
            a.fine, a.coarse, a.out = kern.ptr(fine_T), kern.ptr(coarse_T), kern.ptr(out_Tp)
            N.call("gm_tprime_inject", C.byref(a), kern.stream_ptr(self.stream))
            return
        self._restrict(rmap, idx, cn, fine_T, coarse_T)
        self._interp([(cmap, coarse_T, -1.0)], g.L[fine_lev].nodes, out_Tp, base=fine_T)

    def _s1_restrict(self):
        g = self.geo
        a = N.gm_restrict_s1_args()
        a.dtype = kern.dtype_code(self.T[1])
        rmap, idx = self.tables["r21"], self.tables["r21_idx"]
        for d in range(3):
            a.n[d] = rmap.n[d]
            a.cidx[d] = idx[d]
        a.map = rmap.struct
        a.cnx, a.cny = g.L[1].nodes[0], g.L[1].nodes[1]
        a.fine_ph = C.cast(self.ph[2].data_ptr(), C.POINTER(C.c_uint8))
        a.coarse_ph = C.cast(self.ph[1].data_ptr(), C.POINTER(C.c_uint8))
        a.substrate = self.substrate[1]
        N.call("gm_restrict_s1", C.byref(a), kern.stream_ptr(self.stream))

    # ------------------------------------------------------------------
    # subcycleGOMELT (:3224-3632)
    # ------------------------------------------------------------------
    def subcycle(self, laser_rows, history=False, rows_device=None, dts_device=None):
        """One subcycleGOMELT call, issued natively (gm_subcycle).  laser_rows:
        N2*N3 host rows (x, y, z, jump, dwell, dt, P); rows_device: the same
        rows already on the device; dts_device: also their step dts on the
        device (step_dts; with rows_device, e.g. from a DeviceToolpath, no
        host-to-device copy at all; laser_rows may then be None).  Returns
        (L2all, L3all, L3pall) device tensors when ``history``, else None."""
        g = self.geo
        L1, L2, L3 = g.L[1], g.L[2], g.L[3]
        N2, N3 = self.N2, self.N3
        if self.tmp is None:
            raise N.GomeltError("active Level-1 region not set (call set_layer first)")
        if dts_device is not None:
            if rows_device is None or rows_device.numel() < 7 * N2 * N3 or dts_device.numel() < N2 + 1:
                raise N.GomeltError("device dts need the chunk's device rows")
            rows, dtd = kern.ptr(rows_device), kern.ptr(dts_device)
        else:
            rows_h = np.ascontiguousarray(np.asarray(laser_rows, dtype=np.float64))
            if rows_h.shape != (N2 * N3, 7):
                raise N.GomeltError(f"expected {N2 * N3} laser rows of 7 values, got {rows_h.shape}")
            dts = step_dts(rows_h, N2)
            need = 8 * (rows_h.size + dts.size) + 2 * TableArena.ALIGN
            if need > self.rarena.nbytes:
                self.rarena = TableArena(2 * need, self.dev)
            self.rarena.begin()
            rows = rows_device.data_ptr() if rows_device is not None else self.rarena.put(rows_h, np.float64)
            dtd = self.rarena.put(dts, np.float64)
            self.rarena.upload(self.stream)
        out_hist = None
        if history:
            out_hist = (torch.empty(N2, L2.nn, dtype=self.dtype, device=self.dev),
                        torch.empty(N2, L3.nn, dtype=self.dtype, device=self.dev),
                        torch.empty(N2, L3.nn, dtype=self.dtype, device=self.dev))
        p = self._plan(rows, dtd, out_hist)
        if getattr(self, "_batch_plan", False):  # subcycle_batched collects the plan instead
            self._last_plan = p
            return out_hist
        N.call("gm_subcycle", C.byref(p), C.byref(self.ps), kern.stream_ptr(self.stream),
               kernels=N.subcycle_kernel_count(N2, N3, N.props_constant(self.ps), persist=bool(p.persist),
                                              inject32=bool(p.inj32[0]), inject21=bool(p.inj21[0]),
                                              pairs=self.pairs_active(p)))
        self.s2_prev_lo = [int(np.asarray(g.L0_overlap[d])[0]) for d in range(3)]
        return out_hist

    def _window(self, lev):
        L = self.geo.L[lev]
        w = N.gm_window()
        for d in range(3):
            w.nodes[d] = L.nodes[d]
            w.h[d] = L.spacing()[d]
            w.origin[d] = L.origin()[d]
        w.substrate = self.substrate[lev]
        w.T = self.T[lev].data_ptr()
        w.Tp = self.Tp[lev].data_ptr() if lev > 1 else None
        w.ph = C.cast(self.ph[lev].data_ptr(), C.POINTER(C.c_uint8))
        return w

    def _plan(self, rows, dtd, out_hist):
        g = self.geo
        L1, L2, L3 = g.L[1], g.L[2], g.L[3]
        N2, N3 = self.N2, self.N3
        tb = self.tables
        c32, c31, c21 = tb["c32"], tb["c31"], tb["c21"]
        nn1, nn2, nn3 = L1.nn, L2.nn, L3.nn
        u8 = torch.uint8
        pu = lambda t: C.cast(t.data_ptr(), C.POINTER(C.c_uint8))  # noqa: E731
        p = N.gm_subcycle_plan()
        p.dtype = kern.dtype_code(self.T[3])
        p.N2, p.N3 = N2, N3
        p.L1, p.L2, p.L3 = self._window(1), self._window(2), self._window(3)
        p.L1_ne_planes = self.tmp[0] // (L1.elements[0] * L1.elements[1])
        c = g.conditions
        for i, v in enumerate((c["x"][0], c["x"][1], c["y"][0], c["y"][1], c["z"][0])):
            p.face[i] = float(v)
        p.acc3, p.macc3 = self.acc3.data_ptr(), self.macc3.data_ptr()
        p.bc12, p.bc23, p.r32, p.r21 = tb["bc12"].struct, tb["bc23"].struct, tb["r32"].struct, tb["r21"].struct
        for q in range(9):
            if tb.get("inj32") is not None:
                p.inj32[q] = tb["inj32"][q]
            if tb.get("inj21") is not None:
                p.inj21[q] = tb["inj21"][q]
        for d in range(3):
            p.r32_idx[d] = tb["r32_idx"][d]
            p.r21_idx[d] = tb["r21_idx"][d]
            p.xq32[d] = C.cast(c32.axes[d]["xq"], C.POINTER(C.c_double))
            p.xq31[d] = C.cast(c31.axes[d]["xq"], C.POINTER(C.c_double))
            p.rhs1_lo[d], p.rhs1_n[d] = c21.box_lo[d], c21.box_n[d]
            p.rhs2_lo[d], p.rhs2_n[d] = c32.box_lo[d], c32.box_n[d]
            p.l0_idx3[d] = tb["l0_3"][d]
        p.c32, p.c31, p.c21 = c32.struct, c31.struct, c21.struct
        p.L0 = self.L0.data_ptr()
        p.L0_nx, p.L0_ny = g.L0_nodes[0], g.L0_nodes[1]
        p.rows, p.dts = rows, dtd
        p.T1p, p.T1c = self._buf("T1p", nn1).data_ptr(), self._buf("T1c", nn1).data_ptr()
        p.T2w[0], p.T2w[1] = self._buf("T2a", nn2).data_ptr(), self._buf("T2b", nn2).data_ptr()
        p.T3w[0], p.T3w[1] = self._buf("T3a", nn3).data_ptr(), self._buf("T3b", nn3).data_ptr()
        p.tp3w[0], p.tp3w[1] = self._buf("tp3w0", nn3).data_ptr(), self._buf("tp3w1", nn3).data_ptr()
        p.Tp2w = self._buf("Tp2w", nn2).data_ptr()
        p.rhs1 = self._buf("rhs1", int(np.prod(c21.box_n))).data_ptr()
        p.rhs2 = self._buf("rhs2", int(np.prod(c32.box_n))).data_ptr()
        p.tp3hist = self._buf("tp3hist", N2 * nn3).data_ptr()
        p.ph2w[0], p.ph2w[1] = pu(self._buf("ph2a", nn2, u8)), pu(self._buf("ph2b", nn2, u8))
        p.ph3w[0], p.ph3w[1] = pu(self._buf("ph3a", nn3, u8)), pu(self._buf("ph3b", nn3, u8))
        part = self._work["partials"]
        p.partials, p.partials_cap = part.data_ptr(), part.numel()
        ns = N2 * N3 * max(sum(c31.box_n), sum(c32.box_n))
        scr = self._buf("srcscratch", ns)
        p.src_scratch, p.src_cap = scr.data_ptr(), scr.numel()
        p.src2 = self._buf("src2", N2 * int(np.prod(c32.box_n))).data_ptr()
        if out_hist is not None:
            p.L2all, p.L3all, p.L3pall = (t.data_ptr() for t in out_hist)
        p.zchunk = int(getattr(self, "zchunk", 0))
        p.ring2[0], p.ring2[1] = self._buf("ring2a", nn2).data_ptr(), self._buf("ring2b", nn2).data_ptr()
        p.ring3[0], p.ring3[1] = self._buf("ring3a", nn3).data_ptr(), self._buf("ring3b", nn3).data_ptr()
        p.graph = 1 if self.use_graph else 0
        p.pdl = 1 if self.use_pdl else 0
        if N.props_constant(self.ps):  # the separable Level-3 step reads tabulated laser factors
            p.src3tab = self._buf("src3tab", N2 * N3 * int(sum(L3.nodes))).data_ptr()
            mode = int(self.use_persist)
            nf = 0
            if mode == 1 and self.persist_shape() is not None:
                nf = int(N.lib().gm_level3_persist_flags((C.c_int * 3)(*L3.nodes)))
            elif mode == 2:
                nf = 2 * N2  # a grid-barrier counter per launch
            if nf > 0:
                p.persist = mode
                p.xch3[0], p.xch3[1] = self._buf("xch3a", nn3).data_ptr(), self._buf("xch3b", nn3).data_ptr()
                p.pflags, p.pflags_cap = self._buf("pflags", nf, torch.int32).data_ptr(), nf
            p.l3_pairs = 1 if (self.use_pairs and not p.persist) else 0
        p.pstatus = self.status.data_ptr()  # every level step reports non-finite / out-of-range values here
        return p

    def pairs_active(self, p) -> bool:
        """Whether gm_subcycle takes the Level-3 steps of plan p two at a
        time (its own condition: constant properties, the factor table, no
        persistent steps, at least three node planes)."""
        return bool(p.l3_pairs and not p.persist and p.src3tab and self.geo.L[3].nodes[2] >= 3)

    def persist_shape(self):
        """Tile shape of the persistent Level-3 kernel on this window ({tiles,
        x columns, y rows, z segments}), or None if the window has none."""
        out = (C.c_int * 4)()
        rc = N.lib().gm_level3_persist_shape(kern.dtype_code(self.T[3]), (C.c_int * 3)(*self.geo.L[3].nodes), out)
        return list(out) if rc == N.GM_OK else None

    def check_status(self):
        """Raise GomeltError if a device kernel reported a failure (a bounded
        wait that ran out, a non-finite or out-of-range Level-3 field); reading
        the status synchronises with the engine's stream.  The word is cleared."""
        v = int(self.status.item())
        if v:
            with torch.cuda.stream(self.stream or torch.cuda.current_stream()):
                self.status.zero_()
            what = []
            if v & N.GM_PERSIST_TIMEOUT:
                what.append("a wait between Level-3 tiles ran out")
            if v & N.GM_STATUS_BAD_T:
                what.append("non-finite or out-of-range temperature (above 1e5 K) from a level step")
            raise N.GomeltError("device status: " + ", ".join(what or [f"code {v}"]))

    # ------------------------------------------------------------------
    # stepGOMELT (:2304-2397) and stepGOMELTDwellTime (:2617-2664)
    # ------------------------------------------------------------------
    def _state_props(self, lev, T, ph_in, ph_out):
        a = N.gm_state_props_args()
        a.dtype = kern.dtype_code(T)
        a.n = T.numel()
        a.T = kern.ptr(T)
        a.ph_in = C.cast(ph_in.data_ptr(), C.POINTER(C.c_uint8))
        a.ph_out = C.cast(ph_out.data_ptr(), C.POINTER(C.c_uint8))
        a.substrate = self.substrate[lev]
        N.call("gm_state_properties", C.byref(a), C.byref(self.ps), kern.stream_ptr(self.stream))

    def _clamp(self, T):
        N.call("gm_clamp_min", kern.dtype_code(T), kern.ptr(T), C.c_longlong(T.numel()),
               C.c_double(float(self.P["T_amb"])), kern.stream_ptr(self.stream))

    def step(self, v):
        """One equal-dt step of all levels, predictor + corrector.  v: laser row
        (x, y, z, ..., dt at [5], P at [6]).  Returns the newly-melted mask of
        Level 3 (the reference's resetmask) as a device bool tensor."""
        g = self.geo
        L1, L2, L3 = g.L[1], g.L[2], g.L[3]
        if self.tmp is None:
            raise N.GomeltError("active Level-1 region not set (call set_layer first)")
        row = self._buf("steprow", 7, torch.float64)
        row.copy_(torch.as_tensor(np.asarray(v, dtype=np.float64)[:7]))
        dtd = row[5:6]
        tb = self.tables
        c32, c31, c21 = tb["c32"], tb["c31"], tb["c21"]
        T1s, T2s, T3s = self.T[1], self.T[2], self.T[3]
        Tp2s, Tp3s = self.Tp[2], self.Tp[3]
        ph1, ph2s, ph3s = self.ph[1], self.ph[2], self.ph[3]
        nn1, nn2, nn3 = L1.nn, L2.nn, L3.nn
        pre3 = self._buf("pre_ph3", nn3, torch.uint8)
        pre3.copy_(ph3s)
        # updateStateProperties (:2513-2564)
        phn = self._buf("stph3", nn3, torch.uint8)
        self._state_props(3, T3s, ph3s, phn)
        ph3s.copy_(phn)
        phn2 = self._buf("stph2", nn2, torch.uint8)
        self._state_props(2, T2s, ph2s, phn2)
        ph2s.copy_(phn2)
        self._s1_restrict()
        # sources (computeSources :928-988) and subgrid flux terms (:1477-1565)
        rhs1 = self._buf("rhs1", int(np.prod(c21.box_n)))
        rhs2 = self._buf("rhs2", int(np.prod(c32.box_n)))
        rhs1.zero_()
        rhs2.zero_()
        self._coarse_source(c31, row, 1, rhs1, c21.box_lo, c21.box_n)
        self._coarse_source(c32, row, 1, rhs2, c32.box_lo, c32.box_n)
        self._couple(c31, 3, rhs1, c21.box_lo, c21.box_n, T=T3s, ph=ph3s, Tp=Tp3s)
        self._couple(c21, 2, rhs1, c21.box_lo, c21.box_n, T=T2s, ph=ph2s, Tp=Tp2s)
        self._couple(c32, 3, rhs2, c32.box_lo, c32.box_n, T=T3s, ph=ph3s, Tp=Tp3s)
        box1 = [c21.box_lo[0], c21.box_lo[0] + c21.box_n[0], c21.box_lo[1], c21.box_lo[1] + c21.box_n[1],
                c21.box_lo[2], c21.box_lo[2] + c21.box_n[2]]
        box2 = [c32.box_lo[0], c32.box_lo[0] + c32.box_n[0], c32.box_lo[1], c32.box_lo[1] + c32.box_n[1],
                c32.box_lo[2], c32.box_lo[2] + c32.box_n[2]]

        def solutions(T1o, T2o, T3o):
            # computeSolutions (:2135-2204): the coarse results feed the finer
            # Dirichlet rings before the T >= T_amb clamp
            self._level(1, T1s, T1o, dtd, ph1, None, rhs=rhs1, box=box1, clamp=False)
            self._level(2, T2s, T2o, dtd, ph2s, None, rhs=rhs2, box=box2, bc_new=T1o, bc_old=T1o, alpha=1.0,
                        clamp=False)
            self._level(3, T3s, T3o, dtd, ph3s, None, laser=row, bc_new=T2o, bc_old=T2o, alpha=1.0, clamp=False)
            for T in (T1o, T2o, T3o):
                self._clamp(T)

        T1p, T2p, T3p = self._buf("T1p", nn1), self._buf("T2a", nn2), self._buf("T3a", nn3)
        solutions(T1p, T2p, T3p)
        Tp3n, Tp2n = self._buf("tp3w0", nn3), self._buf("Tp2w", nn2)
        self._new_tprime(3, T3p, T2p, Tp3n)
        self._new_tprime(2, T2p, T1p, Tp2n)
        # mass terms (:1396-1474)
        self._couple(c31, 3, rhs1, c21.box_lo, c21.box_n, T=T3s, ph=ph3s, dTa=Tp3n, dTb=Tp3s, dt=dtd)
        self._couple(c21, 2, rhs1, c21.box_lo, c21.box_n, T=T2s, ph=ph2s, dTa=Tp2n, dTb=Tp2s, dt=dtd)
        self._couple(c32, 3, rhs2, c32.box_lo, c32.box_n, T=T3s, ph=ph3s, dTa=Tp3n, dTb=Tp3s, dt=dtd)
        T1c, T2c, T3c = self._buf("T1c", nn1), self._buf("T2b", nn2), self._buf("T3b", nn3)
        solutions(T1c, T2c, T3c)
        self._new_tprime(3, T3c, T2c, Tp3s)
        self._new_tprime(2, T2c, T1c, Tp2s)
        T3s.copy_(T3c)
        T2s.copy_(T2c)
        T1s.copy_(T1c)
        self.l0_scatter()
        return ((ph3s & PH_S2) != 0) & ((pre3 & PH_S2) == 0)

    def dwell(self, dt):
        """Level 1 only, surface flux, no source, no clamp (stepGOMELTDwellTime)."""
        if self.tmp is None:
            raise N.GomeltError("active Level-1 region not set (call set_layer first)")
        dtd = self._buf("dwelldt", 1, torch.float64)
        dtd.fill_(float(dt))
        T1w = self._buf("T1p", self.geo.L[1].nn)
        self._level(1, self.T[1], T1w, dtd, self.ph[1], None, clamp=False)
        self.T[1].copy_(T1w)

    # ------------------------------------------------------------------
    # state set-up
    # ------------------------------------------------------------------
    def set_layer(self, v):
        """Active Level-1 region and substrate counts for the layer at v[2]."""
        self.tmp = self.geo.tmp_ne_nn(v)
        self.substrate = self.geo.substrate()

    def load_levels(self, Levels):
        """Adopt a reference-layout ``Levels`` list (host arrays): window
        positions, overlap sets, fields, phases and the Level-0 store."""
        g = self.geo
        f = dict(dtype=self.dtype, device=self.dev)
        for lev in (1, 2, 3):
            Ld = Levels[lev]
            g.L[lev].coords = [np.asarray(c, dtype=np.float64).copy() for c in Ld["node_coords"]]
            self.T[lev] = torch.as_tensor(np.asarray(Ld["T0"], dtype=np.float64), **f).contiguous()
            ph = (np.asarray(Ld["S1"], dtype=np.float64) > 0.499).astype(np.uint8)
            if "S2" in Ld:
                ph |= (np.asarray(Ld["S2"]).astype(bool).astype(np.uint8) << 1)
            self.ph[lev] = torch.as_tensor(ph, device=self.dev).contiguous()
            if lev > 1:
                self.Tp[lev] = torch.as_tensor(np.asarray(Ld["Tprime0"], dtype=np.float64), **f).contiguous()
                g.L[lev].overlap_nodes = [np.asarray(a).astype(np.int64) for a in Ld["overlapNodes"]]
                g.L[lev].overlap_coords = [np.asarray(a, dtype=np.float64) for a in Ld["overlapCoords"]]
        L0 = Levels[0]
        g.L0_overlap = [np.asarray(a).astype(np.int64) for a in L0["overlapNodes"]]
        g.L0_overlap_L2 = [np.asarray(a).astype(np.int64) for a in L0["overlapNodes_L2"]]
        g.L0_coords = [np.asarray(c, dtype=np.float64).copy() for c in L0["node_coords"]]
        self.L0 = l0_pack(torch.as_tensor(np.asarray(L0["S1"], dtype=np.float64), device=self.dev), g.L0_nodes)
        s2 = np.asarray(L0["S2"]).astype(bool)
        self.s2_prev_lo = [int(g.L0_overlap[d][0]) for d in range(3)] if s2.any() else None
        self.acc3 = torch.zeros(g.L[3].nn, **f)
        self.macc3 = torch.zeros(g.L[3].nn, **f)
        self.build_tables()

    def l0_s1(self):
        """Level-0 S1 as one uint8 (0/1) per node."""
        return l0_unpack(self.L0, self.geo.L0_nodes)

    def l0_fill(self, first, last, value):
        """Level-0 nodes [first, last) set to value (gm_l0_fill)."""
        n = self.geo.L0_nodes
        N.call("gm_l0_fill", self.L0.data_ptr(), int(n[0]), int(n[1]), int(n[2]), int(first), int(last),
               int(value), kern.stream_ptr(self.stream))

    def fields_numpy(self):
        """Host copies of the state in the reference's field names."""
        out = {}
        for lev in (1, 2, 3):
            ph = self.ph[lev].cpu().numpy()
            out[lev] = {"T0": self.T[lev].double().cpu().numpy(), "S1": (ph & PH_S1).astype(np.float64),
                        "S2": (ph & PH_S2) != 0}
            if lev > 1:
                out[lev]["Tprime0"] = self.Tp[lev].double().cpu().numpy()
        out[0] = {"S1": self.l0_s1().cpu().numpy().astype(np.float64)}
        return out


def subcycle_batched(engines, rows_list, rows_device=None, dts_device=None):
    """subcycleGOMELT of many independent engines (scan instances) as ONE CUDA
    graph (gm_subcycle_batched): each engine plans its call as Engine.subcycle
    does, then all calls are issued as parallel branches of one graph on the
    first engine's stream, which every engine must share.  The persistent
    Level-3 kernel is not used here (its cooperative launches are not
    co-scheduled across concurrent branches).  rows_list[i]: host rows of
    engine i (or None with rows_device[i] / dts_device[i])."""
    st = engines[0].stream
    if st is None or any(e.stream is not st for e in engines):
        raise N.GomeltError("batched engines must share one (non-default) stream")
    plans = (N.gm_subcycle_plan * len(engines))()
    props = (N.gm_props * len(engines))()
    kernels = 0
    for i, e in enumerate(engines):
        e._batch_plan = True
        keep = e.use_persist
        e.use_persist = 0
        try:
            e.subcycle(rows_list[i] if rows_list is not None else None,
                       rows_device=None if rows_device is None else rows_device[i],
                       dts_device=None if dts_device is None else dts_device[i])
        finally:
            e._batch_plan = False
            e.use_persist = keep
        plans[i] = e._last_plan
        props[i] = e.ps
        kernels += N.subcycle_kernel_count(e.N2, e.N3, N.props_constant(e.ps), inject32=bool(plans[i].inj32[0]),
                                           inject21=bool(plans[i].inj21[0]), pairs=e.pairs_active(plans[i]))
    N.call("gm_subcycle_batched", plans, len(engines), props, kern.stream_ptr(st), kernels=kernels)
    for e in engines:
        g = e.geo
        e.s2_prev_lo = [int(np.asarray(g.L0_overlap[d])[0]) for d in range(3)]
        e._last_plan = None



def failed_instances(engines):
    """Indices of the engines whose device status word is set (a level step
    produced a non-finite or out-of-range value, or a bounded wait ran out),
    read with ONE device-to-host copy for all of them; the words are cleared.
    The words are read on the first engine's stream."""
    st = engines[0].stream or torch.cuda.current_stream()
    with torch.cuda.stream(st):
        words = torch.stack([e.status[0] for e in engines])
        for e in engines:
            e.status.zero_()
    return [i for i, v in enumerate(words.cpu().tolist()) if v]
