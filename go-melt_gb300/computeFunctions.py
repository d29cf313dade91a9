"""GO-MELT's computeFunctions call surface on the GB300 engine.

Same function names, positional signatures and return tuples as the
reference module (JLnorthwestern/GO-MELT go_melt/computeFunctions.py) for the
multilevel thermal step and the functions its driver calls, so code written
against the reference (``from computeFunctions import *``) runs on the GPU:

* ``Levels`` is a list of four dict views over one ``Engine``: ``T0``,
  ``Tprime0``, ``S1``, ``S2`` are device tensors (S1/S2 are derived from the
  phase byte when read, stored back into it when assigned); the geometry keys
  (``node_coords``, ``nodes``, ``overlapNodes`` ...) are host arrays.
* ``Shapes`` (computeCoarseFineShapeFunctions) is an opaque handle: the
  coarse-at-fine tables are never materialised, the kernels evaluate them
  per axis.
* arrays passed to and returned from the compute functions are torch CUDA
  tensors (float32 or float64, as the engine).

Errors: a failing kernel call raises ``GomeltError`` (the reference has no
error returns); ``printLevelMaxMin`` keeps the reference's ``sys.exit(1)`` on
non-finite or out-of-range temperatures.
"""

from __future__ import annotations

import copy  # noqa: F401  (the reference driver uses copy via this module's namespace)
import ctypes as C
import json  # noqa: F401
import os
import pickle
import sys

import numpy as np
import torch

import _native as N
import kern
from _native import GomeltError  # noqa: F401
from createPath import count_lines, parsingGcode  # noqa: F401
from engine import PH_S1, PH_S2, CoupleGeom, Engine, TableArena
from geometry import axis_map
from levels import setup_nonmesh, setup_properties

# ---------------------------------------------------------------------------
# Levels views
# ---------------------------------------------------------------------------
_FIELD_KEYS = {"T0", "T", "Tprime0", "Tprime", "S1", "S2"}


class LevelView(dict):
    """Reference-layout dict of one level, backed by the engine."""

    def __init__(self, engine: Engine, lev: int):
        super().__init__()
        self.engine = engine
        self.lev = lev

    # -- fields ----------------------------------------------------------
    def _field(self, k):
        e, lv = self.engine, self.lev
        if lv == 0:
            if k == "S1":
                return e.l0_s1().to(e.dtype)
            if k == "S2":
                return self._l0_s2()
            raise KeyError(k)
        if k in ("T0", "T"):
            return e.T[lv]
        if k in ("Tprime0", "Tprime"):
            if lv == 1:
                raise KeyError(k)
            return e.Tp[lv]
        if k == "S1":
            return (e.ph[lv] & PH_S1).to(e.dtype)
        if k == "S2":
            return (e.ph[lv] & PH_S2) != 0
        raise KeyError(k)

    def _l0_s2(self):
        e = self.engine
        out = torch.zeros(e.geo.L0_nn, dtype=torch.bool, device=e.dev)
        if e.s2_prev_lo is not None:
            idx = _l0_index(e.geo.L0_nodes, [np.asarray(e.s2_prev_lo[d]) + np.arange(e.geo.L[3].nodes[d])
                                             for d in range(3)])
            out[torch.as_tensor(idx, device=e.dev)] = (e.ph[3] & PH_S2) != 0
        return out

    def _set_field(self, k, v):
        e, lv = self.engine, self.lev
        t = torch.as_tensor(v, device=e.dev)
        if lv == 0:
            if k == "S1":
                from engine import l0_pack

                e.L0.copy_(l0_pack(t.reshape(-1), e.geo.L0_nodes))
                return
            raise KeyError(f"Level 0 field {k} is not assignable")
        if k in ("T0", "T"):
            e.T[lv].copy_(t.reshape(-1))
        elif k in ("Tprime0", "Tprime"):
            e.Tp[lv].copy_(t.reshape(-1))
        elif k == "S1":
            b = (t.reshape(-1) > 0.499).to(torch.uint8)
            e.ph[lv].copy_((e.ph[lv] & PH_S2) | b)
        elif k == "S2":
            b = (t.reshape(-1).to(torch.bool)).to(torch.uint8) * PH_S2
            e.ph[lv].copy_((e.ph[lv] & PH_S1) | b)

    # -- geometry --------------------------------------------------------
    def _geom(self, k):
        g = self.engine.geo
        lv = self.lev
        if lv == 0:
            m = {"nodes": lambda: [np.array(x) for x in g.L0_nodes],
                 "nn": lambda: np.array(g.L0_nn),
                 "node_coords": lambda: g.L0_coords,
                 "overlapNodes": lambda: g.L0_overlap,
                 "overlapNodes_L2": lambda: g.L0_overlap_L2,
                 "idx": lambda: _l0_index(g.L0_nodes, g.L0_overlap),
                 "idx_L2": lambda: _l0_index(g.L0_nodes, g.L0_overlap_L2),
                 "layer_idx_delta": lambda: np.array(g.layer_idx_delta)}
        else:
            L = g.L[lv]
            m = {"nodes": lambda: [np.array(x) for x in L.nodes],
                 "elements": lambda: [np.array(x) for x in L.elements],
                 "h": lambda: [np.array(x) for x in L.h],
                 "length": lambda: [np.array(x) for x in L.length],
                 "nn": lambda: np.array(L.nn),
                 "ne": lambda: np.array(L.ne),
                 "node_coords": lambda: L.coords,
                 "bounds": lambda: L.bounds,
                 "BC": lambda: _bc_indices(L.nodes)}
            if lv == 1:
                m["conditions"] = lambda: g.conditions
                m["orig_node_coords"] = lambda: L.orig_coords
            else:
                m.update({"overlapNodes": lambda: L.overlap_nodes, "overlapCoords": lambda: L.overlap_coords,
                          "init_node_coors": lambda: L.init_coords,
                          "orig_overlap_nodes": lambda: L.orig_overlap_nodes,
                          "orig_overlap_coors": lambda: L.orig_overlap_coors})
        if k in m:
            return m[k]()
        raise KeyError(k)

    def __getitem__(self, k):
        if k in _FIELD_KEYS:
            return self._field(k)
        if dict.__contains__(self, k):
            return dict.__getitem__(self, k)
        return self._geom(k)

    def __setitem__(self, k, v):
        if k in _FIELD_KEYS:
            self._set_field(k, v)
        elif k == "node_coords" and self.lev > 0:
            self.engine.geo.L[self.lev].coords = [np.asarray(c, dtype=np.float64) for c in v]
        else:
            dict.__setitem__(self, k, v)

    def __contains__(self, k):
        try:
            self[k]
            return True
        except KeyError:
            return False

    def get(self, k, default=None):
        try:
            return self[k]
        except KeyError:
            return default


class LevelsList(list):
    def __init__(self, engine):
        super().__init__([LevelView(engine, i) for i in range(4)])
        self.engine = engine


def _engine(Levels) -> Engine:
    e = getattr(Levels, "engine", None)
    if e is None and len(Levels) > 1:
        e = getattr(Levels[1], "engine", None)
    if e is None:
        raise GomeltError("Levels must come from SetupLevels of this module")
    return e


def _l0_index(nodes, per_axis):
    x, y, z = (np.asarray(a) for a in per_axis)
    return (x[None, None, :] + y[None, :, None] * nodes[0] + z[:, None, None] * nodes[0] * nodes[1]).reshape(-1)


def _bc_indices(nodes):
    """getBCindices (:520-559)."""
    nx, ny, nz = nodes
    nn = nx * ny * nz
    b = np.arange(0, nx * ny)
    t = np.arange(nx * ny * (nz - 1), nn)
    w = np.arange(0, nn, nx)
    e = np.arange(nx - 1, nn, nx)
    s = (np.arange(0, nx)[:, None] + (nx * ny * np.arange(0, nz))[None, :]).reshape(-1)
    n = (np.arange(nx * (ny - 1), nx * ny)[:, None] + (nx * ny * np.arange(0, nz))[None, :]).reshape(-1)
    return [w, e, s, n, b, t]


def _dev_tensor(x, engine, dtype=None):
    if isinstance(x, torch.Tensor) and x.is_cuda:
        t = x if dtype is None else x.to(dtype)
        return t.contiguous()
    return torch.as_tensor(np.asarray(x), dtype=dtype or engine.dtype, device=engine.dev).contiguous()


def _dt_dev(engine, dt):
    return torch.tensor([float(dt)], dtype=torch.float64, device=engine.dev)


# ---------------------------------------------------------------------------
# set-up (:115-579)
# ---------------------------------------------------------------------------
def SetupProperties(prop_obj):
    return setup_properties(prop_obj)


def SetupNonmesh(nonmesh_input):
    d = setup_nonmesh(nonmesh_input)
    if not os.path.exists(d["save_path"]):
        os.makedirs(d["save_path"])
    return d


def SetupLevels(solver_input, properties, dtype=torch.float32, device="cuda"):
    """Levels 0-3 on the device (SetupLevels, :115-264)."""
    nm = solver_input.get("nonmesh", {})
    eng = Engine(solver_input, properties, nm.get("subcycle_num_L2", 1), nm.get("subcycle_num_L3", 1),
                 dtype=dtype, device=device)
    return LevelsList(eng)


def getStaticNodesAndElements(L):
    return _engine(L).geo.ne_nn()


def getStaticSubcycle(N_):
    N2, N3 = N_["subcycle_num_L2"], N_["subcycle_num_L3"]
    return (N2, N3, N2 * N3, float(N2), float(N3), float(N2 * N3))


def calcStaticTmpNodesAndElements(L, v):
    return _engine(L).geo.tmp_ne_nn(np.asarray(v, dtype=float))


def getSubstrateNodes(Levels):
    return _engine(Levels).geo.substrate()


def getBCindices(x):
    return _bc_indices([int(n) for n in x["nodes"]])


def getOverlapRegion(node_coords, nx, ny):
    return _l0_index([int(nx), int(ny)], node_coords)


# ---------------------------------------------------------------------------
# a2: phase / properties
# ---------------------------------------------------------------------------
def computeStateProperties(T, S1, properties, Level_nodes_substrate):
    """-> (S1 float, S2 bool, k [W/mmK], rhocp) as device tensors."""
    T = T.contiguous()
    ph_in = (S1.reshape(-1) > 0.499).to(torch.uint8).contiguous()
    ph_out = torch.empty_like(ph_in)
    k = torch.empty_like(T)
    rc = torch.empty_like(T)
    a = N.gm_state_props_args()
    a.dtype = kern.dtype_code(T)
    a.n = T.numel()
    a.T = T.data_ptr()
    a.ph_in = C.cast(ph_in.data_ptr(), C.POINTER(C.c_uint8))
    a.ph_out = C.cast(ph_out.data_ptr(), C.POINTER(C.c_uint8))
    a.k_out, a.rc_out = k.data_ptr(), rc.data_ptr()
    a.substrate = int(Level_nodes_substrate)
    N.call("gm_state_properties", C.byref(a), C.byref(N.props_struct(properties)), kern.stream_ptr())
    return (ph_out & PH_S1).to(T.dtype), (ph_out & PH_S2) != 0, k, rc


def updateStateProperties(Levels, properties, substrate):
    """(:2513-2564) -> (Levels, [0, k1, k2, k3], [0, rc1, rc2, rc3])."""
    e = _engine(Levels)
    ks, rcs = [0], [0]
    e.substrate = tuple(substrate)
    for lev in (3, 2):
        S1, S2, k, rc = computeStateProperties(e.T[lev], Levels[lev]["S1"], properties, substrate[lev])
        Levels[lev]["S1"] = S1
        if lev == 3:
            Levels[lev]["S2"] = S2
    e._s1_restrict()
    out = {}
    for lev in (1, 2, 3):
        _, _, k, rc = computeStateProperties(e.T[lev], Levels[lev]["S1"], properties, substrate[lev])
        out[lev] = (k, rc)
    return Levels, [0] + [out[i][0] for i in (1, 2, 3)], [0] + [out[i][1] for i in (1, 2, 3)]


# ---------------------------------------------------------------------------
# a1 / a7: level solves
# ---------------------------------------------------------------------------
def _level_geom(Level):
    g = Level.engine.geo.L[Level.lev]
    return g.nodes, g.spacing(), g.origin()


def solveMatrixFreeFE(Level, nn, ne, k, rhocp, dt, T, Fc, Corr):
    """(:582-642) T_new = (sum_e (diag(Me)-Ke) T_e + Fc + Corr) / sum_e Me over
    elements [0, ne); ne must cover whole element planes."""
    e = Level.engine
    nodes, h, o = _level_geom(Level)
    exy = (nodes[0] - 1) * (nodes[1] - 1)
    if int(ne) % exy != 0:
        raise GomeltError("ne must be a whole number of element planes")
    T = _dev_tensor(T, e)
    out = torch.empty_like(T)
    F = _dev_tensor(Fc, e) if not (np.isscalar(Fc) and Fc == 0) else None
    Cr = _dev_tensor(Corr, e) if not (np.isscalar(Corr) and Corr == 0) else None
    kern.level_step(e.ps, T_in=T, T_out=out, nodes=nodes, h=h, origin=o, ne_planes=int(ne) // exy,
                    dt=_dt_dev(e, dt), k_arr=_dev_tensor(k, e), rc_arr=_dev_tensor(rhocp, e), F_full=F,
                    corr_full=Cr)
    return out


def substitute_Tbar(Tbar, _idx, _val):
    T = Tbar.clone()
    T[int(_idx):] = _val
    return T


def substitute_Tbar2(Tbar, _idx, _val):
    T = Tbar.clone()
    T[torch.as_tensor(np.asarray(_idx), device=T.device)] = _val
    return T


def assignBCs(RHS, Levels):
    R = RHS.clone()
    BC = Levels[1]["BC"]
    c = Levels[1]["conditions"]
    for j, v in ((2, c["y"][0]), (3, c["y"][1]), (0, c["x"][0]), (1, c["x"][1]), (4, c["z"][0])):
        R[torch.as_tensor(BC[j], device=R.device)] = float(v)
    return R


def assignBCsFine(RHS, TfAll, BC):
    R = RHS.clone()
    for j in (2, 3, 0, 1, 4):
        i = torch.as_tensor(BC[j], device=R.device)
        R[i] = TfAll[i]
    return R


def bincount(Nidx, D, nn):
    return torch.bincount(torch.as_tensor(Nidx).reshape(-1), weights=torch.as_tensor(D).reshape(-1),
                          minlength=int(nn))[: int(nn)]


def _fused_solve(Levels, lev, T0, F, V, k, rc, dt, bc_field=None):
    e = _engine(Levels)
    nodes, h, o = _level_geom(Levels[lev])
    out = torch.empty_like(e.T[lev])
    kw = {}
    if lev == 1:
        exy = (nodes[0] - 1) * (nodes[1] - 1)
        ne_planes = e.tmp[0] // exy
        c = e.geo.conditions
        kw.update(bc_mode=1, face=[c["x"][0], c["x"][1], c["y"][0], c["y"][1], c["z"][0]], inactive_amb=1)
    else:
        ne_planes = nodes[2] - 1
        m = e.tables["bc12"] if lev == 2 else e.tables["bc23"]
        bc = _dev_tensor(bc_field, e)
        kw.update(bc_mode=2, bc_new=bc, bc_old=bc, bc_alpha=1.0, bc_beta=0.0, bc_map=m)
    kern.level_step(e.ps, T_in=_dev_tensor(T0, e), T_out=out, nodes=nodes, h=h, origin=o, ne_planes=ne_planes,
                    dt=_dt_dev(e, dt), k_arr=_dev_tensor(k, e), rc_arr=_dev_tensor(rc, e),
                    F_full=None if F is None else _dev_tensor(F, e), corr_full=None if V is None else
                    _dev_tensor(V, e), **kw)
    return out


def computeL1Temperature(Levels, ne_nn, tmp_ne_nn, L1F, L1V, L1k, L1rhocp, dt, properties):
    """(:2813-2854) solve + inactive nodes := T_amb + Dirichlet faces."""
    _engine(Levels).tmp = tuple(tmp_ne_nn)
    return _fused_solve(Levels, 1, Levels[1]["T0"], L1F, L1V, L1k, L1rhocp, dt)


def computeL2Temperature(L1T, L1L2Interp, Levels, ne_nn, L2T0, L2F, L2V, L2k, L2rhocp, dt):
    """(:2917-2957) solve + Dirichlet ring from the prolongated Level-1 field."""
    return _fused_solve(Levels, 2, L2T0, L2F, L2V, L2k, L2rhocp, dt, bc_field=L1T)


def computeSolutions_L3(FinalL2, L2L3Interp, Levels, ne_nn, L3T0, L3F, L3k, L3rhocp, dt):
    """(:3015-3054)."""
    return _fused_solve(Levels, 3, L3T0, L3F, None, L3k, L3rhocp, dt, bc_field=FinalL2)


def computeSolutions(Levels, ne_nn, tmp_ne_nn, LF, L1V, LInterp, Lk, Lrhocp, L2V, dt, properties):
    """(:2135-2204)."""
    _engine(Levels).tmp = tuple(tmp_ne_nn)
    F1 = _fused_solve(Levels, 1, Levels[1]["T0"], LF[1], L1V, Lk[1], Lrhocp[1], dt)
    F2 = _fused_solve(Levels, 2, Levels[2]["T0"], LF[2], L2V, Lk[2], Lrhocp[2], dt, bc_field=F1)
    F3 = _fused_solve(Levels, 3, Levels[3]["T0"], LF[3], None, Lk[3], Lrhocp[3], dt, bc_field=F2)
    return F1, F2, F3


# ---------------------------------------------------------------------------
# a3-a5: sources and surface flux
# ---------------------------------------------------------------------------
def _row_dev(engine, v, P):
    r = np.zeros(7)
    vv = np.asarray(v, dtype=float).reshape(-1)
    r[: min(7, vv.size)] = vv[:7]
    r[6] = float(P)
    return torch.as_tensor(r, device=engine.dev)


def computeSourcesL3(Level, v, ne_nn, properties, laserP):
    e = Level.engine
    nodes, h, o = _level_geom(Level)
    F = torch.zeros(int(np.prod(nodes)), dtype=e.dtype, device=e.dev)
    row = _row_dev(e, v, laserP)
    N.call("gm_fine_source", kern.dtype_code(F), (C.c_int * 3)(*nodes), (C.c_double * 3)(*o),
           (C.c_double * 3)(*h), row.data_ptr(), C.byref(N.props_struct(properties)), F.data_ptr(),
           kern.stream_ptr())
    return F


def computeConvRadBC(Level, LevelT0, ne, nn, properties, F):
    e = Level.engine
    nodes, h, _ = _level_geom(Level)
    exy = (nodes[0] - 1) * (nodes[1] - 1)
    out = torch.zeros(int(nn), dtype=e.dtype, device=e.dev)
    if not (np.isscalar(F) and F == 0):
        out += _dev_tensor(F, e)
    T = _dev_tensor(LevelT0, e)
    N.call("gm_surface_flux", kern.dtype_code(out), (C.c_int * 3)(*nodes), (C.c_double * 3)(*h),
           int(ne) // exy, T.data_ptr(), C.byref(N.props_struct(properties)), out.data_ptr(), kern.stream_ptr())
    return out


class Shape:
    """Opaque coarse-at-fine handle (computeCoarseFineShapeFunctions, :1213-1358)."""

    def __init__(self, engine, coarse_lev, fine_lev):
        g = engine.geo
        self.engine = engine
        self.coarse, self.fine = coarse_lev, fine_lev
        fc, cc = g.L[fine_lev].coords, g.L[coarse_lev].coords
        self.arena = TableArena(1 << 16 | 128 * sum(len(c) for c in fc), engine.dev)
        self.arena.begin()
        self.geom = CoupleGeom(fc, cc, engine.np_dtype, self.arena)
        self.arena.upload(None)


def computeCoarseFineShapeFunctions(Coarse, Fine):
    return Shape(Coarse.engine, Coarse.lev, Fine.lev)


def _full_out(engine, lev):
    n = engine.geo.L[lev].nodes
    return torch.zeros(int(np.prod(n)), dtype=engine.dtype, device=engine.dev), [0, 0, 0], list(n)


def computeLevelSource(Levels, ne_nn, laser_position, LevelShape, properties, laserP):
    e = _engine(Levels)
    lp = np.array(np.asarray(laser_position, dtype=float).reshape(-1, 7))
    lp[:, 6] = np.asarray(laserP, dtype=float).reshape(-1)
    rows = torch.as_tensor(lp, device=e.dev).contiguous()
    out, lo, n = _full_out(e, LevelShape.coarse)
    e._coarse_source(LevelShape.geom, rows, lp.shape[0], out, lo, n)
    return out


def computeSources(Level, v, Shapes, ne_nn, properties, laserP):
    e = Level.engine
    row = _row_dev(e, v, laserP)
    Fc, lo1, n1 = _full_out(e, 1)
    Fm, lo2, n2 = _full_out(e, 2)
    e._coarse_source(Shapes[1].geom, row, 1, Fc, lo1, n1)
    e._coarse_source(Shapes[2].geom, row, 1, Fm, lo2, n2)
    return Fc, Fm, computeSourcesL3(Level, v, ne_nn, properties, laserP)


def computeSourceFunction_jax(x, y, z, v, properties, P):
    """(:991-1025) pointwise Gaussian source (host helper, NumPy)."""
    p = properties
    rc = 1 / (p["laser_radius"] * np.sqrt(np.pi))
    dc = 1 / (p["laser_depth"] * np.sqrt(np.pi))
    return (6 * np.sqrt(3) * P * p["laser_eta"] * rc * np.exp(-3 * (x - v[0]) ** 2 / p["laser_radius"] ** 2)
            * rc * np.exp(-3 * (y - v[1]) ** 2 / p["laser_radius"] ** 2)
            * dc * np.exp(-3 * (z - v[2]) ** 2 / p["laser_depth"] ** 2))


# ---------------------------------------------------------------------------
# a12/a13: subgrid coupling terms
# ---------------------------------------------------------------------------
def _couple_full(engine, shape, Tfine, Sfine, Tp=None, dTa=None, dTb=None, dt=None, k=None, rc=None, out=None):
    fl = shape.fine
    if out is None:
        out, lo, n = _full_out(engine, shape.coarse)
    else:
        lo, n = [0, 0, 0], list(engine.geo.L[shape.coarse].nodes)
    ph = (Sfine.reshape(-1) > 0.499).to(torch.uint8).contiguous()
    a = N.gm_couple_args()
    a.dtype = kern.dtype_code(out)
    a.geom = shape.geom.struct
    L = engine.geo.L[fl]
    for d in range(3):
        a.fine_nodes[d] = L.nodes[d]
        a.fine_h[d] = L.spacing()[d]
        a.out_lo[d] = lo[d]
        a.out_n[d] = n[d]
    a.T = kern.ptr(_dev_tensor(Tfine, engine))
    a.ph = C.cast(ph.data_ptr(), C.POINTER(C.c_uint8))
    a.substrate = 0
    if k is not None:
        kk, rr = _dev_tensor(k, engine), _dev_tensor(rc, engine)
        a.k_arr, a.rc_arr = kk.data_ptr(), rr.data_ptr()
    keep = []
    if Tp is not None:
        t = _dev_tensor(Tp, engine)
        keep.append(t)
        a.Tp = t.data_ptr()
    if dTa is not None:
        ta, tb = _dev_tensor(dTa, engine), _dev_tensor(dTb, engine)
        dtt = _dt_dev(engine, dt)
        keep += [ta, tb, dtt]
        a.dTa, a.dTb, a.dt = ta.data_ptr(), tb.data_ptr(), dtt.data_ptr()
    a.out = out.data_ptr()
    a.scale = 1.0
    part = torch.empty(max(1, shape.geom.partials), dtype=engine.dtype, device=engine.dev)
    a.partials = part.data_ptr()
    a.partials_cap = part.numel()
    N.call("gm_couple", C.byref(a), C.byref(engine.ps), kern.stream_ptr())
    return out


def computeL1TprimeTerms_Part1(Levels, ne_nn, L3k, Shapes, L2k):
    e = _engine(Levels)
    dummy = torch.zeros_like(e.T[3])
    out = _couple_full(e, Shapes[1], e.T[3], dummy, Tp=e.Tp[3], k=L3k, rc=L3k)
    return _couple_full(e, Shapes[0], e.T[2], torch.zeros_like(e.T[2]), Tp=e.Tp[2], k=L2k, rc=L2k, out=out)


def computeL2TprimeTerms_Part1(Levels, ne_nn, L3Tprime0, L3k, Shapes):
    e = _engine(Levels)
    return _couple_full(e, Shapes[2], e.T[3], torch.zeros_like(e.T[3]), Tp=L3Tprime0, k=L3k, rc=L3k)


def computeL1TprimeTerms_Part2(Levels, ne_nn, L3Tp, L2Tp, L3rhocp, L2rhocp, dt, Shapes, Vcu):
    e = _engine(Levels)
    out = _dev_tensor(Vcu, e).clone()
    _couple_full(e, Shapes[1], e.T[3], torch.zeros_like(e.T[3]), dTa=L3Tp, dTb=e.Tp[3], dt=dt, k=L3rhocp,
                 rc=L3rhocp, out=out)
    _couple_full(e, Shapes[0], e.T[2], torch.zeros_like(e.T[2]), dTa=L2Tp, dTb=e.Tp[2], dt=dt, k=L2rhocp,
                 rc=L2rhocp, out=out)
    return out


def computeL2TprimeTerms_Part2(Levels, ne_nn, L3Tp, L3Tp0, L3rhocp, dt, Shapes, L2V):
    e = _engine(Levels)
    out = _dev_tensor(L2V, e).clone()
    return _couple_full(e, Shapes[2], e.T[3], torch.zeros_like(e.T[3]), dTa=L3Tp, dTb=L3Tp0, dt=dt, k=L3rhocp,
                        rc=L3rhocp, out=out)


def computeCoarseTprimeTerm_jax(Levels, L3k, L2k, Shapes):
    Vcu = computeL1TprimeTerms_Part1(Levels, None, L3k, Shapes, L2k)
    Vmu = computeL2TprimeTerms_Part1(Levels, None, _engine(Levels).Tp[3], L3k, Shapes)
    return Vcu, Vmu


def computeCoarseTprimeMassTerm_jax(Levels, Tprimef, Tprimem, L3rhocp, L2rhocp, dt, Shapes, Vcu, Vmu):
    e = _engine(Levels)
    Vcu = computeL1TprimeTerms_Part2(Levels, None, Tprimef, Tprimem, L3rhocp, L2rhocp, dt, Shapes, Vcu)
    Vmu = computeL2TprimeTerms_Part2(Levels, None, Tprimef, e.Tp[3], L3rhocp, dt, Shapes, Vmu)
    return Vcu, Vmu


# ---------------------------------------------------------------------------
# a8-a10: interpolation, restriction + T'
# ---------------------------------------------------------------------------
def _map_to(Level, node_coords_new):
    e = Level.engine
    L = e.geo.L[Level.lev]
    return kern.DeviceMap3([axis_map(L.coords[d], np.asarray(node_coords_new[d], dtype=float)) for d in range(3)],
                           L.nodes, e.dtype, e.dev)


class InterpMatrix(list):
    """[Nc (npts, 8), node (npts, 8)] on the device, plus the separable map."""


def interpolatePointsMatrix(Level, node_coords_new):
    e = Level.engine
    m = _map_to(Level, node_coords_new)
    npts = int(np.prod(m.n))
    Nc = torch.empty(npts * 8, dtype=e.dtype, device=e.dev)
    node = torch.empty(npts * 8, dtype=torch.int32, device=e.dev)
    N.call("gm_interp_matrix", kern.dtype_code(Nc), C.byref(m.struct), Nc.data_ptr(), node.data_ptr(),
           kern.stream_ptr())
    out = InterpMatrix([Nc.view(npts, 8), node.view(npts, 8)])
    out.map = m
    return out


def interpolate_w_matrix(C2F, T):
    Nc, node = C2F[0], C2F[1]
    T = T.contiguous()
    out = torch.empty(Nc.shape[0], dtype=Nc.dtype, device=Nc.device)
    N.call("gm_interp_w_matrix", kern.dtype_code(out), Nc.data_ptr(), node.data_ptr(), T.data_ptr(),
           out.data_ptr(), C.c_longlong(Nc.shape[0]), kern.stream_ptr())
    return out


def interpolatePoints(Level, u, node_coords_new):
    e = Level.engine
    m = _map_to(Level, node_coords_new)
    out = torch.empty(int(np.prod(m.n)), dtype=e.dtype, device=e.dev)
    e._interp([(m, _dev_tensor(u, e), 1.0)], m.n, out)
    return out


def getNewTprime(Fine, FineT0, CoarseT, Coarse, C2F):
    """(:2060-2099) -> (T' of the fine level, coarse T with the overlap restricted).

    The restriction (the fine field interpolated at the coarse overlap nodes,
    written into a copy of the coarse field) is gm_restrict; T' = T_f - I(T_c)
    is one gm_interp with the fine field as its base when C2F carries its
    separable map (interpolatePointsMatrix, moveEverything), else
    gm_interp_w_matrix over the materialised [Nc, node] pair."""
    e = Fine.engine
    FT = _dev_tensor(FineT0, e)
    CT = _dev_tensor(CoarseT, e).clone()
    rmap = _map_to(Fine, Fine["overlapCoords"])
    cn = [int(n) for n in Coarse["nodes"]]
    onodes = Fine["overlapNodes"]
    idx_t = []
    for d in range(3):
        a = np.asarray(onodes[d])
        if a.size == 0 or a.min() < 0 or a.max() >= cn[d]:
            raise GomeltError(f"getNewTprime: overlap nodes of axis {d} outside the coarse grid")
        idx_t.append(torch.as_tensor(a.astype(np.int32), device=e.dev))
    idx = [C.cast(t.data_ptr(), C.POINTER(C.c_int)) for t in idx_t]
    e._restrict(rmap, idx, cn, FT, CT)
    cmap = getattr(C2F, "map", None)
    if cmap is not None:
        Tp = torch.empty_like(FT)
        e._interp([(cmap, CT, -1.0)], e.geo.L[Fine.lev].nodes, Tp, base=FT)
    else:
        Tp = FT - interpolate_w_matrix(C2F, CT)
    return Tp, CT


def getBothNewTprimes(Levels, FineT, MesoT, M2F, CoarseT, C2M):
    lTp, mT0 = getNewTprime(Levels[3], FineT, MesoT, Levels[2], M2F)
    mTp, uT0 = getNewTprime(Levels[2], mT0, CoarseT, Levels[1], C2M)
    return lTp, mTp, mT0, uT0


# ---------------------------------------------------------------------------
# the hot path: moveEverything, subcycleGOMELT, stepGOMELT, dwell
# ---------------------------------------------------------------------------
def moveEverything(v, vstart, Levels, move_v, LInterp, L1L2Eratio, L2L3Eratio, height):
    """(:2400-2510) -> (Levels, Shapes, LInterp, move_v)."""
    e = _engine(Levels)
    mv = e.move(np.asarray(v, dtype=float), np.asarray(vstart, dtype=float))
    Shapes = [_shape_from_table(e, 1, 2, "c21"), _shape_from_table(e, 1, 3, "c31"),
              _shape_from_table(e, 2, 3, "c32")]
    return Levels, Shapes, [_interp_handle(e, "bc12"), _interp_handle(e, "bc23")], mv


def _shape_from_table(e, coarse, fine, key):
    s = Shape.__new__(Shape)
    s.engine, s.coarse, s.fine, s.geom = e, coarse, fine, e.tables[key]
    return s


def _interp_handle(e, key):
    h = InterpMatrix([])
    h.map = e.tables[key]
    return h


def subcycleGOMELT(Levels, ne_nn, Shapes, substrate, LInterp, tmp_ne_nn, laser_position, properties, laserP,
                   subcycle, max_accum_L3, accum_L3, history=True):
    """(:3224-3632) -> (Levels, L2all, L3all, L3pall, max_accum_L3, accum_L3).
    ``history=False`` skips the per-Level-2-step copies (the driver does not
    use them; the reference returns them)."""
    e = _engine(Levels)
    e.tmp = tuple(tmp_ne_nn)
    e.substrate = tuple(substrate)
    if (e.N2, e.N3) != (int(subcycle[0]), int(subcycle[1])):
        e.N2, e.N3 = int(subcycle[0]), int(subcycle[1])
    rows = np.array(np.asarray(laser_position, dtype=np.float64).reshape(-1, 7))
    rows[:, 6] = np.asarray(laserP, dtype=np.float64).reshape(-1)
    e.macc3.copy_(_dev_tensor(max_accum_L3, e).reshape(-1))
    e.acc3.copy_(_dev_tensor(accum_L3, e).reshape(-1))
    hist = e.subcycle(rows, history=history)
    L2all, L3all, L3pall = hist if hist is not None else (None, None, None)
    return Levels, L2all, L3all, L3pall, e.macc3, e.acc3


def stepGOMELT(Levels, ne_nn, tmp_ne_nn, Shapes, LInterp, v, properties, dt, laserP, substrate):
    """(:2304-2397) -> (Levels, resetmask)."""
    e = _engine(Levels)
    e.tmp = tuple(tmp_ne_nn)
    e.substrate = tuple(substrate)
    row = np.zeros(7)
    vv = np.asarray(v, dtype=float).reshape(-1)
    row[: min(7, vv.size)] = vv[:7]
    row[5] = float(dt)
    row[6] = float(laserP)
    return Levels, e.step(row)


def stepGOMELTDwellTime(Levels, tmp_ne_nn, ne_nn, properties, dt, substrate):
    e = _engine(Levels)
    e.tmp = tuple(tmp_ne_nn)
    e.substrate = tuple(substrate)
    e.dwell(float(dt))
    return Levels


# ---------------------------------------------------------------------------
# driver helpers
# ---------------------------------------------------------------------------
def melting_temp(temps, delt_T, T_melt, accum_time, idx):
    """(:3696-3712) accum_time[idx] += (T > T_melt) * dt."""
    out = accum_time.clone()
    i = torch.as_tensor(np.asarray(idx), device=out.device)
    out.index_add_(0, i, (temps > T_melt).to(out.dtype) * float(delt_T))
    return out


def printLevelMaxMin(Ls, Lnames):
    """(:3635-3665) print min/max T per level; exit(1) on invalid values."""
    print("Temps:", end=" ")
    flag = False
    for i in range(1, len(Ls)):
        T = Ls[i]["T0"]
        mm = torch.stack([T.min(), T.max()]).double().cpu().numpy()
        Lmin, Lmax = float(mm[0]), float(mm[1])
        for name, val in (("Lmax", Lmax), ("Lmin", Lmin)):
            if not np.isfinite(val) or val <= 0 or val > 1e5:
                print(f"\nTerminating program: {name} for {Lnames[i - 1]} is NaN, 0, or invalid.")
                flag = True
        print(f"{Lnames[i - 1]}: [{Lmin:.2f}, {Lmax:.2f}]", end=" ")
    if flag:
        sys.exit(1)
    print("")


# ---------------------------------------------------------------------------
# Output files (saveResult & co., :1945-2057, :3668-3693), written by vtk.py
# ---------------------------------------------------------------------------
def _host(a):
    return a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)


def saveResult(Level, save_str, record_lab, save_path, zoffset):
    """:1945-1982: temperature and S1 of a level as a rectilinear grid
    ``{save_path}{save_str}{record_lab:08}.vtr`` (z shifted by -zoffset)."""
    import vtk

    c = [np.asarray(Level["node_coords"][d], dtype=np.float64) for d in range(3)]
    vtk.write_vtr(f"{save_path}{save_str}{record_lab:08}", c[0], c[1], c[2] - zoffset,
                  {"Temperature (K)": _host(Level["T0"]), "State (Powder/Solid)": _host(Level["S1"])})


def saveFinalResult(Level, save_str, save_path, zoffset):
    """:1985-2021: as saveResult, file ``{save_path}{save_str}Final.vtr``."""
    import vtk

    c = [np.asarray(Level["node_coords"][d], dtype=np.float64) for d in range(3)]
    vtk.write_vtr(f"{save_path}{save_str}Final", c[0], c[1], c[2] - zoffset,
                  {"Temperature (K)": _host(Level["T0"]), "State (Powder/Solid)": _host(Level["S1"])})


def saveState(Level, save_str, record_lab, save_path, zoffset):
    """:2024-2057: S1 only (Level 0 unpacked from its bit store to one byte a node)."""
    import vtk

    c = [np.asarray(Level["node_coords"][d], dtype=np.float64) for d in range(3)]
    s1 = Level.engine.l0_s1() if isinstance(Level, LevelView) and Level.lev == 0 else Level["S1"]
    vtk.write_vtr(f"{save_path}{save_str}{record_lab:08}", c[0], c[1], c[2] - zoffset,
                  {"State (Powder/Solid)": _host(s1)})


def saveResults(Levels, Nonmesh, savenum):
    """:3668-3682."""
    if Nonmesh["output_files"] == 1:
        if savenum == 1 or (np.mod(savenum, Nonmesh["Level1_record_step"]) == 1
                            or Nonmesh["Level1_record_step"] == 1):
            saveResult(Levels[1], "Level1_", savenum, Nonmesh["save_path"], 2e-3)
        saveResult(Levels[2], "Level2_", savenum, Nonmesh["save_path"], 1e-3)
        saveResult(Levels[3], "Level3_", savenum, Nonmesh["save_path"], 0)
        print(f"Saved Levels_{savenum:08}")


def saveResultsFinal(Levels, Nonmesh):
    """:3685-3693."""
    if Nonmesh["output_files"] == 1:
        saveFinalResult(Levels[1], "Level1_", Nonmesh["save_path"], 2e-3)
        saveFinalResult(Levels[2], "Level2_", Nonmesh["save_path"], 1e-3)
        saveFinalResult(Levels[3], "Level3_", Nonmesh["save_path"], 0)
        print("Saved Final Results")


def save_object(obj, filename):
    with open(filename, "wb") as f:
        pickle.dump(obj, f, pickle.HIGHEST_PROTOCOL)
