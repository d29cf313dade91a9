"""Thin Python wrappers over the C ABI taking torch CUDA tensors.

These keep the argument marshalling in one place; the GO-MELT call surface in
computeFunctions.py and the subcycle engine are built on them.
"""

from __future__ import annotations

import ctypes as C
from typing import NamedTuple

import torch

import _native as N


def ptr(t):
    if t is None:
        return None
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise N.GomeltError("device tensors are required (got %r)" % type(t))
    if not t.is_contiguous():
        raise N.GomeltError("tensors must be contiguous")
    return t.data_ptr()


def dtype_code(t: torch.Tensor) -> int:
    if t.dtype == torch.float32:
        return N.GM_F32
    if t.dtype == torch.float64:
        return N.GM_F64
    raise N.GomeltError(f"unsupported dtype {t.dtype}")


def stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


class DeviceMap3:
    """Three AxisMaps uploaded to the device, plus the gm_map3 struct."""

    def __init__(self, maps, src_nodes, dtype, device="cuda"):
        self.e = [torch.tensor(m.elem, dtype=torch.int32, device=device) for m in maps]
        self.w = [torch.tensor(m.w.reshape(-1), dtype=dtype, device=device) for m in maps]
        self.n = [int(m.elem.size) for m in maps]
        self.src_nodes = [int(x) for x in src_nodes]
        s = N.gm_map3()
        for d in range(3):
            s.n[d] = self.n[d]
            s.elem[d] = self.e[d].data_ptr()
            s.w[d] = self.w[d].data_ptr()
        s.src_nx, s.src_ny = self.src_nodes[0], self.src_nodes[1]
        self.struct = s


def level_step(props: N.gm_props, *, stream=None, **kw):
    """gm_level_step with the arguments of level_args."""
    a = level_args(**kw)
    N.call("gm_level_step", C.byref(a), C.byref(props), stream_ptr(stream))


class TunedShape(NamedTuple):
    """A measured launch shape (gm_tune_result): kernel 0 = element tiles
    tile_x x tile_y, kernel 1 = separable stencil with tile_y thread rows of
    `rows` y rows (tile_x threads across x)."""
    tile_x: int
    tile_y: int
    zchunk: int
    us: float
    kernel: int
    rows: int


def level_autotune(props: N.gm_props, *, reps=5, stream=None, **kw) -> TunedShape:
    """gm_level_autotune for the call level_args(**kw) describes."""
    a = level_args(**kw)
    r = N.gm_tune_result()
    N.call("gm_level_autotune", C.byref(a), C.byref(props), int(reps), C.byref(r), stream_ptr(stream), kernels=0)
    return TunedShape(r.tile_x, r.tile_y, r.zchunk, r.us, r.kernel, r.rows)


def level_step_shape(props: N.gm_props, *, kernel, zchunk, tile_x=32, tile_y=1, rows=4, stream=None, **kw):
    """gm_level_step_shape: one level step with an explicit launch shape
    (kernel 0: tile_x 32 or 16; kernel 1: tile_y thread rows of `rows` rows)."""
    a = level_args(**kw)
    s = N.gm_level_shape(int(kernel), int(tile_x), int(tile_y), int(rows), int(zchunk))
    N.call("gm_level_step_shape", C.byref(a), C.byref(props), C.byref(s), stream_ptr(stream))


def level2_args(*, dt2, src_tab2, bc_alpha2, bc_beta2, **kw):
    """gm_level2_args: the first step as level_args(**kw), then the second
    step's dt, laser factor row and ring blend."""
    a = N.gm_level2_args()
    a.level = level_args(**kw)
    a.dt2 = ptr(dt2)
    a.src_tab2 = ptr(src_tab2)
    a.bc_alpha2, a.bc_beta2 = float(bc_alpha2), float(bc_beta2)
    return a


def level_step2(props: N.gm_props, *, stream=None, shape=None, **kw):
    """gm_level_step2 (two Level-3 fine steps in one launch) with the
    arguments of level2_args; shape = (rows, tile_y, zchunk) forces a launch
    shape (gm_level_step2_shape)."""
    a = level2_args(**kw)
    if shape is None:
        N.call("gm_level_step2", C.byref(a), C.byref(props), stream_ptr(stream))
    else:
        s = N.gm_level_shape(2, 28, int(shape[1]), int(shape[0]), int(shape[2]))
        N.call("gm_level_step2_shape", C.byref(a), C.byref(props), C.byref(s), stream_ptr(stream))


def level_autotune2(props: N.gm_props, *, reps=5, stream=None, **kw) -> TunedShape:
    """gm_level_autotune2 for the two-step call level2_args(**kw) describes."""
    a = level2_args(**kw)
    r = N.gm_tune_result()
    N.call("gm_level_autotune2", C.byref(a), C.byref(props), int(reps), C.byref(r), stream_ptr(stream), kernels=0)
    return TunedShape(r.tile_x, r.tile_y, r.zchunk, r.us, r.kernel, r.rows)


def level_args(*, T_in, T_out, nodes, h, origin, ne_planes, dt, ph_in=None, ph_out=None,
               substrate=0, k_arr=None, rc_arr=None, F_full=None, corr_full=None, rhs_box=None, box=None,
               laser=None, surface=0, bc_mode=0, face=None, inactive_amb=0, bc_new=None, bc_old=None,
               bc_alpha=0.0, bc_beta=0.0, bc_map: DeviceMap3 | None = None, clamp=0, accum=None, max_accum=None,
               zchunk=0, pdl=0, src_tab=None, status=None):
    a = N.gm_level_args()
    a.dtype = dtype_code(T_in)
    a.nx, a.ny, a.nz = (int(x) for x in nodes)
    for d in range(3):
        a.h[d] = float(h[d])
        a.origin[d] = float(origin[d])
    a.ne_planes = int(ne_planes)
    a.dt = ptr(dt)
    a.T_in, a.T_out = ptr(T_in), ptr(T_out)
    a.ph_in, a.ph_out = ptr(ph_in), ptr(ph_out)
    a.substrate = int(substrate)
    a.k_arr, a.rc_arr = ptr(k_arr), ptr(rc_arr)
    a.F_full, a.corr_full = ptr(F_full), ptr(corr_full)
    a.rhs_box = ptr(rhs_box)
    if box is not None:
        for i in range(6):
            a.box[i] = int(box[i])
    a.laser = ptr(laser)
    a.surface = int(surface)
    a.bc_mode = int(bc_mode)
    if face is not None:
        for i in range(5):
            a.face[i] = float(face[i])
    a.inactive_amb = int(inactive_amb)
    a.bc_new, a.bc_old = ptr(bc_new), ptr(bc_old)
    a.bc_alpha, a.bc_beta = float(bc_alpha), float(bc_beta)
    if bc_map is not None:
        a.bc_map = bc_map.struct
    a.clamp = int(clamp)
    a.accum, a.max_accum = ptr(accum), ptr(max_accum)
    a.zchunk = int(zchunk)
    a.pdl = int(pdl)
    a.src_tab = ptr(src_tab)
    a.status = ptr(status)
    return a
