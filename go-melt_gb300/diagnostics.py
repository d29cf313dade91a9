"""Diagnostics of a level window, computed on the device in FP64
(libgomelt ``gm_energy_balance``, ``gm_melt_pool``, ``gm_field_error``).

* ``energy_balance`` — heat stored in the interior nodes of a window over an
  interval against the laser energy deposited, the surface flux and the
  conduction across the Dirichlet ring; the relative residual is the test that
  accepts or rejects a predicted Level-3 field.
* ``melt_pool`` — length / width / depth of the region above an isotherm
  (1900 K for the precision study).
* ``field_error`` — max and RMS difference of two fields (an FP32 run against
  an FP64 run of the same case).

The reference has no counterpart of these quantities; their definitions are
stated in ``include/gomelt.h``.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

import _native as N
import kern


def _join(stream):
    """Order the current stream after ``stream`` (results are read or used on
    the current stream)."""
    if stream is not None:
        cur = torch.cuda.current_stream(stream.device)
        if cur != stream:
            cur.wait_stream(stream)


class Diagnostics:
    """Device scratch and result buffers for the diagnostics of one device."""

    def __init__(self, device="cuda", npos_max=256):
        self.dev = torch.device(device)
        self.npos_max = int(npos_max)
        n = int(N.lib().gm_diag_scratch_size(self.npos_max))
        self.scratch = torch.empty(n, dtype=torch.float64, device=self.dev)
        self.out = torch.zeros(8, dtype=torch.float64, device=self.dev)

    def energy_terms(self, props: N.gm_props, *, nodes, h, origin, ne_planes, T0, T1, ph, substrate, interval,
                     rows, stream=None):
        """Device tensor (4,) FP64: stored, source, surface, conduction [J]."""
        rows = torch.as_tensor(rows, dtype=torch.float64, device=self.dev).reshape(-1, 7).contiguous()
        if rows.shape[0] > self.npos_max:
            raise N.GomeltError(f"{rows.shape[0]} laser rows > {self.npos_max}")
        a = N.gm_energy_args()
        a.dtype = kern.dtype_code(T0)
        if T1.dtype != T0.dtype:
            raise N.GomeltError("T0 and T1 must have the same dtype")
        for d in range(3):
            a.nodes[d] = int(nodes[d])
            a.h[d] = float(h[d])
            a.origin[d] = float(origin[d])
        a.ne_planes = int(ne_planes)
        a.T0, a.T1 = kern.ptr(T0), kern.ptr(T1)
        a.ph = kern.ptr(ph)
        a.substrate = int(substrate)
        a.interval = float(interval)
        a.rows = rows.data_ptr()
        a.npos = int(rows.shape[0])
        a.scratch = self.scratch.data_ptr()
        a.scratch_cap = self.scratch.numel()
        out = torch.empty(4, dtype=torch.float64, device=self.dev)
        a.out = out.data_ptr()
        N.call("gm_energy_balance", C.byref(a), C.byref(props), kern.stream_ptr(stream),
               kernels=3 if a.npos > 0 else 2)
        self._keep = rows  # alive until the kernels ran
        _join(stream)
        return out

    @staticmethod
    def residual(terms, rows, eta):
        """|stored - source - surface - conduction| / (eta * sum dt P)."""
        t = [float(x) for x in (terms.tolist() if torch.is_tensor(terms) else terms)]
        r = np.asarray(rows, dtype=np.float64).reshape(-1, 7)
        e_in = eta * float((r[:, 5] * r[:, 6]).sum())
        return abs(t[0] - t[1] - t[2] - t[3]) / e_in if e_in > 0 else float("inf")

    def melt_pool(self, *, nodes, h, origin, T, iso, stream=None):
        """dict(length, width, depth, count, extents) of the region T >= iso."""
        a = N.gm_meltpool_args()
        a.dtype = kern.dtype_code(T)
        for d in range(3):
            a.nodes[d] = int(nodes[d])
            a.h[d] = float(h[d])
            a.origin[d] = float(origin[d])
        a.T = kern.ptr(T)
        a.iso = float(iso)
        a.scratch = self.scratch.data_ptr()
        a.scratch_cap = self.scratch.numel()
        out = torch.empty(7, dtype=torch.float64, device=self.dev)
        a.out = out.data_ptr()
        N.call("gm_melt_pool", C.byref(a), kern.stream_ptr(stream), kernels=2)
        _join(stream)
        v = out.tolist()
        ztop = float(origin[2]) + float(h[2]) * (int(nodes[2]) - 1)
        if v[6] == 0:
            return dict(length=0.0, width=0.0, depth=0.0, count=0, extents=v[:6])
        return dict(length=v[1] - v[0], width=v[3] - v[2], depth=ztop - v[4], count=int(v[6]), extents=v[:6])

    def field_error(self, A, B, stream=None):
        """(max |A - B|, RMS(A - B)) in FP64."""
        if A.numel() != B.numel():
            raise N.GomeltError("field_error: sizes differ")
        out = torch.empty(2, dtype=torch.float64, device=self.dev)
        N.call("gm_field_error", kern.dtype_code(A), kern.ptr(A), kern.dtype_code(B), kern.ptr(B), int(A.numel()),
               self.scratch.data_ptr(), self.scratch.numel(), out.data_ptr(), kern.stream_ptr(stream), kernels=2)
        _join(stream)
        m, r = out.tolist()
        return m, r
