"""Snapshots, training and evaluation of the Level-3 surrogate.

* ``generate`` — plain multilevel runs of the batched single-track instances
  (``workloads.batched_instances``); per Level-2 step of every subcycle call one
  snapshot: the Level-2 field at the step's end prolongated to Level 3, the
  Level-3 field at its start and at its end, and the window / laser
  parameters.  Kept on the device (FP32).
* ``train`` — Adam on mini-batches of snapshots (``surrogate.UNet``).
* ``evaluate`` — on a part-scale scan: per Level-2 step, the prediction from
  the plain run's start state against the plain run's end state (max / RMS
  error of the Level-3 field), the energy-balance residual of the prediction
  (accepted below 1 %), and the time of one prediction against the time of
  the plain Level-3 work it replaces.
"""

from __future__ import annotations

import time

import numpy as np
import torch

import diagnostics
import engine
import levels
import surrogate

ACCEPT_RESIDUAL = 0.01


class Snapshots:
    def __init__(self, nn, cap, device):
        self.nn, self.cap, self.n = nn, cap, 0
        f = dict(dtype=torch.float32, device=device)
        self.T2i = torch.empty(cap, nn, **f)
        self.T3o = torch.empty(cap, nn, **f)
        self.T3n = torch.empty(cap, nn, **f)
        self.par = torch.empty(cap, 8, dtype=torch.float64, device=device)
        self.par_h = np.zeros((cap, 8))


def _instance_rows(cfg):
    import createPath

    P = levels.setup_properties(cfg["properties"])
    nm = levels.setup_nonmesh(cfg["nonmesh"])
    if "gcode" in cfg:
        gcode = cfg["gcode"]
    else:
        r = cfg["raster"]
        gcode = createPath.serpentine_gcode(r["x0"], r["y0"], r["length"], r["hatch"], r["ntracks"])
    rows = np.asarray(createPath.toolpath(nm, P, gcode), dtype=np.float64)
    return P, nm, rows


def _prolong(eng, T2, out):
    """Level-2 field prolongated to every Level-3 node (interpolate_w_matrix)."""
    eng._interp([(eng.tables["bc23"], T2, 1.0)], eng.geo.L[3].nodes, out)


def run_with_snapshots(cfg, snaps, device, stream, max_steps=None, on_step=None):
    """Plain run of one instance; appends a snapshot per Level-2 step."""
    P, nm, rows = _instance_rows(cfg)
    N2, N3 = nm["subcycle_num_L2"], nm["subcycle_num_L3"]
    n23 = N2 * N3
    nsteps = len(rows) // n23 if max_steps is None else min(max_steps, len(rows) // n23)
    vstart = np.asarray(cfg["properties"]["laser_center"], dtype=float)
    r, pw, vel = P["laser_radius"], P["laser_power"], nm["laser_velocity"]
    with torch.cuda.stream(stream):
        eng = engine.Engine(cfg, P, N2, N3, device=device, stream=stream)
        eng.set_layer(rows[0])
        eng.move(rows[0], vstart)
        for k in range(nsteps):
            c = rows[k * n23:(k + 1) * n23]
            eng.move(c[0], vstart)
            T3s = eng.T[3].clone()
            L2all, L3all, _ = eng.subcycle(c, history=True)
            L3 = eng.geo.L[3]
            o, h = L3.origin(), L3.spacing()[0]
            for j in range(N2 if snaps is not None else 0):
                if snaps.n >= snaps.cap:
                    return eng
                i = snaps.n
                _prolong(eng, L2all[j], snaps.T2i[i])
                snaps.T3o[i].copy_(T3s if j == 0 else L3all[j - 1])
                snaps.T3n[i].copy_(L3all[j])
                mid = c[j * N3 + N3 // 2]
                snaps.par_h[i] = surrogate.window_params(o, h, mid[:2], r, pw, vel)
                snaps.n += 1
            if on_step is not None:
                on_step(eng, k, c, T3s, L2all, L3all)
    return eng


def generate(instances, device, cap=20000, max_steps=None):
    stream = torch.cuda.Stream(device=device)
    nn = None
    snaps = None
    t0 = time.perf_counter()
    for cfg in instances:
        if snaps is None:
            g = levels.Geometry(cfg, levels.setup_properties(cfg["properties"]))
            nn = g.L[3].nn
            snaps = Snapshots(nn, cap, device)
        run_with_snapshots(cfg, snaps, device, stream, max_steps=max_steps)
        if snaps.n >= snaps.cap:
            break
    stream.synchronize()
    snaps.par.copy_(torch.as_tensor(snaps.par_h))
    return snaps, time.perf_counter() - t0


def train(net, snaps, nodes, grid_xyz, steps, batch, lr, device, seed=0, log_every=0):
    """Adam on random mini-batches of the snapshots; returns the loss curve."""
    rng = np.random.default_rng(seed)
    X, Y, Z = grid_xyz
    grid = (batch, X, Y, Z)
    V = batch * X * Y * Z
    x = torch.empty(V, 16, dtype=torch.bfloat16, device=device)
    target = torch.empty(V, dtype=torch.float32, device=device)
    lmask = torch.empty(V, dtype=torch.float32, device=device)
    nn = snaps.nn
    bT2 = torch.empty(batch, nn, device=device)
    bT3o = torch.empty(batch, nn, device=device)
    bT3n = torch.empty(batch, nn, device=device)
    bpar = torch.empty(batch, 8, dtype=torch.float64, device=device)
    count = float(batch * (X - 1) * (Y - 1) * Z)
    losses = []
    t0 = time.perf_counter()
    for s in range(steps):
        idx = torch.as_tensor(rng.integers(0, snaps.n, batch), device=device)
        torch.index_select(snaps.T2i, 0, idx, out=bT2)
        torch.index_select(snaps.T3o, 0, idx, out=bT3o)
        torch.index_select(snaps.T3n, 0, idx, out=bT3n)
        torch.index_select(snaps.par, 0, idx, out=bpar)
        surrogate.pack(grid=grid, nodes=nodes, T2i=bT2, T3o=bT3o, T3n=bT3n, par=bpar, T_amb=300.0, x=x,
                       target=target, lmask=lmask)
        net.forward(x, grid)
        loss = net.backward(target, lmask, 1.0 / count)
        net.step(lr=lr * (0.5 * (1 + np.cos(np.pi * s / steps)) * 0.9 + 0.1))
        if log_every and (s % log_every == 0 or s == steps - 1):
            losses.append((s, float(loss)))
    torch.cuda.synchronize()
    return losses, time.perf_counter() - t0


def evaluate(net, cfg, device, nsteps, warm=2):
    """Part-scale evaluation: plain run with history; per Level-2 step the
    surrogate's prediction against the plain result."""
    P, nm, rows = _instance_rows(cfg)
    N2, N3 = nm["subcycle_num_L2"], nm["subcycle_num_L3"]
    n23 = N2 * N3
    stream = torch.cuda.Stream(device=device)
    dg = diagnostics.Diagnostics(device)
    g = levels.Geometry(cfg, P)
    L3 = g.L[3]
    nodes = L3.nodes
    X, Y, Z = nodes[0] - 1, nodes[1] - 1, nodes[2] - 1
    X, Y, Z = X - X % 4, Y - Y % 4, Z - Z % 4
    grid = (1, X, Y, Z)
    V = X * Y * Z
    x = torch.empty(V, 16, dtype=torch.bfloat16, device=device)
    T2i = torch.empty(L3.nn, device=device)
    pred_T3 = torch.empty(L3.nn, device=device)
    par = torch.empty(1, 8, dtype=torch.float64, device=device)
    stats = dict(max_err=[], rms_err=[], residual=[], plain_residual=[], accepted=0, total=0, t_pred_ms=[])
    r, pw, vel = P["laser_radius"], P["laser_power"], nm["laser_velocity"]
    eta = P["laser_eta"]

    def on_step(eng, k, c, T3s, L2all, L3all):
        if k < warm:
            return
        Lc = eng.geo.L[3]
        o, h = Lc.origin(), Lc.spacing()[0]
        ne_planes = Lc.nodes[2] - 1
        for j in range(N2):
            T3o = T3s if j == 0 else L3all[j - 1]
            jrows = c[j * N3:(j + 1) * N3]
            mid = jrows[N3 // 2]
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _prolong(eng, L2all[j], T2i)
            par.copy_(torch.as_tensor([surrogate.window_params(o, h, mid[:2], r, pw, vel)], dtype=torch.float64))
            a = surrogate.pack(grid=grid, nodes=Lc.nodes, T2i=T2i, T3o=T3o, par=par, T_amb=P["T_amb"], x=x)
            pred = net.forward(x, grid)
            pred_T3.copy_(L3all[j])  # Dirichlet ring and planes outside the network grid: the plain values
            surrogate.unpack(a, pred, pred_T3)
            torch.cuda.synchronize()
            stats["t_pred_ms"].append(1000.0 * (time.perf_counter() - t0))
            m, rms = dg.field_error(pred_T3, L3all[j])
            stats["max_err"].append(m)
            stats["rms_err"].append(rms)
            kw = dict(nodes=Lc.nodes, h=Lc.spacing(), origin=Lc.origin(), ne_planes=ne_planes, T0=T3o,
                      ph=eng.ph[3], substrate=eng.substrate[3], interval=float(jrows[:, 5].sum()), rows=jrows)
            res = dg.residual(dg.energy_terms(eng.ps, T1=pred_T3, **kw), jrows, eta)
            res_plain = dg.residual(dg.energy_terms(eng.ps, T1=L3all[j], **kw), jrows, eta)
            stats["residual"].append(res)
            stats["plain_residual"].append(res_plain)
            stats["total"] += 1
            stats["accepted"] += int(res < ACCEPT_RESIDUAL)

    run_with_snapshots(cfg, None, device, stream, max_steps=nsteps + warm, on_step=on_step)
    return stats
