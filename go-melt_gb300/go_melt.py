"""JSON-driven GO-MELT driver on the GB300 engine.

Same input file, command line and control flow as the reference driver
(JLnorthwestern/GO-MELT go_melt/go_melt.py): the toolpath is read N2*N3 lines
at a time; a chunk runs as one subcycled step (moveEverything +
subcycleGOMELT) unless it starts a layer, ends the file, contains a long
pause or a jump, in which case its lines run as single equal-dt steps
(stepGOMELT), or as Level-1-only dwell steps once the laser has been off
longer than ``wait_time``.  A new layer shifts Level 1 and the Level-0 phase
store, saves the melt-time record and writes a checkpoint.

Usage: python go_melt.py [DEVICE_ID] [input.json]
"""

from __future__ import annotations

import json
import os
import pickle
import sys
import time

import numpy as np
import torch

from computeFunctions import (  # noqa: F401
    SetupLevels, SetupNonmesh, SetupProperties, calcStaticTmpNodesAndElements, getStaticNodesAndElements,
    getStaticSubcycle, getSubstrateNodes, moveEverything, printLevelMaxMin, saveResults, saveResultsFinal,
    saveState, stepGOMELT, stepGOMELTDwellTime, subcycleGOMELT)
from createPath import count_lines, parsingGcode


def _read_chunk(fh, n):
    rows, eof = [], False
    for _ in range(n):
        line = fh.readline()
        if line == "":
            eof = True
            break
        rows.append([float(x) for x in line.split(",")])
    return np.asarray(rows, dtype=np.float64).reshape(-1, 7), eof


class AccumStore:
    """Melt-time records over Level 0 (go_melt.py:86-92): accumulated time above
    liquidus and its maximum over separate melt events, device float arrays."""

    def __init__(self, engine):
        n = engine.geo.L0_nn
        self.e = engine
        self.accum = torch.zeros(n, dtype=engine.dtype, device=engine.dev)
        self.max_accum = torch.zeros(n, dtype=engine.dtype, device=engine.dev)

    def idx(self):
        """Level-0 node ids of the Level-3 window (Levels[0]["idx"]), formed on
        the device from the three per-axis index arrays."""
        g = self.e.geo
        x, y, z = (torch.as_tensor(np.asarray(a, dtype=np.int64), device=self.e.dev) for a in g.L0_overlap)
        nx, nxy = int(g.L0_nodes[0]), int(g.L0_nodes[0]) * int(g.L0_nodes[1])
        return (x[None, None, :] + y[None, :, None] * nx + z[:, None, None] * nxy).reshape(-1)


def go_melt(solver_input: dict, dtype=torch.float32, device="cuda"):
    tstart = time.time()
    names = ["L1", "L2", "L3"]
    Properties = SetupProperties(solver_input.get("properties", {}))
    Nonmesh = SetupNonmesh(solver_input.get("nonmesh", {}))
    Levels = SetupLevels(solver_input, Properties, dtype=dtype, device=device)
    eng = Levels.engine
    geo = eng.geo
    ne_nn = getStaticNodesAndElements(Levels)
    subcycle = getStaticSubcycle(Nonmesh)
    r12, r23 = geo.L1L2Eratio, geo.L2L3Eratio
    height = Properties["layer_height"]

    if Nonmesh["use_txt"]:
        total = count_lines(Nonmesh["toolpath"])
    else:
        total = parsingGcode(Nonmesh, Properties, geo.L[2].h)
    if not Properties["laser_center"]:
        with open(Nonmesh["toolpath"]) as f:
            laser_start = np.array([float(x) for x in f.readline().split(",")])
    else:
        laser_start = np.asarray(Properties["laser_center"], dtype=float)

    time_inc = record_inc = wait_inc = 0
    t_output = 0.0
    savenum = int(time_inc / Nonmesh["record_step"]) + 1
    saveResults(Levels, Nonmesh, savenum)
    laser_prev_z = float("inf")
    dwell_count = 0.0
    acc = AccumStore(eng)
    move_hist = [0, 0, 0]
    tmp_ne_nn = None
    substrate = None
    s1_storage = torch.zeros((geo.s1_storage_rows, geo.L[1].nn), dtype=torch.uint8, device=eng.dev)
    force_move = move_vert = new_checkpoint = False
    ongoing = True
    ckpt_dir = os.path.join(Nonmesh["save_path"], "checkpoint")
    layer_check = Nonmesh["layer_num"] + Nonmesh["restart_layer_num"]
    fh = open(Nonmesh["toolpath"], "r")
    load_chkpt = False
    if Nonmesh["layer_num"] > 0:
        name = os.path.join(ckpt_dir, f"Checkpoint{str(Nonmesh['layer_num']).zfill(4)}.pkl")
        with open(name, "rb") as f:
            st = pickle.load(f)
        restore_state(eng, acc, st, s1_storage)
        record_inc = st["record_inc"]
        line_len = len(fh.readline())
        fh.seek(st["time_inc"] * line_len)
        time_inc += st["time_inc"]
        load_chkpt = True
    n23 = subcycle[0] * subcycle[1]

    while ongoing:
        t_loop = time.time()
        laser_all, eof = _read_chunk(fh, n23)
        t_add = subcycle[2]
        if eof:
            t_add = laser_all.shape[0]
            ongoing = False
            if t_add == 0:
                break
        jumps = False
        if laser_all.shape[0] > 1:
            jumps = bool((np.abs(np.diff(laser_all, axis=0)[:, :2] / laser_all[:-1, 5].max())
                          > 100 * Nonmesh["laser_velocity"]).any())
        single = (bool((laser_all[:, 2] != laser_prev_z).any()) or load_chkpt
                  or wait_inc > max(0, Nonmesh["wait_time"] - n23 * 2) or not ongoing
                  or laser_all.shape[0] == 1 or jumps)
        if single:
            for lp in laser_all:
                wait_inc = wait_inc + 1 if lp[4] == 0 else 0
                if lp[2] != laser_prev_z and time_inc > 0 and not load_chkpt:
                    new_checkpoint = True
                if lp[2] != laser_prev_z:
                    z_new, sidx = geo.layer_shift_L1(lp[2])
                    if not load_chkpt:
                        shift_level1(eng, z_new, sidx, s1_storage)
                    tmp_ne_nn = calcStaticTmpNodesAndElements(Levels, lp)
                    eng.tmp = tmp_ne_nn
                    laser_prev_z = lp[2]
                    force_move = True
                    wait_inc = 0
                    move_vert = True
                    if not load_chkpt:
                        save_accum(acc, Nonmesh)
                        shift_level0(eng, acc, lp[2])
                force_move = True
                if force_move:
                    force_move = False
                    Levels, _, _, move_hist = moveEverything(lp, laser_start, Levels, move_hist, None, r12, r23,
                                                             height)
                    if move_vert:
                        move_vert = False
                        substrate = getSubstrateNodes(Levels)
                        eng.substrate = substrate
                        eng.l0_fill(0, substrate[0], 1)
                if wait_inc <= Nonmesh["wait_time"]:
                    Levels, reset = stepGOMELT(Levels, ne_nn, tmp_ne_nn, None, None, lp, Properties, lp[5], lp[6],
                                               substrate)
                    if Nonmesh["info_T"]:
                        print(f"Step {time_inc + 1} / {total}")
                        printLevelMaxMin(Levels, names)
                    i0 = acc.idx()
                    racc = acc.accum[i0] * reset.to(acc.accum.dtype)
                    acc.max_accum[i0] = torch.maximum(racc, acc.max_accum[i0])
                    acc.accum[i0] -= racc
                    acc.accum[i0] += (eng.T[3] > Properties["T_liquidus"]).to(acc.accum.dtype) * float(lp[5])
                else:
                    if not bool((eng.Tp[2] == 0).all()) and not bool((eng.Tp[3] == 0).all()):
                        dwell_count = Nonmesh["wait_time"] * Nonmesh["timestep_L3"]
                        eng.Tp[2].zero_()
                        eng.Tp[3].zero_()
                    Levels = stepGOMELTDwellTime(Levels, tmp_ne_nn, ne_nn, Properties, lp[5], substrate)
                    dwell_count += lp[5]
                    print(f"Dwell Time {dwell_count:.6f} s")
                time_inc += 1
                record_inc += 1
            if new_checkpoint:
                Nonmesh["layer_num"] += 1
                print(f"Saving checkpoint for Layer {Nonmesh['layer_num']}")
                os.makedirs(ckpt_dir, exist_ok=True)
                name = os.path.join(ckpt_dir, f"Checkpoint{str(Nonmesh['layer_num']).zfill(4)}.pkl")
                with open(name, "wb") as f:
                    pickle.dump(snapshot_state(eng, acc, time_inc, record_inc, s1_storage), f,
                                pickle.HIGHEST_PROTOCOL)
                if Nonmesh["layer_num"] == layer_check:
                    fh.close()
                    return Levels
                new_checkpoint = False
                load_chkpt = True
            else:
                load_chkpt = False
        else:
            wait_inc = (wait_inc + len(laser_all) - laser_all[:, 4].sum()) if (laser_all[:, 4] == 0).any() else 0
            Levels, Shapes, LInterp, move_hist = moveEverything(laser_all[0], laser_start, Levels, move_hist, None,
                                                                r12, r23, height)
            i0 = acc.idx()
            Levels, _, _, _, macc, a = subcycleGOMELT(Levels, ne_nn, Shapes, substrate, LInterp, tmp_ne_nn,
                                                       laser_all, Properties, laser_all[:, 6], subcycle,
                                                       acc.max_accum[i0], acc.accum[i0], history=False)
            acc.max_accum[i0] = macc
            acc.accum[i0] = a
            time_inc += t_add
            record_inc += t_add
        t_output += float(laser_all[:, 5].sum())
        if record_inc >= Nonmesh["record_step"]:
            record_inc = 0
            savenum = int(time_inc / Nonmesh["record_step"]) + 1
            saveResults(Levels, Nonmesh, savenum)
        if Nonmesh["info_T"]:
            printLevelMaxMin(Levels, names)
        tend = time.time()
        print("%d/%d, Real: %.6f s, Wall: %.2f s, Loop: %5.2f ms, Avg: %5.2f ms/dt"
              % (time_inc, total, t_output, tend - tstart, 1000 * (tend - t_loop),
                 1000 * (tend - tstart) / max(time_inc, 1)))
    fh.close()
    saveState(Levels[0], "Level0_", Nonmesh["layer_num"], Nonmesh["save_path"], 0)
    saveResultsFinal(Levels, Nonmesh)
    T = {lv: eng.T[lv].double().cpu().numpy() for lv in (1, 2, 3)}
    np.savez(os.path.join(Nonmesh["save_path"], "FinalTemperatureFields"), L1T=T[1], L2T=T[2], L3T=T[3])
    save_accum(acc, Nonmesh)
    print("End of simulation")
    return Levels


def shift_level1(eng, z_new, sidx, s1_storage):
    """New layer (go_melt.py:206-234): Level-1 temperature re-sampled on the
    z-shifted mesh (clamped to T_amb), S1 rows swapped with the layer store."""
    import kern
    from geometry import axis_map

    L1 = eng.geo.L[1]
    new = [L1.coords[0], L1.coords[1], z_new]
    m = kern.DeviceMap3([axis_map(L1.coords[d], new[d]) for d in range(3)], L1.nodes, eng.dtype, eng.dev)
    out = torch.empty_like(eng.T[1])
    eng._interp([(m, eng.T[1], 1.0)], L1.nodes, out)
    eng._clamp(out)
    eng.T[1].copy_(out)
    # the reference indexes its JAX S1_storage: an update at a row outside the
    # store is dropped, a read outside it takes the nearest row
    rows = s1_storage.shape[0]
    s1 = (eng.ph[1] & 1)
    if -rows <= sidx - 1 < rows:
        s1_storage[sidx - 1].copy_(s1)
    eng.ph[1].copy_((eng.ph[1] & 2) | s1_storage[min(max(sidx, 0), rows - 1)])
    L1.coords = [L1.coords[0], L1.coords[1], np.asarray(z_new, dtype=float)]


def shift_level0(eng, acc, laser_z):
    """New layer (go_melt.py:258-296): Level-0 S1 and the melt-time record move
    down by layer_idx_delta planes; Level-0 z coordinates follow the laser."""
    g = eng.geo
    nxy = g.L0_nodes[0] * g.L0_nodes[1]
    n1 = nxy * g.layer_idx_delta
    n2 = nxy * (g.L0_nodes[2] - g.layer_idx_delta)
    wpl = ((g.L0_nodes[0] + 31) // 32) * g.L0_nodes[1]  # words of one Level-0 plane in the bit store
    w1, w2 = wpl * g.layer_idx_delta, wpl * (g.L0_nodes[2] - g.layer_idx_delta)
    eng.L0[:w2] = eng.L0[w1:].clone()
    eng.L0[w2:] = 0
    g.L0_coords[2] = g.L0_orig_coords[2] + laser_z - g.L0_orig_coords[2][-1]
    acc.max_accum.zero_()
    acc.accum[:n2] = acc.accum[n1:].clone()
    acc.accum[n2:] = 0


def save_accum(acc, Nonmesh):
    """The layer's melt-time record (go_melt.py:246-256), in the engine's precision."""
    a = torch.maximum(acc.accum, acc.max_accum)
    acc.accum.copy_(a)
    np.savez(os.path.join(Nonmesh["save_path"], "accum_time" + str(Nonmesh["layer_num"]).zfill(4)),
             accum_time=a.cpu().numpy())


def snapshot_state(eng, acc, time_inc, record_inc, s1_storage):
    """Host copy of everything the reference's checkpoint holds (Levels with
    its Level-1 S1 layer store, the melt-time records, time and record
    counters; go_melt.py:390-411)."""
    g = eng.geo
    st = {"time_inc": time_inc, "record_inc": record_inc, "s1_storage": s1_storage.cpu(),
          "T": {k: v.cpu() for k, v in eng.T.items()}, "Tp": {k: v.cpu() for k, v in eng.Tp.items()},
          "ph": {k: v.cpu() for k, v in eng.ph.items()}, "L0": eng.L0.cpu(), "accum": acc.accum.cpu(),
          "max_accum": acc.max_accum.cpu(), "s2_prev_lo": eng.s2_prev_lo,
          "coords": {lv: [c.copy() for c in g.L[lv].coords] for lv in (1, 2, 3)},
          "overlap": {lv: ([a.copy() for a in g.L[lv].overlap_nodes], [a.copy() for a in g.L[lv].overlap_coords])
                      for lv in (2, 3)},
          "L0_overlap": ([a.copy() for a in g.L0_overlap], [a.copy() for a in g.L0_overlap_L2]),
          "L0_coords": [c.copy() for c in g.L0_coords]}
    return st


def restore_state(eng, acc, st, s1_storage):
    g = eng.geo
    s1_storage.copy_(st["s1_storage"].to(eng.dev))
    for k, v in st["T"].items():
        eng.T[k].copy_(v.to(eng.dev))
    for k, v in st["Tp"].items():
        eng.Tp[k].copy_(v.to(eng.dev))
    for k, v in st["ph"].items():
        eng.ph[k].copy_(v.to(eng.dev))
    eng.L0.copy_(st["L0"].to(eng.dev))
    acc.accum.copy_(st["accum"].to(eng.dev))
    acc.max_accum.copy_(st["max_accum"].to(eng.dev))
    eng.s2_prev_lo = st["s2_prev_lo"]
    for lv in (1, 2, 3):
        g.L[lv].coords = st["coords"][lv]
    for lv in (2, 3):
        g.L[lv].overlap_nodes, g.L[lv].overlap_coords = st["overlap"][lv]
    g.L0_overlap, g.L0_overlap_L2 = st["L0_overlap"]
    g.L0_coords = st["L0_coords"]
    eng.build_tables()


if __name__ == "__main__":
    dev_id = int(sys.argv[1]) if len(sys.argv) > 1 and sys.argv[1].isdigit() else 0
    input_file = sys.argv[2] if len(sys.argv) > 2 else "examples/example.json"
    try:
        with open(input_file) as f:
            solver_input = json.load(f)
    except FileNotFoundError:
        print(f"Error: Input file '{input_file}' not found.")
        sys.exit(1)
    print("Running GO-MELT (GB300)")
    print(f"GPU: {dev_id}, Input File: {input_file}")
    go_melt(solver_input, device=f"cuda:{dev_id}")
