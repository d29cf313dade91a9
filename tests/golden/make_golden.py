"""Generate golden vectors by running the unmodified GO-MELT reference.

Run with ``--reference <GO-MELT checkout>`` (or the environment variable
GOMELT_REFERENCE naming it); the sources are only read.  JAX 0.4.16, which the
reference pins, is not installed, so ``oracle/jaxshim.py`` supplies a NumPy
(FP64) implementation of the JAX primitives the reference uses; the
reference's own ``computeFunctions.py`` / ``go_melt.py`` run unchanged on top.

For each case this script runs the reference driver ``go_melt()`` on a tiny
three-level configuration and G-code, and records:

* the toolpath file the reference wrote (``createPath.parsingGcode``);
* state snapshots before/after the first calls of ``moveEverything``,
  ``stepGOMELT``, ``subcycleGOMELT`` and ``stepGOMELTDwellTime``;
* the final temperature fields and the melt-time arrays the driver saves;
* unit vectors for single functions evaluated on perturbed states.

Usage: python tests/golden/make_golden.py [--reference DIR] [--out DIR]
"""

from __future__ import annotations

import argparse
import copy
import json
import os
import shutil
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))

import jaxshim  # noqa: E402
import stateio  # noqa: E402


# ---------------------------------------------------------------------------
# Cases (tiny meshes so the reference's per-element Python loops stay fast)
# ---------------------------------------------------------------------------
CONST_PROPS = {
    # Material of the benchmark workloads: constant k=22 W/mK, rho=4400 kg/m^3,
    # cp=700 J/kgK in every phase; convection + radiation, no evaporation.
    "thermal_conductivity_powder": 22.0,
    "thermal_conductivity_bulk_a0": 22.0,
    "thermal_conductivity_bulk_a1": 0.0,
    "thermal_conductivity_fluid_a0": 22.0,
    "heat_capacity_solid_a0": 700.0,
    "heat_capacity_solid_a1": 0.0,
    "heat_capacity_mushy": 700.0,
    "heat_capacity_fluid": 700.0,
    "density": 4.4e-6,
    "laser_radius": 0.05,
    "laser_depth": 0.05,
    "laser_power": 200.0,
    "laser_absorptivity": 0.35,
    "T_amb": 300.0,
    "T_solidus": 1878.0,
    "T_liquidus": 1900.0,
    "h_conv": 1e-5,
    "emissivity": 0.3,
    "evaporation_coefficient": 0.0,
    "layer_height": 0.05,
}

PHASE_PROPS = {
    # Temperature- and phase-dependent material with evaporation (the values
    # of the reference's examples/example.json).
    "thermal_conductivity_powder": 0.4,
    "thermal_conductivity_bulk_a0": 4.23,
    "thermal_conductivity_bulk_a1": 0.016,
    "thermal_conductivity_fluid_a0": 29.0,
    "heat_capacity_solid_a0": 383.1,
    "heat_capacity_solid_a1": 0.174,
    "heat_capacity_mushy": 3235.0,
    "heat_capacity_fluid": 769.0,
    "density": 8e-06,
    "laser_radius": 0.04,
    "laser_depth": 0.03,
    "laser_power": 250.0,
    "laser_absorptivity": 0.45,
    "T_amb": 298.15,
    "T_solidus": 1533,
    "T_liquidus": 1609,
    "T_boiling": 3038.0,
    "h_conv": 1.5e-05,
    "emissivity": 0.3,
    "evaporation_coefficient": 0.82,
    "boltzmann_constant": 1.38e-23,
    "atomic_mass": 9.746e-26,
    "latent_heat_evap": 6457000.0,
    "molar_mass": 58.69,
    "layer_height": 0.05,
}


def case_track_const():
    cfg = {
        "Level1": {
            "elements": [10, 10, 5],
            "bounds": {"x": [0, 1.0], "y": [0, 1.0], "z": [-0.5, 0]},
            "conditions": {"x": [300, 300], "y": [300, 300], "z": [300, 300]},
        },
        "Level2": {"elements": [8, 8, 4], "bounds": {"x": [0.3, 0.7], "y": [0.3, 0.7], "z": [-0.2, 0]}},
        "Level3": {"elements": [8, 8, 4], "bounds": {"x": [0.4, 0.6], "y": [0.4, 0.6], "z": [-0.1, 0]}},
        "properties": dict(CONST_PROPS, laser_center=[0.5, 0.5, 0, 0, 0, 0, 0]),
        "nonmesh": {
            "timestep_L3": 1e-5, "subcycle_num_L2": 2, "subcycle_num_L3": 2,
            "output_files": 0, "wait_time": 4, "dwell_time": 2e-4, "laser_velocity": 1000,
            "info_T": 0, "dwell_time_multiplier": 1,
        },
    }
    gcode = "G0 X0.42 Y0.5 Z0.0\nG1 X0.58 Y0.47 Z0.0\n"
    return cfg, gcode


def case_phase_powder():
    # Temperature-dependent material, evaporation on, one powder layer on top
    # of the substrate (inactive Level-1 layers above it), anisotropic fine
    # level, N2 != N3.
    cfg = {
        "Level1": {
            "elements": [10, 8, 8],
            "bounds": {"x": [0, 1.0], "y": [0, 0.8], "z": [-0.5, 0.3]},
            "conditions": {"x": [298.15, 305.0], "y": [301.0, 298.15], "z": [298.15, 298.15]},
        },
        "Level2": {"elements": [8, 8, 4], "bounds": {"x": [0.3, 0.7], "y": [0.2, 0.6], "z": [-0.2, 0]}},
        "Level3": {"elements": [8, 8, 4], "bounds": {"x": [0.45, 0.55], "y": [0.35, 0.45], "z": [-0.1, 0]}},
        "properties": dict(PHASE_PROPS, laser_center=[0.5, 0.4, 0, 0, 0, 0, 0]),
        "nonmesh": {
            "timestep_L3": 4e-6, "subcycle_num_L2": 3, "subcycle_num_L3": 2,
            "output_files": 0, "wait_time": 3, "dwell_time": 6e-5, "laser_velocity": 800,
            "info_T": 0, "dwell_time_multiplier": 1,
        },
    }
    gcode = "G0 X0.47 Y0.41 Z0.05\nG1 X0.53 Y0.39 Z0.05\n"
    return cfg, gcode


def case_two_layers():
    # Two layers: exercises the layer change (Level-1 z shift, S1_storage,
    # Level-0 shift, checkpoint) between tracks.
    cfg = {
        "Level1": {
            "elements": [10, 10, 8],
            "bounds": {"x": [0, 1.0], "y": [0, 1.0], "z": [-0.5, 0.3]},
            "conditions": {"x": [300, 300], "y": [300, 300], "z": [300, 300]},
        },
        "Level2": {"elements": [8, 8, 4], "bounds": {"x": [0.3, 0.7], "y": [0.3, 0.7], "z": [-0.2, 0]}},
        "Level3": {"elements": [8, 8, 4], "bounds": {"x": [0.4, 0.6], "y": [0.4, 0.6], "z": [-0.1, 0]}},
        "properties": dict(CONST_PROPS, laser_center=[0.5, 0.5, 0, 0, 0, 0, 0], T_solidus=700.0,
                           T_liquidus=800.0),
        "nonmesh": {
            "timestep_L3": 1e-5, "subcycle_num_L2": 2, "subcycle_num_L3": 2,
            "output_files": 0, "wait_time": 2, "dwell_time": 4e-5, "laser_velocity": 1000,
            "info_T": 0, "dwell_time_multiplier": 1,
        },
    }
    gcode = ("G0 X0.44 Y0.5 Z0.05\nG1 X0.52 Y0.5 Z0.05\n"
             "G0 X0.52 Y0.48 Z0.1\nG1 X0.44 Y0.48 Z0.1\n")
    return cfg, gcode


CASES = {
    "track_const": case_track_const,
    "phase_powder": case_phase_powder,
    "two_layers": case_two_layers,
}


# ---------------------------------------------------------------------------
# Recording wrappers
# ---------------------------------------------------------------------------
class Recorder:
    def __init__(self, store: dict, max_calls: int = 2):
        self.store = store
        self.max_calls = max_calls
        self.count = {}

    def wrap(self, name, fn, in_names, out_names, skip_in=(), skip_out=()):
        def inner(*args):
            n = self.count.get(name, 0)
            self.count[name] = n + 1
            rec = n < self.max_calls
            if rec:
                for a_name, a in zip(in_names, args):
                    if a_name in skip_in:
                        continue
                    stateio.flatten(copy.deepcopy(a), f"{name}{n}.in.{a_name}", self.store)
            out = fn(*args)
            if rec:
                outs = out if isinstance(out, tuple) else (out,)
                for o_name, o in zip(out_names, outs):
                    if o_name in skip_out:
                        continue
                    if o_name == "Shapes":
                        for i, s in enumerate(o):
                            stateio.flatten([s[0], s[1]], f"{name}{n}.out.Shapes#{i}", self.store)
                            self.store[f"{name}{n}.out.Shapes#{i}.bcoo"] = np.asarray(s[2].indices)
                        continue
                    stateio.flatten(copy.deepcopy(o), f"{name}{n}.out.{o_name}", self.store)
            return out

        return inner


def run_case(name, make, ref_dir, out_dir):
    cfg, gcode = make()
    work = tempfile.mkdtemp(prefix=f"gm_golden_{name}_")
    gpath = os.path.join(work, "path.gcode")
    with open(gpath, "w") as f:
        f.write(gcode)
    cfg = copy.deepcopy(cfg)
    cfg["nonmesh"]["gcode"] = gpath
    cfg["nonmesh"]["save_path"] = os.path.join(work, "out") + "/"
    cfg["nonmesh"]["toolpath"] = os.path.join(work, "toolpath.txt")

    import go_melt as gm  # reference driver (imported after jaxshim.install)
    import computeFunctions as cf

    store: dict = {}
    rec = Recorder(store)
    orig = {k: getattr(gm, k) for k in ("moveEverything", "subcycleGOMELT", "stepGOMELT",
                                         "stepGOMELTDwellTime")}
    gm.moveEverything = rec.wrap(
        "move", orig["moveEverything"],
        ["v", "vstart", "Levels", "move_v", "LInterp", "L1L2Eratio", "L2L3Eratio", "height"],
        ["Levels", "Shapes", "LInterp", "move_v"], skip_in=("LInterp",))
    gm.subcycleGOMELT = rec.wrap(
        "sub", orig["subcycleGOMELT"],
        ["Levels", "ne_nn", "Shapes", "substrate", "LInterp", "tmp_ne_nn", "laser_position",
         "properties", "laserP", "subcycle", "max_accum_L3", "accum_L3"],
        ["Levels", "L2all", "L3all", "L3pall", "max_accum", "accum"],
        skip_in=("Shapes", "LInterp", "properties"))
    gm.stepGOMELT = rec.wrap(
        "step", orig["stepGOMELT"],
        ["Levels", "ne_nn", "tmp_ne_nn", "Shapes", "LInterp", "v", "properties", "dt", "laserP",
         "substrate"],
        ["Levels", "resetmask"], skip_in=("Shapes", "LInterp", "properties"))
    gm.stepGOMELTDwellTime = rec.wrap(
        "dwell", orig["stepGOMELTDwellTime"],
        ["Levels", "tmp_ne_nn", "ne_nn", "properties", "dt", "substrate"],
        ["Levels"], skip_in=("properties",))

    t0 = time.time()
    cwd = os.getcwd()
    os.chdir(work)
    try:
        gm.go_melt(copy.deepcopy(cfg))
    finally:
        os.chdir(cwd)
        for k, v in orig.items():
            setattr(gm, k, v)
    print(f"[{name}] reference driver ran in {time.time() - t0:.1f} s; calls {rec.count}")

    with open(cfg["nonmesh"]["toolpath"]) as f:
        store["toolpath_txt"] = np.asarray(f.read())
    store["cfg_json"] = np.asarray(json.dumps(cfg))
    store["gcode"] = np.asarray(gcode)
    fin = np.load(os.path.join(cfg["nonmesh"]["save_path"], "FinalTemperatureFields.npz"))
    for k in fin.files:
        store[f"final.{k}"] = fin[k]
    acc_files = sorted(f for f in os.listdir(cfg["nonmesh"]["save_path"]) if f.startswith("accum_time"))
    for fname in acc_files:
        a = np.load(os.path.join(cfg["nonmesh"]["save_path"], fname))
        store[f"final.{fname[:-4]}"] = a["accum_time"]
    props = cf.SetupProperties(copy.deepcopy(cfg["properties"]))
    stateio.flatten(props, "properties", store)

    unit_vectors(name, cf, cfg, props, store)

    path = os.path.join(out_dir, f"{name}.npz")
    np.savez_compressed(path, **store)
    print(f"[{name}] wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB, {len(store)} arrays)")
    shutil.rmtree(work, ignore_errors=True)


# ---------------------------------------------------------------------------
# Unit vectors: single reference functions on perturbed states
# ---------------------------------------------------------------------------
def unit_vectors(name, cf, cfg, props, store):
    rng = np.random.default_rng(1234)
    L = cf.SetupLevels(copy.deepcopy(cfg), props)
    Nonmesh = cfg["nonmesh"]
    # Move the windows to a non-trivial place (negative x move, positive y).
    vstart = np.array(cfg["properties"]["laser_center"], dtype=float)
    v = vstart + np.array([-0.061, 0.043, 0.0, 0, 0, 0, 0])
    L1L2E = [int(np.round(L[1]["h"][i] / L[2]["h"][i])) for i in range(2)] + [
        int(np.round(props["layer_height"] / L[2]["h"][2]))]
    L2L3E = [int(np.round(L[2]["h"][i] / L[3]["h"][i])) for i in range(3)]
    L1L2I = cf.interpolatePointsMatrix(L[1], L[2]["node_coords"])
    L2L3I = cf.interpolatePointsMatrix(L[2], L[3]["node_coords"])
    # Give every level a smooth non-trivial temperature and subgrid field.
    for lev in (1, 2, 3):
        x, y, z = (np.asarray(c) for c in L[lev]["node_coords"])
        X = np.tile(x, len(y) * len(z))
        Y = np.repeat(np.tile(y, len(z)), len(x))
        Z = np.repeat(z, len(x) * len(y))
        T = props["T_amb"] + 1800 * np.exp(-((X - 0.5) ** 2 + (Y - 0.45) ** 2) / 0.02 + Z * 3)
        L[lev]["T0"] = jaxshim._w(T + 30 * rng.standard_normal(T.shape))
        if lev > 1:
            L[lev]["Tprime0"] = jaxshim._w(40 * np.sin(9 * X) * np.cos(7 * Y) * np.exp(Z))
    L[0]["S1"] = jaxshim._w((rng.random(np.asarray(L[0]["nn"]).item()) > 0.5).astype(float))
    L[0]["S2"] = jaxshim._w(rng.random(np.asarray(L[0]["nn"]).item()) > 0.8)
    stateio.flatten(copy.deepcopy(L), "u.move.in.Levels", store)
    store["u.move.in.v"] = v
    store["u.move.in.vstart"] = vstart
    Lm, Shapes, LInterp, move_v = cf.moveEverything(v, vstart, L, [0, 0, 0], [L1L2I, L2L3I], L1L2E,
                                                    L2L3E, props["layer_height"])
    stateio.flatten(copy.deepcopy(Lm), "u.move.out.Levels", store)
    stateio.flatten(LInterp, "u.move.out.LInterp", store)
    stateio.flatten(move_v, "u.move.out.move_v", store)
    for i, s in enumerate(Shapes):
        stateio.flatten([s[0], s[1]], f"u.move.out.Shapes#{i}", store)
        store[f"u.move.out.Shapes#{i}.bcoo"] = np.asarray(s[2].indices)

    L = Lm
    substrate = cf.getSubstrateNodes(L)
    ne_nn = cf.getStaticNodesAndElements(L)
    tmp_ne_nn = cf.calcStaticTmpNodesAndElements(L, v)
    store["u.substrate"] = np.asarray(substrate)
    store["u.tmp_ne_nn"] = np.asarray(tmp_ne_nn)
    store["u.ne_nn"] = np.asarray(ne_nn)

    # Phase / property update on a field that spans every phase.
    nn3 = int(np.asarray(L[3]["nn"]))
    Tph = jaxshim._w(rng.uniform(200.0, 3600.0, nn3))
    S1ph = jaxshim._w(rng.choice([0.0, 1.0, 0.3, 0.7, 0.499, 0.5], nn3))
    out = cf.computeStateProperties(Tph, S1ph, props, substrate[3] // 2)
    store["u.props.T"], store["u.props.S1"] = np.asarray(Tph), np.asarray(S1ph)
    store["u.props.substrate"] = np.asarray(substrate[3] // 2)
    for k, o in zip(("S1", "S2", "k", "rhocp"), out):
        store[f"u.props.out.{k}"] = np.asarray(o)

    # Fine-level source and surface flux.
    P = float(cfg["properties"]["laser_power"])
    store["u.src3.out"] = np.asarray(cf.computeSourcesL3(L[3], v, ne_nn, props, P))
    store["u.conv3.out"] = np.asarray(cf.computeConvRadBC(L[3], L[3]["T0"], ne_nn[1], ne_nn[4], props, 0))
    store["u.conv1.out"] = np.asarray(cf.computeConvRadBC(L[1], L[1]["T0"], tmp_ne_nn[0], ne_nn[2], props, 0))

    # Level solves with random positive properties and random RHS.
    for lev, nn, ne in ((3, ne_nn[4], ne_nn[1]), (1, ne_nn[2], tmp_ne_nn[0])):
        k = jaxshim._w(rng.uniform(0.005, 0.03, nn))
        rc = jaxshim._w(rng.uniform(0.002, 0.005, nn))
        F = jaxshim._w(rng.standard_normal(nn) * 1e-3)
        C = jaxshim._w(rng.standard_normal(nn) * 1e-4)
        dt = 3e-6
        Tn = cf.solveMatrixFreeFE(L[lev], nn, ne, k, rc, dt, L[lev]["T0"], F, C)
        for kk, a in (("k", k), ("rhocp", rc), ("F", F), ("Corr", C), ("out", Tn)):
            store[f"u.solve{lev}.{kk}"] = np.asarray(a)
        store[f"u.solve{lev}.dt"] = np.asarray(dt)

    # Prolongation tables and the full-field interpolation, with points partly
    # outside the source mesh (validity mask).
    xs = [np.asarray(c) for c in L[3]["node_coords"]]
    pts = [xs[0] + 0.13, xs[1] - 0.021, xs[2]]
    store["u.interp.pts"] = np.concatenate(pts)
    store["u.interp.pts_len"] = np.asarray([len(p) for p in pts])
    Mi = cf.interpolatePointsMatrix(L[2], [jaxshim._w(p) for p in pts])
    store["u.interp.Nc"], store["u.interp.node"] = np.asarray(Mi[0]), np.asarray(Mi[1])
    store["u.interp.out"] = np.asarray(cf.interpolatePoints(L[2], L[2]["T0"], [jaxshim._w(p) for p in pts]))

    # Restriction + T'.
    Tp, Tc = cf.getNewTprime(L[3], L[3]["T0"], L[2]["T0"], L[2], LInterp[1])
    store["u.tprime.Tp"], store["u.tprime.Tc"] = np.asarray(Tp), np.asarray(Tc)

    # Coarse source projection (several laser positions) and subgrid terms.
    npos = 3
    lp = np.tile(v, (npos, 1))
    lp[:, 0] += np.array([0.0, 0.004, 0.009])
    lp[:, 1] += np.array([0.0, -0.002, 0.001])
    lp[:, 5] = np.array([1e-5, 1.1e-5, 0.9e-5])
    lP = np.array([P, 0.5 * P, 0.0])
    store["u.lsrc.lp"], store["u.lsrc.lP"] = lp, lP
    store["u.lsrc.out1"] = np.asarray(cf.computeLevelSource(L, ne_nn, jaxshim._w(lp), Shapes[1], props, jaxshim._w(lP)))
    store["u.lsrc.out2"] = np.asarray(cf.computeLevelSource(L, ne_nn, jaxshim._w(lp), Shapes[2], props, jaxshim._w(lP)))
    _, _, k3, rc3 = cf.computeStateProperties(L[3]["T0"], L[3]["S1"], props, substrate[3])
    _, _, k2, rc2 = cf.computeStateProperties(L[2]["T0"], L[2]["S1"], props, substrate[2])
    store["u.tp1.L1"] = np.asarray(cf.computeL1TprimeTerms_Part1(L, ne_nn, k3, Shapes, k2))
    store["u.tp1.L2"] = np.asarray(cf.computeL2TprimeTerms_Part1(L, ne_nn, L[3]["Tprime0"], k3, Shapes))
    Tp3n = jaxshim._w(np.asarray(L[3]["Tprime0"]) + 5 * rng.standard_normal(nn3))
    Tp2n = jaxshim._w(np.asarray(L[2]["Tprime0"]) + 5 * rng.standard_normal(int(np.asarray(L[2]["nn"]))))
    store["u.tp2.Tp3n"], store["u.tp2.Tp2n"] = np.asarray(Tp3n), np.asarray(Tp2n)
    store["u.tp2.L1"] = np.asarray(cf.computeL1TprimeTerms_Part2(L, ne_nn, Tp3n, Tp2n, rc3, rc2, 2e-5, Shapes,
                                                                  jaxshim._w(np.zeros(ne_nn[2]))))
    store["u.tp2.L2"] = np.asarray(cf.computeL2TprimeTerms_Part2(L, ne_nn, Tp3n, L[3]["Tprime0"], rc3, 2e-5, Shapes,
                                                                  jaxshim._w(np.zeros(ne_nn[3]))))
    stateio.flatten(copy.deepcopy(L), "u.state", store)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("GOMELT_REFERENCE"),
                    help="a checkout of JLnorthwestern/GO-MELT (default: $GOMELT_REFERENCE)")
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--cases", default=",".join(CASES))
    args = ap.parse_args()
    if not args.reference:
        ap.error("name the reference checkout with --reference or GOMELT_REFERENCE")
    jaxshim.install()
    sys.path.insert(0, os.path.join(args.reference, "go_melt"))
    for name in args.cases.split(","):
        run_case(name, CASES[name], args.reference, args.out)


if __name__ == "__main__":
    main()
