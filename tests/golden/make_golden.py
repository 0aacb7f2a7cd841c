"""Regenerate the golden fixtures in this folder from the reference's regtests.

Run in a container that holds the reference tree:

    python tests/golden/make_golden.py [/path/to/plumed2]

It only READS the reference's regtest inputs and expected outputs (the
``*.reference`` files) and stores them, reshaped, as JSON next to this script,
so that the tests run where the reference tree is absent.  Sources:

* regtest/basic/rt20-switch-*           two-atom COORDINATION over
  regtest/trajectories/switchtraj.xyz: COLVAR.reference, deriv.reference
* regtest/basic/rt-make-switch          out_*.reference (value, derivative
  at 10 points per switch type, stretched and not)
* regtest/basic/rt42, rt42c             108-atom COORDINATION in a triclinic
  box: check_{c,e,g}.reference, colvar.reference, ff.reference
  (forces and virial of a RESTRAINT with SLOPE=1 on c+d)
* regtest/basic/rt42b                   GROUPA=GROUPB=1-108 R_0=1 over a .gro
  trajectory with triclinic boxes: colvar.reference (%8.4f), every 9th frame
* regtest/basic/rt-mpi0                 a two-list whose groups share atom 5,
  RATIONAL, EXP and GAUSSIAN over regtest/trajectories/trajectory.xyz:
  COLVAR.reference (%6.3f), deriv.reference (EXP and GAUSSIAN, %8.4f),
  ff.0.reference (forces and virial diagonal of RESTRAINT KAPPA=5 AT=15 on
  the RATIONAL one, %f)
* regtest/basic/rt42-cells{,-cos,-gauss}  108 atoms, GROUPA=GROUPB=1-108,
  NLIST against NLISTCELLS (NL_STRIDE=4, NL_CUTOFF=2.0) for RATIONAL D_MAX=1.5,
  COSINUS and GAUSSIAN D_MAX=1.5: check_diff.reference (d - c at %8.4f) and
  ff.reference (forces of SLOPE=0.001 on d - c at %10.5f, all zero)
* plugins/cudaCoord/regtest/{cudatest,cudatestPair,cudatestWB}/rt-*  the
  reference's CUDA plugin against COORDINATION on the same input: the
  COORDINATION line (@mdatoms written as the trajectory's atom range),
  colvar.reference (gpu - cpu at %8.4f), deriv_delta.reference (at %8.5f),
  over trajectories/traj-{nopbc,ortho}.xyz.  The two rt-double-bigbox cases
  are left out: their trajectory is written by `plumed benchmark` when the
  test runs and is not in the tree.
* regtest/tools/rt-make-CellLists      outputRequiredCells.reference and
  outputRequiredCellsNotOrtho.reference (cell counts and the cells searched
  from corner, edge, face and middle cells, with and without PBC),
  outputIndexes.reference (cell counts of three boxes at cutoff 1.5).  The
  boxes of the orthorhombic and the index parts are those of main.cpp
  (testRequiredCells, testIndexes); the other part prints its own.
* regtest/tools/rt-Neigbourlist         unitTest.reference / testNoNL.reference
  (exact neighbour sets on a simple-cubic lattice)
* regtest/basic/rt-dhenergy, rt-dhenergy2  DHENERGY between atoms 1-3 and 4-10
  of regtest/trajectories/trajectory.xyz, charges from test.pdb:
  COLVAR.reference, deriv.reference (rt-dhenergy2: UNITS CHARGE=0.1)
* regtest/basic/rt-ghbfix               GHBFIX PAIR of two atoms 0.002*i apart
  (the regtest's own generated trajectory), typesTable.dat and
  scalingParameters.dat as text: colvar.reference, der.reference
* regtest/symfunc/rt-dumpmulti          COORDINATIONNUMBER SPECIES=1-64 of
  regtest/trajectories/64.xyz: coordination.xyz.reference (per-atom values)
* regtest/symfunc/rt-single-groupb      COORDINATIONNUMBER SPECIESA=1-5
  SPECIESB=6 over trajectory.xyz: colvar.reference
* regtest/basic/rt28, rt72              CONTACTMAP (CMDIST and components over
  the regtest's trajectory.xyz; SUM of 278 Q contacts on trpcage.gro):
  colvar.reference, deriv.reference; the contacts are parsed from plumed.dat
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def read_xyz(path):
    frames, boxes = [], []
    with open(path) as f:
        lines = f.read().split("\n")
    i = 0
    while i < len(lines) and lines[i].strip():
        n = int(lines[i].split()[0])
        box = [float(x) for x in lines[i + 1].split()]
        pos = [[float(x) for x in lines[i + 2 + k].split()[1:4]] for k in range(n)]
        frames.append(pos)
        boxes.append(box)
        i += n + 2
    return frames, boxes


def read_gro(path, lines=None):
    """The first frame of a .gro file (or of the given lines)."""
    if lines is None:
        lines = open(path).read().split("\n")
    n = int(lines[1].split()[0])
    pos = [[float(lines[2 + k][20 + 8 * j:28 + 8 * j]) for j in range(3)] for k in range(n)]
    v = [float(x) for x in lines[2 + n].split()]
    if len(v) == 3:
        v += [0.0] * 6
    # v1(x) v2(y) v3(z) v1(y) v1(z) v2(x) v2(z) v3(x) v3(y): rows are lattice vectors
    box = [v[0], v[3], v[4], v[5], v[1], v[6], v[7], v[8], v[2]]
    return pos, box


def read_gro_frames(path):
    """Every frame of a .gro trajectory: title, atom count, atoms, box."""
    lines = open(path).read().split("\n")
    frames, boxes, i = [], [], 0
    while i + 1 < len(lines) and lines[i + 1].strip():
        n = int(lines[i + 1].split()[0])
        pos, box = read_gro(None, lines[i:i + n + 3])
        frames.append(pos)
        boxes.append(box)
        i += n + 3
    return frames, boxes


def contactmap_blocks(plumed_dat):
    """The CONTACTMAP ... blocks of a plumed.dat: label, flags, contacts."""
    text = open(plumed_dat).read()
    out = []
    for blk in re.findall(r"CONTACTMAP \.\.\.(.*?)\.\.\. CONTACTMAP", text, re.S):
        cm = {"label": re.search(r"LABEL=(\S+)", blk).group(1), "sum": bool(re.search(r"^\s*SUM\s*$", blk, re.M)),
              "cmdist": bool(re.search(r"^\s*CMDIST\s*$", blk, re.M)), "contacts": []}
        i = 1
        while True:
            m = re.search(r"ATOMS%d=(\d+),(\d+)" % i, blk)
            if not m:
                break
            sw = re.search(r"SWITCH%d=\{([^}]*)\}" % i, blk).group(1)
            ref = re.search(r"REFERENCE%d=(\S+)" % i, blk)
            w = re.search(r"WEIGHT%d=(\S+)" % i, blk)
            cm["contacts"].append({"atoms": [int(m.group(1)), int(m.group(2))], "switch": " ".join(sw.split()),
                                   "reference": float(ref.group(1)) if ref else 0.0,
                                   "weight": float(w.group(1)) if w else 1.0})
            i += 1
        out.append(cm)
    return out


def read_table(path):
    rows = []
    with open(path) as f:
        for line in f:
            if line.startswith("#"):
                continue
            if line.strip():
                rows.append([float(x) for x in line.split()])
    return rows


def switch_defs(plumed_dat):
    out = {}
    for line in open(plumed_dat):
        m = re.match(r"\s*(\w+):\s*COORDINATION\s+GROUPA=1\s+GROUPB=2\s+SWITCH=\{([^}]*)\}(.*)", line)
        if m and "NUMERICAL_DERIVATIVES" not in m.group(3):
            out[m.group(1)] = " ".join(m.group(2).split())
    return out


def main(ref):
    reg = os.path.join(ref, "regtest")
    # --- rt20-switch-* -----------------------------------------------------
    traj, boxes = read_xyz(os.path.join(reg, "trajectories", "switchtraj.xyz"))
    cases = {}
    for name in sorted(os.listdir(os.path.join(reg, "basic"))):
        if not name.startswith("rt20-switch-") or name in ("rt20-switch-lepton",):
            continue
        d = os.path.join(reg, "basic", name)
        defs = switch_defs(os.path.join(d, "plumed.dat"))
        if set(defs) != {"c", "cs"}:
            continue
        cases[name] = {"c": defs["c"], "cs": defs["cs"],
                       "colvar": read_table(os.path.join(d, "COLVAR.reference")),
                       "deriv": read_table(os.path.join(d, "deriv.reference"))}
    json.dump({"source": "regtest/basic/rt20-switch-*, regtest/trajectories/switchtraj.xyz",
               "traj": traj, "box": boxes, "cases": cases},
              open(os.path.join(HERE, "rt20_switch.json"), "w"))

    # --- rt-make-switch ----------------------------------------------------
    src = open(os.path.join(reg, "basic", "rt-make-switch", "main.cpp")).read()
    triples = re.findall(r'"([^"]+)",\s*(?://[^\n]*\n\s*)?"[^"]+",\s*"([^"]+)"', src)
    table = {}
    for definition, name in triples:
        for stretch in (True, False):
            fn = "out_%s%s.reference" % (name, "" if stretch else "_nostretch")
            p = os.path.join(reg, "basic", "rt-make-switch", fn)
            if not os.path.exists(p):
                continue
            rows = []
            for line in open(p):
                if ":" not in line or line.startswith("point"):
                    continue
                a, b = line.split(":")
                v = b.split()
                rows.append([float(a), float(v[0]), float(v[1])])
            table[fn] = {"definition": definition + ("" if stretch else " NOSTRETCH"), "rows": rows}
    json.dump({"source": "regtest/basic/rt-make-switch/out_*.reference (value, deriv at 6 decimals)",
               "cases": table}, open(os.path.join(HERE, "rt_make_switch.json"), "w"))

    # --- rt42 / rt42c ------------------------------------------------------
    d42 = os.path.join(reg, "basic", "rt42")
    frames, boxes = read_xyz(os.path.join(d42, "trajectory.xyz"))
    keep = list(range(0, len(frames), 9))
    ff_lines = open(os.path.join(d42, "ff.reference")).read().split("\n")
    forces, virials = [], []
    i = 0
    while i < len(ff_lines) and ff_lines[i].strip():
        n = int(ff_lines[i])
        virials.append([float(x) for x in ff_lines[i + 1].split()])
        forces.append([[float(x) for x in ff_lines[i + 2 + k].split()[1:4]] for k in range(n)])
        i += n + 2
    checks = {}
    for lab in ("c", "e", "g"):
        checks[lab] = [r[1] for r in read_table(os.path.join(d42, "check_%s.reference" % lab))]
    colvar_c1 = [r[1] for r in read_table(os.path.join(reg, "basic", "rt42c", "colvar.reference"))]
    json.dump({"source": "regtest/basic/rt42 (plumed.dat, trajectory.xyz, check_*.reference, ff.reference) "
                         "and regtest/basic/rt42c/colvar.reference; every 9th frame",
               "frames": [frames[k] for k in keep], "box": [boxes[k] for k in keep],
               "c": [checks["c"][k] for k in keep], "e": [checks["e"][k] for k in keep],
               "g": [checks["g"][k] for k in keep], "c_single": [colvar_c1[k] for k in keep],
               "ff_forces": [forces[k] for k in keep], "ff_virial": [virials[k] for k in keep],
               "inputs": {"c": "R0SYNTAX 6 0 1.0 0.0 twolist", "d": "CUSTOM FUNC=1/(1+x^6) R_0=1",
                          "dfast": "CUSTOM FUNC=1/(1+x2^3) R_0=1",
                          "e": "R0SYNTAX 7 0 1.0 0.1 twolist", "f": "CUSTOM FUNC=1/(1+x^7) R_0=1 D_0=0.1",
                          "g": "EXP R_0=1", "h": "CUSTOM FUNC=exp(-x) R_0=1",
                          "c_single": "R0SYNTAX 6 0 1.0 0.0 single",
                          "forces": "-(dc+dd) - 0.001*(dc - 0.5 dd - 0.5 dfast + de - df + dg - dh)"}},
              open(os.path.join(HERE, "rt42.json"), "w"))

    # --- rt42b ---------------------------------------------------------------
    frames, boxes = read_gro_frames(os.path.join(reg, "basic", "rt42b", "trajectory.gro"))
    col = [r[1] for r in read_table(os.path.join(reg, "basic", "rt42b", "colvar.reference"))]
    keep = list(range(0, len(frames), 9))
    json.dump({"source": "regtest/basic/rt42b (plumed.dat, trajectory.gro, colvar.reference); every 9th frame",
               "line": "GROUPA=1-108 GROUPB=1-108 R_0=1", "frames": [frames[k] for k in keep],
               "box": [boxes[k] for k in keep], "c": [col[k] for k in keep], "fmt": "%8.4f"},
              open(os.path.join(HERE, "rt42b.json"), "w"))

    # --- rt-mpi0 -------------------------------------------------------------
    dm = os.path.join(reg, "basic", "rt-mpi0")
    frames, boxes = read_xyz(os.path.join(reg, "trajectories", "trajectory.xyz"))
    colvar = read_table(os.path.join(dm, "COLVAR.reference"))
    der = read_table(os.path.join(dm, "deriv.reference"))
    nd = len(der) // len(colvar)
    ffl, fforces, fvir, i = open(os.path.join(dm, "ff.0.reference")).read().split("\n"), [], [], 0
    while i < len(ffl) and ffl[i].strip():
        n = int(ffl[i])
        fvir.append([float(x) for x in ffl[i + 1].split()])
        fforces.append([[float(x) for x in ffl[i + 2 + k].split()[1:4]] for k in range(n)])
        i += n + 2
    json.dump({"source": "regtest/basic/rt-mpi0 (plumed.dat, COLVAR.reference, deriv.reference, ff.0.reference) "
                         "over regtest/trajectories/trajectory.xyz",
               "groupa": "1-10", "groupb": "30-40,5,50-100",
               "switch": {"c": "RATIONAL R_0=1.0", "cexp": "EXP R_0=0.7", "cgaus": "GAUSSIAN R_0=0.2 D_0=0.6"},
               "restraint": {"arg": "c", "kappa": 5.0, "at": 15.0},
               "frames": frames[:len(colvar)], "box": boxes[:len(colvar)],
               "colvar": [{"c": r[1], "cexp": r[2], "cgaus": r[3]} for r in colvar],
               "deriv_cexp": [[r[2] for r in der[f * nd:(f + 1) * nd]] for f in range(len(colvar))],
               "deriv_cgaus": [[r[3] for r in der[f * nd:(f + 1) * nd]] for f in range(len(colvar))],
               "ff_forces": fforces, "ff_virial_diag": fvir,
               "fmt": "COLVAR %6.3f, deriv %8.4f, forces and virial %f"},
              open(os.path.join(HERE, "rt_mpi0.json"), "w"))

    # --- rt42-cells, rt42-cells-cos, rt42-cells-gauss -------------------------
    variants = {}
    for name in ("rt42-cells", "rt42-cells-cos", "rt42-cells-gauss"):
        dd = os.path.join(reg, "basic", name)
        coord = {}
        for line in open(os.path.join(dd, "plumed.dat")):
            m = re.match(r"\s*(\w+):\s*COORDINATION\s+(.*\S)\s*$", line)
            if m:
                coord[m.group(1)] = " ".join(m.group(2).split())
        ff, lines, i = [], open(os.path.join(dd, "ff.reference")).read().split("\n"), 0
        while i < len(lines) and lines[i].strip():  # per frame: count, virial, one force line per atom
            n = int(lines[i])
            ff += [float(x) for x in lines[i + 1].split()]
            ff += [float(x) for k in range(n) for x in lines[i + 2 + k].split()[1:4]]
            i += n + 2
        variants[name] = {"c": coord["c"], "d": coord["d"],
                          "check_diff": [r[1] for r in read_table(os.path.join(dd, "check_diff.reference"))],
                          "ff_max_abs": max(abs(x) for x in ff)}
    frames, boxes = read_xyz(os.path.join(reg, "basic", "rt42-cells", "trajectory.xyz"))
    json.dump({"source": "regtest/basic/rt42-cells{,-cos,-gauss} (plumed.dat COORDINATION lines, trajectory.xyz "
                         "shared by the three, check_diff.reference, ff.reference)",
               "frames": frames, "box": boxes, "variants": variants,
               "fmt": "check_diff %8.4f; forces and virial %10.5f"},
              open(os.path.join(HERE, "rt42_cells.json"), "w"))

    # --- plugins/cudaCoord/regtest -------------------------------------------
    dcc = os.path.join(ref, "plugins", "cudaCoord", "regtest")
    trajs = {}
    for t in ("traj-nopbc.xyz", "traj-ortho.xyz"):
        fr, bx = read_xyz(os.path.join(dcc, "trajectories", t))
        # three numbers: an orthorhombic box given by its edges; stored as 3x3
        bx = [b if len(b) == 9 else [b[0], 0.0, 0.0, 0.0, b[1], 0.0, 0.0, 0.0, b[2]] for b in bx]
        trajs[t] = {"frames": fr, "box": bx}
    cases = {}
    for suite in ("cudatest", "cudatestPair", "cudatestWB"):
        for name in sorted(os.listdir(os.path.join(dcc, suite))):
            dd = os.path.join(dcc, suite, name)
            if not name.startswith("rt-"):
                continue
            traj = re.search(r"--ixyz\s+([^\s\"']+)", open(os.path.join(dd, "config")).read()).group(1)
            if traj not in trajs:
                continue
            lines = [l.split("#", 1)[0].rstrip() for l in open(os.path.join(dd, "plumed.dat"))]
            k = next(i for i, l in enumerate(lines) if re.match(r"\s*cpu:\s*COORDINATION\b", l))
            text = lines[k]
            if text.endswith("..."):  # continued until a line holding only "..."
                text = text[:-3]
                k += 1
                while lines[k].strip() != "...":
                    text += " " + lines[k]
                    k += 1
            line = " ".join(text.split(":", 1)[1].split()[1:])
            line = line.replace("@mdatoms", "1-%d" % len(trajs[traj]["frames"][0]))
            cases["%s/%s" % (suite, name)] = {
                "line": line, "traj": traj, "float": name.startswith("rt-float"),
                "diff": [r[1] for r in read_table(os.path.join(dd, "colvar.reference"))],
                "deriv_delta_max": max(abs(r[2]) for r in read_table(os.path.join(dd, "deriv_delta.reference")))}
    json.dump({"source": "plugins/cudaCoord/regtest (plumed.dat cpu: lines, colvar.reference, "
                         "deriv_delta.reference, trajectories/)",
               "trajectories": trajs, "cases": cases, "fmt": "diff %8.4f; derivative deltas %8.5f"},
              open(os.path.join(HERE, "cudacoord_plugin.json"), "w"))

    # --- rt-make-CellLists ---------------------------------------------------
    dcl = os.path.join(reg, "tools", "rt-make-CellLists")
    case_re = re.compile(r'^\[(?:"(?P<title>[^"]+)" )?co=(?P<co>[0-9.]+) -(?P<name>.+?)- \{(?P<cell>[0-9, ]+)\}'
                         r'(?P<nopbc> noPBC)?\] Cells:(?P<cells>[0-9 ]*)$')
    counts, req = [], []
    cube10 = [10.0, 0, 0, 0, 10.0, 0, 0, 0, 10.0]  # main.cpp testRequiredCells
    for fn in ("outputRequiredCells.reference", "outputRequiredCellsNotOrtho.reference"):
        boxes_by_title, pending = {}, None
        for line in open(os.path.join(dcl, fn)).read().split("\n"):
            m = re.match(r"NUMBER of cells: (\d+) \((\d+) (\d+) (\d+)\)", line)
            if m:
                pending = [int(m.group(k)) for k in (2, 3, 4)]
                continue
            m = re.match(r"^([^\[#][^:]*): ([-0-9. ]+)$", line)
            if m and len(m.group(2).split()) == 9:
                boxes_by_title[m.group(1)] = [float(x) for x in m.group(2).split()]
                continue
            m = case_re.match(line)
            if not m:
                continue
            box = boxes_by_title[m.group("title")] if m.group("title") else cube10
            co = float(m.group("co"))
            if pending is not None:
                counts.append({"box": box, "cutoff": co, "ncells": pending})
                pending = None
            req.append({"box": box, "cutoff": co, "cell": [int(x) for x in m.group("cell").split(",")],
                        "pbc": m.group("nopbc") is None, "cells": [int(x) for x in m.group("cells").split()]})
    idx_boxes = [[10.0, 0, 0, 0, 10.0, 0, 0, 0, 10.0], [10.0, 10.0, 0, 0, 10.0, 0, 0, 0, 10.0],
                 [10.0, 5.0, 3.0, 5.0, 10.0, 2.0, 3.0, 2.0, 10.0]]  # main.cpp testIndexes, cutoff 1.5
    nc_idx = [int(l.split(":")[1]) for l in open(os.path.join(dcl, "outputIndexes.reference")) if l.startswith("Ncells")]
    json.dump({"source": "regtest/tools/rt-make-CellLists (outputRequiredCells.reference, "
                         "outputRequiredCellsNotOrtho.reference, outputIndexes.reference; boxes of main.cpp)",
               "counts": counts, "required": req,
               "index_boxes": [{"box": b, "cutoff": 1.5, "ncells_total": n} for b, n in zip(idx_boxes, nc_idx)]},
              open(os.path.join(HERE, "rt_celllists.json"), "w"))

    # --- rt-Neigbourlist ---------------------------------------------------
    dnl = os.path.join(reg, "tools", "rt-Neigbourlist")
    sets = {}
    for fn in ("unitTest.reference", "testNoNL.reference"):
        for line in open(os.path.join(dnl, fn)):
            m = re.match(r"\[(.*), pbc (on|off)\] atom (\d+):(.*)", line)
            if not m:
                continue
            key = "%s|%s" % (m.group(1), m.group(2))
            sets.setdefault(key, {})[m.group(3)] = [int(x) for x in m.group(4).split()]
    json.dump({"source": "regtest/tools/rt-Neigbourlist/{unitTest,testNoNL}.reference",
               "lattice": "sc (AtomDistribution.cpp:205-240): integer sites i,j,k, x fastest; box = ceil(cbrt(N))",
               "cutoff_factor": 1.999, "sets": sets},
              open(os.path.join(HERE, "rt_neighbourlist.json"), "w"))
    # --- rt-dhenergy / rt-dhenergy2 -----------------------------------------
    ddh = os.path.join(reg, "basic", "rt-dhenergy")
    frames, boxes = read_xyz(os.path.join(reg, "trajectories", "trajectory.xyz"))
    charges = []
    for line in open(os.path.join(ddh, "test.pdb")):
        if line.startswith("ATOM"):
            charges.append(float(line.split()[-1]))
    colvar = read_table(os.path.join(ddh, "COLVAR.reference"))
    deriv = read_table(os.path.join(ddh, "deriv.reference"))
    nat = len(charges)
    npar = 3 * nat + 9
    der = [[r[2:] for r in deriv[f * npar:(f + 1) * npar]] for f in range(len(colvar))]
    colvar2 = read_table(os.path.join(reg, "basic", "rt-dhenergy2", "COLVAR.reference"))
    json.dump({"source": "regtest/basic/rt-dhenergy (plumed.dat, test.pdb, COLVAR.reference, deriv.reference), "
                         "regtest/basic/rt-dhenergy2/COLVAR.reference, regtest/trajectories/trajectory.xyz",
               "group_a": [1, 2, 3], "group_b": list(range(4, nat + 1)),
               "actions": {"dh1": {"I": 0.1, "TEMP": 300.0, "EPSILON": 80.0},
                           "dh2": {"I": 0.1, "TEMP": 300.0, "EPSILON": 80.0},
                           "dh3": {"I": 0.0, "TEMP": 300.0, "EPSILON": 80.0},
                           "dh4": {"I": 0.1, "TEMP": 10.0, "EPSILON": 200.0}},
               "order": ["dh1", "dh2", "dh3", "dh4"], "charges": charges,
               "frames": [fr[:nat] for fr in frames], "box": boxes,
               "colvar": [r[1:] for r in colvar], "deriv": der,
               "colvar_units_charge_0.1": [r[1:] for r in colvar2], "fmt": "%6.5f"},
              open(os.path.join(HERE, "rt_dhenergy.json"), "w"))

    # --- rt-ghbfix -----------------------------------------------------------
    dgh = os.path.join(reg, "basic", "rt-ghbfix")
    colvar = read_table(os.path.join(dgh, "colvar.reference"))
    deriv = read_table(os.path.join(dgh, "der.reference"))
    der = [[r[3] for r in deriv[f * 15:(f + 1) * 15]] for f in range(len(colvar))]
    json.dump({"source": "regtest/basic/rt-ghbfix (plumed.dat, config, typesTable.dat, scalingParameters.dat, "
                         "colvar.reference, der.reference)",
               "line": "PAIR GROUPA=1 GROUPB=2 D_0=0.2 D_MAX=0.3 C=0.8 ENERGY_UNITS=kcal/mol",
               "types_file": open(os.path.join(dgh, "typesTable.dat")).read(),
               "params_file": open(os.path.join(dgh, "scalingParameters.dat")).read(),
               "trajectory": "frame i = 1..150: atom 1 at (0,0,0), atom 2 at (0,0,0.002 i), box 100 100 100",
               "c1_minus_ghbfix": 4.184, "colvar_c1": [r[2] for r in colvar], "deriv_ghbfix": der,
               "fmt": "%8.4f"},
              open(os.path.join(HERE, "rt_ghbfix.json"), "w"))
    # --- COORDINATIONNUMBER: rt-dumpmulti, rt-single-groupb ---------------------
    f64, b64 = read_xyz(os.path.join(reg, "trajectories", "64.xyz"))
    cref = [float(l.split()[4]) for l in open(os.path.join(reg, "symfunc", "rt-dumpmulti",
                                                           "coordination.xyz.reference")).read().split("\n")[2:]
            if l.strip()]
    ftr, btr = read_xyz(os.path.join(reg, "trajectories", "trajectory.xyz"))
    sg = read_table(os.path.join(reg, "symfunc", "rt-single-groupb", "colvar.reference"))
    json.dump({"source": "regtest/symfunc/rt-dumpmulti (plumed.dat, coordination.xyz.reference), "
                         "regtest/trajectories/64.xyz, regtest/symfunc/rt-single-groupb (plumed.dat, "
                         "colvar.reference), regtest/trajectories/trajectory.xyz",
               "dumpmulti": {"spec": "RATIONAL D_0=3.0 R_0=1.5", "species": "1-64", "pos": f64[0], "box": b64[0],
                             "cn": cref, "fmt": "%.4f"},
               "single_groupb": {"spec": "RATIONAL R_0=1.0", "speciesa": "1-5", "speciesb": "6",
                                 "frames": [fr[:6] for fr in ftr], "box": btr, "cn": [r[1:] for r in sg],
                                 "fmt": "%8.4f"}},
              open(os.path.join(HERE, "rt_peratom.json"), "w"))
    # --- CONTACTMAP: rt28, rt72 ------------------------------------------------
    d28 = os.path.join(reg, "basic", "rt28")
    fr28, bx28 = read_xyz(os.path.join(d28, "trajectory.xyz"))
    col28 = read_table(os.path.join(d28, "colvar.reference"))
    der28 = read_table(os.path.join(d28, "deriv.reference"))
    maps28 = contactmap_blocks(os.path.join(d28, "plumed.dat"))
    atoms28 = sorted({a for cm in maps28 for c in cm["contacts"] for a in c["atoms"]})
    npar = 3 * 2 * len(maps28[0]["contacts"]) + 9
    d72 = os.path.join(reg, "basic", "rt72")
    pos72, box72 = read_gro(os.path.join(d72, "trpcage.gro"))
    col72 = read_table(os.path.join(d72, "colvar.reference"))
    der72 = read_table(os.path.join(d72, "deriv.reference"))
    maps72 = contactmap_blocks(os.path.join(d72, "plumed.dat"))
    json.dump({"source": "regtest/basic/rt28 (plumed.dat, trajectory.xyz, colvar.reference, deriv.reference), "
                         "regtest/basic/rt72 (plumed.dat, trpcage.gro, colvar.reference, deriv.reference)",
               "rt28": {"maps": maps28, "atoms": atoms28,
                        "frames": [[fr[a - 1] for a in atoms28] for fr in fr28], "box": bx28,
                        "colvar": [r[1:] for r in col28], "colvar_fields": ["a", "c.contact-1", "c.contact-5"],
                        "deriv_a": [[r[2] for r in der28[f * npar:(f + 1) * npar]] for f in range(len(col28))],
                        "fmt": "colvar %f, deriv %8.6f"},
               "rt72": {"map": maps72[0], "pos": pos72, "box": box72, "value": col72[0][1],
                        "deriv": [r[2] for r in der72], "fmt": "colvar %f, deriv %12.8f"}},
              open(os.path.join(HERE, "rt_contactmap.json"), "w"))
    # --- rt-metad-numder: METAD on one distance, the reference's forces -------
    dmn = os.path.join(reg, "basic", "rt-metad-numder")
    trm, bxm = read_xyz(os.path.join(reg, "trajectories", "trajectory.xyz"))
    natm = len(trm[0])
    rows = read_table(os.path.join(dmn, "forces.reference"))
    per = 3 * natm + 9
    nfr = len(rows) // per
    forces = [[r[1] for r in rows[k * per:(k + 1) * per]] for k in range(nfr)]
    json.dump({"source": "regtest/basic/rt-metad-numder (plumed.dat: d1: DISTANCE ATOMS=1,10; METAD ARG=d1 "
                         "SIGMA=0.1 HEIGHT=1.0 PACE=10; config: --trajectory-stride 10, --debug-forces, %8.4f), "
                         "regtest/trajectories/trajectory.xyz",
               "atoms": [1, 10], "sigma": 0.1, "height": 1.0, "pace": 10, "trajectory_stride": 10,
               "frames": [[fr[0], fr[9]] for fr in trm[:nfr]], "box": bxm[:nfr],
               "forces_atom1": [f[0:3] for f in forces], "forces_atom10": [f[27:30] for f in forces],
               "virial": [f[3 * natm:3 * natm + 9] for f in forces],
               "max_abs_other_forces": max(abs(x) for f in forces for i, x in enumerate(f[:3 * natm])
                                           if not (i < 3 or 27 <= i < 30)),
               "fmt": "%8.4f (analytical column of --debug-forces)"},
              open(os.path.join(HERE, "rt_metad_numder.json"), "w"), indent=0)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle import REFERENCE_TREE
    main(sys.argv[1] if len(sys.argv) > 1 else REFERENCE_TREE)
