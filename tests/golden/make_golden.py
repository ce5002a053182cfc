"""Extract the golden fixtures of the p121 path from a ParaFEM source tree.

Usage: python tests/golden/make_golden.py /path/to/parafem

Reads the reference's own recorded runs (examples/5th_ed/p121, p123) and writes
  p121_golden.json      .res figures of the demo and book runs, the .mg
                        inputs, and sha256 of the demo deck files
  p121_demo_displ.npz   the demo displacement field (p121_demo.ensi.DISPL-000001)
  p123_golden.json      .res figures of the p123 book run and its .mg input
  p122_golden.json      per-increment .res figures of the p122 book and demo runs, the
                        book's .mg input and the demo's .dat record
  p122_demo.npz         the p122 demo deck (8-node bricks: connectivity, material
                        ids, coordinates, restraints, fixed freedoms) and its
                        ten recorded displacement fields (ensi.DISPL-0000nn)
The fixtures let the tests run where the reference tree is absent.
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_res(path):
    txt = open(path).read()
    out = {}
    m = re.search(r"There are\s+(\d+) nodes\s+(\d+) restrained and\s+(\d+) equations", txt)
    out["nn"], out["nr"], out["neq"] = (int(g) for g in m.groups())
    m = re.search(r"This job ran on\s+(\d+) processes", txt)
    out["processes"] = int(m.group(1))
    m = re.search(r"The total load is:\s*(\S+)", txt)
    if m:
        out["total_load_text"] = m.group(1)
    m = re.search(r"The number of iterations to convergence was\s+(\d+)", txt)
    out["iterations"] = int(m.group(1))
    m = re.search(r"The central nodal displacement is :\s*(\S+)", txt)
    out["central_text"] = m.group(1)
    lines = txt.splitlines()
    i = next(k for k, ln in enumerate(lines) if ln.startswith("Point"))
    out["stress_text"] = lines[i + 1].split()
    out["lines"] = {
        "iterations": next(ln for ln in lines if ln.startswith("The number of iterations")),
        "central": next(ln for ln in lines if ln.startswith("The central nodal")),
        "stress": lines[i + 1],
    }
    tl = [ln for ln in lines if ln.startswith("The total load")]
    if tl:
        out["lines"]["total_load"] = tl[0]
    return out


def main(root):
    ex = os.path.join(root, "examples", "5th_ed", "p121")
    demo = os.path.join(ex, "demo", "p121_demo")
    gold = {
        "source": "examples/5th_ed/p121 of the ParaFEM tree",
        "demo": parse_res(demo + ".res"),
        "book": parse_res(os.path.join(ex, "book", "p121.res")),
        "demo_mg": open(demo + ".mg").read(),
        "book_mg": open(os.path.join(ex, "book", "p121.mg")).read(),
        "demo_deck_sha256": {},
    }
    for ext in ("dat", "d", "bnd", "lds"):
        with open(demo + "." + ext, "rb") as f:
            gold["demo_deck_sha256"][ext] = hashlib.sha256(f.read()).hexdigest()
    with open(os.path.join(HERE, "p121_golden.json"), "w") as f:
        json.dump(gold, f, indent=1, sort_keys=True)
    # displacement field: 4 header lines, then x block, y block, z block (e12.4 text)
    vals = []
    with open(demo + ".ensi.DISPL-000001") as f:
        lines = f.read().splitlines()[4:]
    vals = np.array([float(t) for t in lines if t.strip()], dtype=np.float64)
    nn = gold["demo"]["nn"]
    disp = vals.reshape(3, nn).T.astype(np.float32)
    np.savez_compressed(os.path.join(HERE, "p121_demo_displ.npz"), disp=disp)
    print("wrote", os.path.join(HERE, "p121_golden.json"), disp.shape)


def parse_res123(path):
    txt = open(path).read()
    lines = txt.splitlines()
    out = {}
    m = re.search(r"There are\s+(\d+) nodes\s+(\d+) restrained and\s+(\d+) equations", txt)
    out["nn"], out["nr"], out["neq"] = (int(g) for g in m.groups())
    out["processes"] = int(re.search(r"This job ran on\s+(\d+)\s+processes", txt).group(1))
    out["iterations"] = int(re.search(r"The number of iterations to convergence was\s+(\d+)", txt).group(1))
    out["total_load_text"] = re.search(r"The total load is\s+(\S+)", txt).group(1)
    i = next(k for k, ln in enumerate(lines) if ln.strip().startswith("Freedom"))
    out["potentials"] = [[int(ln.split()[0]), ln.split()[1]] for ln in lines[i + 1:i + 5]]
    out["lines"] = {"potentials": lines[i + 1:i + 5],
                    "total_load": next(ln for ln in lines if ln.startswith("The total load"))}
    return out


def main123(root):
    ex = os.path.join(root, "examples", "5th_ed", "p123", "book")
    gold = {"source": "examples/5th_ed/p123/book of the ParaFEM tree",
            "book": parse_res123(os.path.join(ex, "p123.res")),
            "book_mg": open(os.path.join(ex, "p123.mg")).read()}
    with open(os.path.join(HERE, "p123_golden.json"), "w") as f:
        json.dump(gold, f, indent=1, sort_keys=True)
    print("wrote", os.path.join(HERE, "p123_golden.json"))


def parse_res122(path):
    txt = open(path).read()
    lines = txt.splitlines()
    out = {}
    m = re.search(r"There are\s+(\d+) nodes\s+(\d+) restrained and\s+(\d+) equations", txt)
    out["nn"], out["nr"], out["neq"] = (int(g) for g in m.groups())
    out["processes"] = int(re.search(r"This job ran on\s+(\d+)\s+processes", txt).group(1))
    out["dt_text"] = re.search(r"The critical timestep is\s+(\S+)", txt).group(1)
    incs = []
    for k, ln in enumerate(lines):
        if ln.startswith("Load Increment"):
            inc = {"increment": int(ln.split()[-1])}
            inc["displacement_text"] = lines[k + 1].split()[-1]
            inc["stress_text"] = lines[k + 3].split()
            inc["cj_iterations"] = int(lines[k + 4].split()[-1])
            inc["plastic_iterations"] = int(lines[k + 5].split()[-1])
            incs.append(inc)
    out["increments"] = incs
    return out


def read_displ(path, nn):
    """An ensi.DISPL file: 4 header lines, then the x, y and z blocks."""
    with open(path) as f:
        lines = f.read().splitlines()[4:]
    vals = np.array([float(t) for t in lines if t.strip()], dtype=np.float64)
    return vals.reshape(3, nn).T


def main122(root):
    ex = os.path.join(root, "examples", "5th_ed", "p122", "book")
    gold = {"source": "examples/5th_ed/p122/book and demo of the ParaFEM tree",
            "book": parse_res122(os.path.join(ex, "p122.res")),
            "book_mg": open(os.path.join(ex, "p122.mg")).read()}
    demo = os.path.join(root, "examples", "5th_ed", "p122", "demo", "p122_demo")
    gold["demo"] = parse_res122(demo + ".res")
    gold["demo_dat"] = open(demo + ".dat").read()
    gold["demo_deck_sha256"] = {}
    for ext in ("dat", "d", "bnd", "fix"):
        with open(demo + "." + ext, "rb") as f:
            gold["demo_deck_sha256"][ext] = hashlib.sha256(f.read()).hexdigest()
    with open(os.path.join(HERE, "p122_golden.json"), "w") as f:
        json.dump(gold, f, indent=1, sort_keys=True)
    # the demo deck: .d (nodes; elements "id 3 8 1 n1..n8 matid"), .bnd, .fix
    tok = gold["demo_dat"].replace("'", " ").split()
    nels, nn, nr, nod, nfix = int(tok[3]), int(tok[4]), int(tok[5]), int(tok[7]), int(tok[8])
    incs = int(tok[15])
    with open(demo + ".d") as f:
        lines = f.read().splitlines()
    i = lines.index("*NODES") + 1
    coords = np.array([[float(t) for t in ln.split()[1:4]] for ln in lines[i:i + nn]])
    j = lines.index("*ELEMENTS") + 1
    el = np.array([[int(t) for t in ln.split()] for ln in lines[j:j + nels]], dtype=np.int64)
    g_num, matid = el[:, 4:4 + nod].astype(np.int32), el[:, 4 + nod].astype(np.int32)
    rest = np.array([[int(t) for t in ln.split()] for ln in open(demo + ".bnd").read().splitlines()[:nr]],
                    dtype=np.int32)
    fx = [ln.split() for ln in open(demo + ".fix").read().splitlines()[:nfix]]
    fix_node = np.array([int(t[0]) for t in fx], dtype=np.int32)
    fix_sense = np.array([int(t[1]) for t in fx], dtype=np.int32)
    fix_val = np.array([float(t[2]) for t in fx])
    displ = np.stack([read_displ(demo + ".ensi.DISPL-%06d" % k, nn) for k in range(1, incs + 1)])
    np.savez_compressed(os.path.join(HERE, "p122_demo.npz"), g_num=g_num, matid=matid, coords=coords, rest=rest,
                        fix_node=fix_node, fix_sense=fix_sense, fix_val=fix_val, displ=displ)
    print("wrote", os.path.join(HERE, "p122_golden.json"), os.path.join(HERE, "p122_demo.npz"), displ.shape)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <root of the ParaFEM tree (the directory holding examples/)>")
    main(sys.argv[1])
    main123(sys.argv[1])
    main122(sys.argv[1])
