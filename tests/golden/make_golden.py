"""Generate the golden fixtures under tests/golden/ (run where the reference sources are).

Inputs: the reference's own input fixtures TestCaseA.txt, TestCaseB.txt and
TestCaseC.txt (Apache-2.0, copied verbatim as test inputs) and its
SampleInputFile.txt (legacy keys the parser does not recognise).

Output fixtures: the reference's committed vars.csv and k_eff.csv (verbatim)
and interface.csv cut to its first 40 fields per row, under plot_output/.
They were written by an older revision with f64 values, so they pin the text
layout and the f64 float text of plot_solution (src/plot_solution.rs:36-58),
not numbers of the current solver.

Expected values: computed by the pure-Python restatement below of
  scan_ascii_chunk / get_index / process_input  (src/process_input.rs:6-175)
  mesh_gen                                       (src/main.rs:85-143)
which is independent of the C++ front end under test.  f32 arithmetic is
reproduced with numpy float32.

    python tests/golden/make_golden.py /path/to/reference
"""
from __future__ import annotations

import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
KEYS = {("lk", 5): 0, ("es", 8): 1, ("ps", 12): 2, ("ns", 11): 3, ("es", 9): 4, ("ip", 4): 5,
        ("ss", 6): 6, ("ds", 7): 7, ("ia", 6): 8, ("ch", 8): 9, ("fr", 4): 10, ("wr", 4): 11,
        ("dl", 6): 12, ("dr", 6): 13, ("gt", 4): 14, ("gs", 4): 15, ("mu", 2): 16, ("ga", 4): 17,
        ("gf", 4): 18, ("ut", 3): 19, ("it", 4): 20, ("at", 4): 21, ("id", 5): 22, ("on", 8): 23,
        ("er", 6): 24}


def scan(buf: bytes):
    temp = [""] * 26
    end = len(buf)
    pos = line_start = name_end = val_start = 0
    while pos < end:
        c = buf[pos]
        if c == ord("#"):
            while pos < end and buf[pos] != ord("\n"):
                pos += 1
            pos += 1
            line_start = pos
        elif c == ord("="):
            name_end = pos - 1
            val_start = pos + 1
        elif c == ord("\n"):
            if name_end > line_start:
                key = buf[line_start:name_end].decode().strip().lower()
                value = buf[val_start:pos].decode().strip()
                temp[KEYS.get((key[-2:], len(key)), 25)] += " " + value
            line_start = pos + 1
        pos += 1
    return temp


def f32(s):
    return np.float32(float(s))


def process_input(path):
    temp = scan(open(path, "rb").read())
    v = dict(analk=int(temp[0]), mattypes=int(temp[1]), energygroups=int(temp[2]),
             generations=int(temp[3]), histories=int(temp[4]), skip=int(temp[5]),
             numass=int(temp[6]), numrods=int(temp[7]), roddia=f32(temp[8]),
             rodpitch=np.float32(f32(temp[9]) - f32(temp[8])), mpfr=int(temp[10]), mpwr=int(temp[11]),
             boundl=f32(temp[12]), boundr=f32(temp[13]))
    lists = {k: np.array([f32(t) for t in temp[i].split()], np.float32)
             for k, i in (("sigt", 14), ("sigs", 15), ("mu", 16), ("siga", 17), ("sigf", 18),
                          ("nut", 19), ("chit", 20), ("scat", 21))}
    inv = (np.float32(1.0) / (lists["sigt"] - lists["mu"] * lists["sigs"])).astype(np.float32)
    matid = [int(t) for t in temp[22].split()]
    solution = int(temp[23]) != 1
    sv = temp[24].strip()
    solver = {"1": 1, "2": 2, "3": 3}.get(sv, 0)
    dx = dict(fuel=np.float32(v["roddia"] / np.float32(v["mpfr"])),
              water=np.float32(v["rodpitch"] / np.float32(v["mpwr"])))
    return v, lists, inv, matid, solution, solver, dx


def mesh_gen(matid, v, dx):
    temp = []
    for x in matid:
        temp += [x] * (v["mpfr"] if x in (0, 1) else v["mpwr"])
    for a in range(1, v["numass"]):
        for _ in range(v["mpwr"]):
            del temp[(a * len(temp)) // v["numass"]]
    h = v["mpwr"] // 2
    temp = temp[h:]
    temp = temp[: len(temp) - h]
    fuel = [i for i, r in enumerate(temp) if r in (0, 1)]
    left = np.float32(0.0)
    lefts, rights, dxs = [], [], []
    for r in temp:
        d = dx["fuel"] if r in (0, 1) else dx["water"]
        lefts.append(float(left))
        rights.append(float(np.float32(left + d)))
        dxs.append(float(d))
        left = np.float32(left + d)
    return temp, lefts, rights, dxs, fuel


def main(ref: str):
    os.makedirs(os.path.join(HERE, "inputs"), exist_ok=True)
    out = {}
    for name in ("TestCaseA.txt", "TestCaseB.txt", "TestCaseC.txt"):
        src = os.path.join(ref, name)
        dst = os.path.join(HERE, "inputs", name)
        shutil.copyfile(src, dst)
        v, lists, inv, matid, solution, solver, dx = process_input(src)
        mats, lefts, rights, dxs, fuel = mesh_gen(matid, v, dx)
        out[name] = dict(
            variables={k: (float(val) if isinstance(val, np.floating) else val) for k, val in v.items()},
            delta_x={k: float(val) for k, val in dx.items()},
            xs={k: [float(x) for x in a] for k, a in lists.items()},
            inv_sigtr=[float(x) for x in inv], matid=matid, solution=solution, solver=solver,
            mesh=dict(n_cells=len(mats), matid=mats, mesh_left=lefts, mesh_right=rights, delta_x=dxs,
                      fuel_indices=fuel))
    shutil.copyfile(os.path.join(ref, "SampleInputFile.txt"), os.path.join(HERE, "inputs", "SampleInputFile.txt"))
    po = os.path.join(HERE, "plot_output")
    os.makedirs(po, exist_ok=True)
    for name in ("vars.csv", "k_eff.csv"):
        shutil.copyfile(os.path.join(ref, name), os.path.join(po, name))
    with open(os.path.join(ref, "interface.csv"), "rb") as fh, \
            open(os.path.join(po, "interface_head.csv"), "wb") as out_fh:
        for line in fh:
            out_fh.write(b",".join(line.rstrip(b"\n").split(b",")[:40]) + b"\n")
    with open(os.path.join(HERE, "frontend_golden.json"), "w") as fh:
        json.dump(out, fh, indent=0)
    print("wrote", os.path.join(HERE, "frontend_golden.json"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_golden.py <path to the NRAPS source tree>")
    main(sys.argv[1])
