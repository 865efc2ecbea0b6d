"""Generate tests/golden/ref_tool_pin.npz from the reference's own rigid-tool
geometry.

Builds oracle/_ref/ref_tool_pin (oracle/Makefile target ``ref``: the
reference's tool.cpp and geometric_primitives.cpp compiled for the host from
the read-only reference tree) and records, for the tool of setup_ref_cut
(benchmarks.cpp:384-412) over rake / clearance angles, edge radii, feeds,
particle spacings and extra travel:
  * the outline: per segment left, right, normal, line (a, b, vertical)
  * the fillet (centre, radius, start / end angle) or none
  * low(), front(), safe_bb(0.1 dx)
  * the tool particles of sample_tool(dx)
Run here (where the reference tree exists); the fixture travels, the
reference does not.  Usage: python tests/golden/make_tool_golden.py
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = Path(__file__).resolve().parent / "ref_tool_pin.npz"
REF_BIN = ROOT / "oracle" / "_ref" / "ref_tool_pin"

TL = (-0.05 + 0.004, 0.0986074)
LENGTH = -0.0086824 - -0.05
HEIGHT = 0.0986074 - 0.0555074
VEL = 83.333328 * 1e-5

# rake, clearance (degrees), edge radius (cm), feed (cm), dx (cm), extra travel (particle spacings)
CASES = [
    (0.0, 7.0, 5e-4, 0.002, 2.0 * 0.002 * 3 / 29, 0.0),
    (0.0, 7.0, 0.0, 0.002, 0.006 / 9, 1.5),
    (6.0, 7.0, 5e-4, 0.002, 0.006 / 9, 0.0),
    (-6.0, 5.0, 2e-3, 0.003, 0.009 / 14, 2.5),
    (10.0, 3.0, 1e-3, 0.001, 0.003 / 7, 0.0),
    (15.0, 10.0, 0.0, 0.004, 0.012 / 19, 0.7),
    (-10.0, 11.0, 3e-4, 0.0025, 0.0075 / 11, 3.0),
]


def parse(text: str):
    out, cur, lines, i = [], None, text.strip().splitlines(), 0
    while i < len(lines):
        tok = lines[i].split()
        if tok[0] == "seg":
            cur = cur or dict(segs=[])
            cur["segs"].append([float(v) for v in tok[2:]])
        elif tok[0] == "fillet":
            cur["fillet"] = np.full(5, np.nan) if tok[1] == "none" else np.array([float(v) for v in tok[1:]])
        elif tok[0] in ("low", "front"):
            cur[tok[0]] = float(tok[1])
        elif tok[0] == "bb":
            cur["bb"] = np.array([float(v) for v in tok[1:]])
        elif tok[0] == "samples":
            n = int(tok[1])
            cur["samples"] = np.array([[float(v) for v in lines[i + 1 + k].split()] for k in range(n)]).reshape(n, 2)
            i += n
        elif tok[0] == "end":
            out.append(cur)
            cur = None
        i += 1
    return out


def main():
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref"], check=True)
    rows = []
    for rake, clear, r, feed, dx, travel in CASES:
        rows.append([TL[0], TL[1], LENGTH, HEIGHT, rake, clear, r, 0.35, VEL, 0.005, 0.060, feed, dx,
                     travel * dx / VEL])
    rows = np.array(rows)
    txt = "\n".join(" ".join(f"{v:.17g}" for v in r) for r in rows) + "\n"
    res = subprocess.run([str(REF_BIN)], input=txt, capture_output=True, text=True, check=True)
    tools = parse(res.stdout)
    assert len(tools) == len(rows)
    arrays = dict(inputs=rows)
    for k, t in enumerate(tools):
        arrays[f"segs_{k}"] = np.array(t["segs"])
        arrays[f"fillet_{k}"] = t["fillet"]
        arrays[f"scalars_{k}"] = np.array([t["low"], t["front"]])
        arrays[f"bb_{k}"] = t["bb"]
        arrays[f"samples_{k}"] = t["samples"]
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT}: {len(tools)} tools, {sum(len(t['samples']) for t in tools)} tool particles")


if __name__ == "__main__":
    sys.exit(main())
