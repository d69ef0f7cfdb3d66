"""Regenerates the converter fixtures in this folder from the reference's own
``3d_tool_convert`` (``src/3d/tool/convert_cmd.cpp``), built by
``oracle/build_ref.sh`` into ``oracle/_ref/ref_convert``.

The inputs are synthetic, seeded: hits inside (and a few outside) the square
detectors of one or two rings, in the Warsaw column layout the tool reads
("x1 y1 z1 t1 x2 y2 z2 t2 <extra columns> scatter", cm and ps), and detector
time quadruples in the T. Bednarski layout ("du dd t_ul t_ur t_dl t_dr").  The
reference tool smears with std::mt19937_64 and std::normal_distribution, so its
output for a given --seed is reproducible and the fixtures are exact text.

  convert_warsaw_hits.txt      Warsaw-layout hits
  convert_bednarski_times.txt  Bednarski-layout times
  convert_ref.json             {case name: [arguments, reference stdout]}

usage: python tests/golden/make_convert_golden.py
"""
from __future__ import annotations

import json
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref", "ref_convert")
WARSAW = "convert_warsaw_hits.txt"
BEDNARSKI = "convert_bednarski_times.txt"

SCANNER = ["-r", "0.43", "-d", "48", "-w", "0.007", "-h", "0.019"]
CASES = {
    "warsaw": SCANNER + ["-l", "0.5", "--s-z", "0.01", "--s-dl", "0.04", "--seed", "5", WARSAW],
    "warsaw_default_seed": SCANNER + ["-l", "0.5", "--warsaw", WARSAW],
    "warsaw_only_scatter_1": SCANNER + ["-l", "0.5", "--only", "1", "--seed", "3", WARSAW],
    "warsaw_two_rings": ["-r", "0.43,0.5", "-d", "48,96", "--rotation", "0,0.5", "-w", "0.007",
                         "-h", "0.019", "-l", "0.5", "--seed", "9", WARSAW],
    "warsaw_auto_width": ["-r", "0.43", "-d", "48", "-h", "0.019", "-l", "0.5", "--seed", "2",
                          WARSAW],
    "bednarski": SCANNER + ["--tbednarski", BEDNARSKI],
    "bednarski_relative": SCANNER + ["--tbednarski", "--relative-time", BEDNARSKI],
}


def _hit(rng, ring_r, n, d, h=0.019, w=0.007, rot=0.0):
    """A point inside detector d of a ring (its centre at radius + h/2, rotated
    like scanner_builder.h:72-79), in cm."""
    ang = 2 * math.pi * d / n - math.pi / 2 + 2 * math.pi * rot / n
    cx, cy = -(ring_r + h / 2) * math.sin(ang), (ring_r + h / 2) * math.cos(ang)
    u, v = rng.uniform(-0.45 * w, 0.45 * w), rng.uniform(-0.45 * h, 0.45 * h)
    return (100 * (cx + u * math.cos(ang) - v * math.sin(ang)),
            100 * (cy + u * math.sin(ang) + v * math.cos(ang)))


def write_inputs() -> None:
    rng = np.random.default_rng(2024)
    lines = []
    for k in range(300):
        ring = k % 3 == 2  # every third event on the outer ring of the two-ring case
        r, n, rot = (0.5, 96, 0.5) if ring else (0.43, 48, 0.0)
        d1, d2 = rng.integers(0, n, 2)
        x1, y1 = _hit(rng, r, n, int(d1), rot=rot)
        x2, y2 = _hit(rng, r, n, int(d2), rot=rot)
        if k % 17 == 0:
            x1, y1 = 0.0, 0.0  # inside no detector
        z1, z2 = rng.uniform(-30.0, 30.0, 2)
        t1, t2 = rng.uniform(0.0, 3000.0, 2)
        extra = rng.uniform(0.0, 1.0, 3)
        scatter = int(rng.integers(1, 4))
        vals = [x1, y1, z1, t1, x2, y2, z2, t2, *extra]
        lines.append(" ".join(f"{v:.6f}" for v in vals) + f" {scatter}")
    with open(os.path.join(HERE, WARSAW), "w") as f:
        f.write("\n".join(lines) + "\n")
    lines = []
    for _ in range(100):
        du, dd = rng.integers(1, 49, 2)
        times = rng.uniform(1000.0, 2000.0, 4)
        lines.append(f"{du} {dd} " + " ".join(f"{v:.3f}" for v in times))
    with open(os.path.join(HERE, BEDNARSKI), "w") as f:
        f.write("\n".join(lines) + "\n")


def main() -> None:
    if not os.path.exists(REF):
        raise SystemExit("oracle/_ref/ref_convert not built (run oracle/build_ref.sh)")
    write_inputs()
    out = {}
    for name, args in CASES.items():
        r = subprocess.run([REF] + args, cwd=HERE, capture_output=True, text=True, check=True)
        out[name] = [args, r.stdout]
    with open(os.path.join(HERE, "convert_ref.json"), "w") as f:
        json.dump(out, f, indent=1)
    print({k: v[1].count("\n") for k, v in out.items()})


if __name__ == "__main__":
    main()
