"""Regenerates the event-generator fixtures in this folder from the reference's own
``2d_strip_phantom`` tool (``src/2d/strip/phantom_cmd.cpp``), built by
``oracle/build_ref.sh`` into ``oracle/_ref/ref_phantom``.

The reference tool seeds its generator from the default std::mt19937 state per
OpenMP thread, so its events are a sample of the reference's distribution, not
a reproducible stream; the tests compare distributions (two-sample KS) and the
detected fraction of emissions (binomial).

  phantom_three.txt            the phantom description passed to the tool
  phantom_ref_events.npy       float32[50000, 3], the first detected responses
  phantom_ref.json             command, emissions, detected count

usage: python tests/golden/make_phantom_golden.py
"""
from __future__ import annotations

import json
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref", "ref_phantom")

PHANTOM = """ellipse 120 -40 150 150 0 2.0
ellipse -100 50 180 150 30 0.5
ellipse 0 0 300 250 0 1.0
"""
EMISSIONS = 2000000
KEEP = 50000


def main() -> None:
    if not os.path.exists(REF):
        raise SystemExit("oracle/_ref/ref_phantom not built (run oracle/build_ref.sh)")
    with open(os.path.join(HERE, "phantom_three.txt"), "w") as f:
        f.write(PHANTOM)
    with tempfile.TemporaryDirectory() as tmp:
        txt = os.path.join(tmp, "three.txt")
        with open(txt, "w") as f:
            f.write(PHANTOM)
        out = os.path.join(tmp, "ph.bin")
        cmd = [REF, "-r", "450", "-l", "1000", "-p", "5", "--n-z-pixels", "200",
               "--n-y-pixels", "180", "--s-z", "10", "--s-dl", "42", "-e", str(EMISSIONS),
               "-o", out, txt]
        subprocess.run(cmd, check=True, cwd=tmp, stdout=subprocess.DEVNULL,
                       stderr=subprocess.DEVNULL)
        ev = np.fromfile(out, dtype=np.float32).reshape(-1, 3)
    np.save(os.path.join(HERE, "phantom_ref_events.npy"), ev[:KEEP])
    meta = dict(command=" ".join(["ref_phantom"] + cmd[1:-3] + ["-o", "<tmp>/ph.bin",
                                                                 "phantom_three.txt"]),
                emissions=EMISSIONS, detected=int(len(ev)), kept=KEEP,
                R=450.0, L=1000.0, sigma_z=10.0, sigma_dl=42.0)
    with open(os.path.join(HERE, "phantom_ref.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(meta)


if __name__ == "__main__":
    main()
