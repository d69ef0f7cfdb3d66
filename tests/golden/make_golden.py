"""Regenerates the golden fixtures in this folder from the reference's own CPU tools.

Needs the reference binaries built by ``oracle/build_ref.sh`` (only possible where
the reference sources are present).  The events come from the project's seeded
generator; the images come from the *reference* ``2d_strip_reconstruction``
(``src/2d/strip/reconstruction_cmd.cpp``) and from the reference
``Reconstruction`` template at double (``oracle/ref_fp64_harness.cpp``):

  <case>_events.npy            float32[n, 3] responses (z_u, z_d, dl)
  <case>_strict_itNN.npy       float32[n_y, n_z]  ref_rec_strict (no FMA contraction), 1 thread
  <case>_release_itNN.npy      float32[n_y, n_z]  ref_rec (reference release flags), 1 thread
  <case>_fp64_itNN.npy         float64[n_y, n_z]  ref_fp64, 1 thread
  manifest.json                geometry, commands and image sums

usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "j-pet-mlem_gb300", "python"))
from jpet_strip import phantom  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")

CASES = {
    # 5 mm plain workload geometry, 200 x 180 pixels
    "c1": dict(R=450.0, L=1000.0, p=5.0, n_z=200, n_y=180, sz=10.0, sdl=42.0,
               n=10000, seed=11, iters=3, keep=(1, 3)),
    # cropped 2 mm grid covering |z| <= 100, |y| <= 90 only: most boxes are clamped
    "crop": dict(R=450.0, L=1000.0, p=2.0, n_z=100, n_y=90, sz=10.0, sdl=42.0,
                 n=4000, seed=12, iters=2, keep=(1, 2)),
}


def run_ref(tool, ev_path, c, out_prefix):
    cmd = [os.path.join(REF, tool), ev_path, "-r", str(c["R"]), "-l", str(c["L"]),
           "-p", str(c["p"]), "--n-z-pixels", str(c["n_z"]), "--n-y-pixels", str(c["n_y"]),
           "--s-z", str(c["sz"]), "--s-dl", str(c["sdl"]), "-i", str(c["iters"]), "-I", "1",
           "-T", "1", "-o", out_prefix + ".bin"]
    subprocess.run(cmd, check=True)
    return cmd


def main():
    manifest = {}
    for name, c in CASES.items():
        ev = phantom.generate_events(phantom.three_ellipse_phantom(), c["n"], c["R"], c["L"],
                                     c["sz"], c["sdl"], seed=c["seed"])
        np.save(os.path.join(HERE, f"{name}_events.npy"), ev)
        entry = dict(geometry={k: c[k] for k in ("R", "L", "p", "n_z", "n_y", "sz", "sdl")},
                     n_events=int(len(ev)), seed=c["seed"], iterations=list(c["keep"]),
                     commands={}, sums={})
        with tempfile.TemporaryDirectory() as tmp:
            ev_path = os.path.join(tmp, "events.bin")
            ev.tofile(ev_path)
            for tool, tag in (("ref_rec_strict", "strict"), ("ref_rec", "release")):
                prefix = os.path.join(tmp, tag)
                entry["commands"][tag] = " ".join(
                    os.path.basename(a) if i == 0 else a
                    for i, a in enumerate(run_ref(tool, ev_path, c, prefix)))
                width = len(str(c["iters"]))
                for it in c["keep"]:
                    if tag == "release" and it != c["keep"][-1]:
                        continue
                    img = np.fromfile(f"{prefix}_{it:0{width}d}.bin", np.float32)
                    img = img.reshape(c["n_y"], c["n_z"])
                    np.save(os.path.join(HERE, f"{name}_{tag}_it{it:02d}.npy"), img)
                    entry["sums"][f"{tag}_it{it:02d}"] = float(img.astype(np.float64).sum())
            if name == "c1":
                prefix = os.path.join(tmp, "fp64")
                cmd = [os.path.join(REF, "ref_fp64"), ev_path, str(c["R"]), str(c["L"]),
                       str(c["n_y"]), str(c["n_z"]), str(c["p"]), str(c["sz"]), str(c["sdl"]),
                       str(c["iters"]), "1", prefix]
                subprocess.run(cmd, check=True)
                entry["commands"]["fp64"] = " ".join(["ref_fp64"] + cmd[1:-1] + ["<prefix>"])
                it = c["keep"][-1]
                img = np.fromfile(f"{prefix}_{it:03d}.f64", np.float64).reshape(c["n_y"], c["n_z"])
                np.save(os.path.join(HERE, f"{name}_fp64_it{it:02d}.npy"), img)
                entry["sums"][f"fp64_it{it:02d}"] = float(img.sum())
        for tag, cmd in entry["commands"].items():
            entry["commands"][tag] = cmd.replace(tmp + os.sep, "<tmp>/")
        manifest[name] = entry
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)



if __name__ == "__main__":
    main()
