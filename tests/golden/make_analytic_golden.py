"""Regenerates analytic_ref.json: values of the reference's own AnalyticKernel and
Scanner::pixel_sensitivity (src/2d/strip/analytic_kernel.h:28-62,
src/2d/strip/scanner.h:174-185), compiled from the reference headers by
oracle/build_ref.sh into oracle/_ref/ref_analytic (float and double, no FP
contraction).  These pin the GPU-reference mode's kernel and sensitivity: the
reference's own known answers for the analytic kernel are disabled
(kernel_test.cpp:66-79) and its GPU code does not compile with CUDA >= 12.

Contents (5 mm geometry of the CPU-runnable case):
  kernel   seeded (y, tan, sec, dz, dy) cases and the reference's values at
           float and double
  pixels   seeded pixels and their 5-point sensitivities at float and double
  events   four responses and, for each, the one-event GPU-reference image from
           a uniform rho: K_p / sum_q K_q s5_q over the box pixels that pass the
           3-sigma test, with K and s5 from the reference harness (sparse)

usage: python tests/golden/make_analytic_golden.py
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402  (box and response helpers of the restatement)

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_analytic")
GEOM = dict(R=450.0, L=1000.0, n_y=180, n_z=200, ph=5.0, pw=5.0, sz=10.0, sdl=42.0)
f32 = np.float32


def run_harness(kernel_cases, pixels):
    g = GEOM
    with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
        f.write(f"{g['R']} {g['L']} {g['n_y']} {g['n_z']} {g['ph']} {g['pw']} {g['sz']} {g['sdl']}\n")
        f.write(f"{len(kernel_cases)}\n")
        for c in kernel_cases:
            f.write(" ".join(repr(float(v)) for v in c) + "\n")
        f.write(f"{len(pixels)}\n")
        for px, py in pixels:
            f.write(f"{px} {py}\n")
        path = f.name
    out = subprocess.run([HARNESS, path], check=True, capture_output=True, text=True).stdout
    os.unlink(path)
    rows = [tuple(float(x) for x in line.split()) for line in out.splitlines()]
    return rows[:len(kernel_cases)], rows[len(kernel_cases):]


def event_pixels(ev):
    """Box pixels passing the 3-sigma test and their (dz, dy), in float as the
    restatement of the reference GPU kernel computes them."""
    g = GEOM
    L = oracle.lib()
    t, y, z = C.c_float(), C.c_float(), C.c_float()
    L.orc_response_tan_y_z_f(f32(g["R"]), f32(ev[0]), f32(ev[1]), f32(ev[2]), C.byref(t),
                             C.byref(y), C.byref(z))
    sec, A, B, Cc, by, bz = (C.c_float() for _ in range(6))
    L.orc_ellipse_bb_f(f32(g["sz"]), f32(g["sdl"]), t, C.byref(sec), C.byref(A), C.byref(B),
                       C.byref(Cc), C.byref(by), C.byref(bz))
    og = oracle.Geometry(g["R"], g["L"], g["n_y"], g["n_z"], g["pw"], g["sz"], g["sdl"]).c()
    b = [C.c_int32() for _ in range(4)]
    L.orc_event_box_f(C.byref(og), f32(ev[0]), f32(ev[1]), f32(ev[2]), *[C.byref(v) for v in b])
    tlx, tly, brx, bry = (v.value for v in b)
    size_y, size_z = f32(g["n_y"] * f32(g["ph"])), f32(g["n_z"] * f32(g["pw"]))
    tl_y_half_h = f32(f32(size_y / f32(2)) - f32(g["ph"]) / f32(2))
    tl_z_half_w = f32(f32(-size_z / f32(2)) + f32(g["pw"]) / f32(2))
    out = []
    for iy in range(tly, bry):
        for iz in range(tlx, brx):
            px = f32(tl_z_half_w + f32(iz) * f32(g["pw"]))
            py = f32(tl_y_half_h - f32(iy) * f32(g["ph"]))
            dy, dz = f32(py - f32(y.value)), f32(px - f32(z.value))
            q = f32(f32(f32(A.value * dy) * dy) + f32(f32(B.value * dy) * dz)) + f32(
                f32(Cc.value * dz) * dz)
            if q <= 9:
                out.append((iy, iz, float(dz), float(dy)))
    return (float(y.value), float(t.value), float(sec.value)), out


def main():
    rng = np.random.default_rng(2024)
    cases = []
    for _ in range(300):
        t = f32(rng.uniform(-1.1, 1.1))
        sec = f32(np.sqrt(f32(1) + t * t))
        cases.append((f32(rng.uniform(-400, 400)), t, sec, f32(rng.uniform(-40, 40)),
                      f32(rng.uniform(-60, 60))))
    pixels = [(int(rng.integers(0, GEOM["n_z"])), int(rng.integers(0, GEOM["n_y"])))
              for _ in range(300)]
    kv, sv = run_harness(cases, pixels)
    events = np.load(os.path.join(HERE, "c1_events.npy"))[[3, 50, 700, 4321]]
    ev_out = []
    for ev in events:
        (y, t, sec), pix = event_pixels(ev)
        k, s5 = run_harness([(y, t, sec, dz, dy) for (_, _, dz, dy) in pix],
                            [(iz, iy) for (iy, iz, _, _) in pix])
        kf = np.array([a for a, _ in k], np.float64)
        sf = np.array([a for a, _ in s5], np.float64)
        den = float(np.sum(kf * sf))
        ev_out.append({"response": [float(v) for v in ev],
                       "pixels": [[iy, iz, float(kv_ / den)]
                                  for (iy, iz, _, _), kv_ in zip(pix, kf)]})
    data = {"geometry": GEOM,
            "harness": "oracle/ref_analytic_harness.cpp (reference AnalyticKernel<F>, "
                       "Scanner<F, short>::pixel_sensitivity; no FP contraction)",
            "kernel": {"cases": [[float(v) for v in c] for c in cases],
                       "float": [a for a, _ in kv], "double": [b for _, b in kv]},
            "pixels": {"cases": pixels, "float": [a for a, _ in sv], "double": [b for _, b in sv]},
            "events": ev_out}
    with open(os.path.join(HERE, "analytic_ref.json"), "w") as f:
        json.dump(data, f)
    print("wrote analytic_ref.json:", len(cases), "kernel cases,", len(pixels), "pixels,",
          sum(len(e["pixels"]) for e in ev_out), "event pixels")


if __name__ == "__main__":
    main()
