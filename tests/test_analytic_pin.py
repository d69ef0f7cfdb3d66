"""Pins the GPU-reference semantics (analytic kernel + 5-point pixel sensitivity)
to values of the reference's own code: tests/golden/analytic_ref.json holds
AnalyticKernel<F> (src/2d/strip/analytic_kernel.h:28-62) and
Scanner<F, short>::pixel_sensitivity (src/2d/strip/scanner.h:174-185) compiled
from the reference headers (oracle/ref_analytic_harness.cpp, written by
tests/golden/make_analytic_golden.py).

CPU: the restatement in the oracle equals them bit for bit at float and within
1e-14 at double.  GPU: one-event iterations of JPET_MODE_GPU_REFERENCE from a
uniform image give K_p / sum_q K_q s5_q with those reference values, within
float rounding.  The reference GPU kernel's own loop (warp_granularity.cuh)
cannot be compiled with CUDA >= 12 and stays unpinned."""
import ctypes as C
import json
import os

import numpy as np
import pytest

import oracle as O
from jpet_strip import capi

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def ref():
    with open(os.path.join(HERE, "golden", "analytic_ref.json")) as f:
        return json.load(f)


def _ogeom(g):
    return O.Geometry(g["R"], g["L"], g["n_y"], g["n_z"], g["pw"], g["sz"], g["sdl"],
                      pixel_height=g["ph"])


def test_restated_analytic_kernel_equals_reference(ref):
    L = O.lib()
    g = ref["geometry"]
    for (y, t, sec, dz, dy), vf, vd in zip(ref["kernel"]["cases"], ref["kernel"]["float"],
                                           ref["kernel"]["double"]):
        got_f = L.orc_analytic_kernel_f(g["sz"], g["sdl"], y, t, sec, g["R"], dz, dy)
        assert np.float32(got_f) == np.float32(vf), (y, t, dz, dy, got_f, vf)
        got_d = L.orc_analytic_kernel_d(g["sz"], g["sdl"], y, t, sec, g["R"], dz, dy)
        assert got_d == pytest.approx(vd, rel=1e-14, abs=1e-300)


def test_restated_pixel_sensitivity_equals_reference(ref):
    L = O.lib()
    L.orc_pixel_sensitivity_f.restype = C.c_float
    L.orc_pixel_sensitivity_f.argtypes = [C.POINTER(O.OrcGeom), C.c_int32, C.c_int32]
    og = _ogeom(ref["geometry"]).c()
    for (px, py), sf in zip(ref["pixels"]["cases"], ref["pixels"]["float"]):
        got = L.orc_pixel_sensitivity_f(C.byref(og), px, py)
        assert np.float32(got) == np.float32(sf), (px, py, got, sf)


@pytest.mark.gpu
def test_gpu_reference_mode_one_event_images(ref):
    g = ref["geometry"]
    cg = capi.Geometry(g["R"], g["L"], g["n_y"], g["n_z"], g["pw"], g["sz"], g["sdl"])
    for ev in ref["events"]:
        want = np.zeros((g["n_y"], g["n_z"]), np.float64)
        for iy, iz, v in ev["pixels"]:
            want[iy, iz] = v
        with capi.StripReconstruction(cg, mode=capi.MODE_GPU_REFERENCE) as rec:
            rec.set_events(np.array([ev["response"]], np.float32))
            rec.iterate(1)
            got = rec.rho.astype(np.float64)
        assert np.count_nonzero(got) == len(ev["pixels"])
        rel = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert rel < 1e-5, rel
