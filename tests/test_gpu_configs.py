"""Parity at the stated workload configurations (through the C ABI).

  config 1  200 x 180 at 5 mm, sigma 10 / 42, 1e6 events of the 3-ellipse
            phantom, 10 iterations from a uniform image;
  config 2  500 x 450 at 2 mm, 2e7 events of the 10-ellipse phantom, 20
            iterations: a 2e6-event prefix iterated against the reference float
            path, and every event for one iteration against the reference
            iteration at double on the GPU.

Tolerances: each iteration started from the reference float path's previous
image within 1e-5 relative L2 of the reference's next one (single step); the
free-running iterations within 1e-4 of the reference's own free-running ones
(MLEM amplifies float summation-order differences from one iteration to the
next, as it does between two runs of the reference).
"""
import os

import numpy as np
import pytest

import oracle as O
from jpet_strip import capi
from jpet_strip.workloads import WORKLOADS

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-5
TOL_FREE = 1e-4


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _chain(og, ev, n):
    out, rho = [], None
    for _ in range(n):
        rho, st = O.mlem_f(og, ev, 1, rho, threads=os.cpu_count() or 1)
        out.append((rho, st))
    return out


def _against_reference(wl, n_events, n_iter):
    ev = wl.events(n_events, device=0)
    cg, og = capi.Geometry(*wl.geometry_args()), O.Geometry(*wl.geometry_args())
    ref = _chain(og, ev, n_iter)
    single, free = [], []
    with capi.StripReconstruction(cg) as step, capi.StripReconstruction(cg) as run:
        step.set_events(ev)
        run.set_events(ev)
        for it in range(n_iter):
            if it > 0:
                step.rho = ref[it - 1][0]
            step.iterate(1)
            single.append(rel_l2(step.rho, ref[it][0]))
            assert step.counters()["n_kernel_calls"] == ref[it][1]["n_kernel_calls"]
            assert step.counters()["n_contributing"] == ref[it][1]["n_contributing"]
            run.iterate(1)
            free.append(rel_l2(run.rho, ref[it][0]))
    return single, free


def test_config1_ten_iterations():
    wl = WORKLOADS["plain-5mm-1M"]
    single, free = _against_reference(wl, wl.n_events, wl.iterations)
    assert max(single) < TOL_STEP, single
    assert max(free) < TOL_FREE, free


def test_config2_prefix_twenty_iterations():
    wl = WORKLOADS["plain-2mm-20M"]
    single, free = _against_reference(wl, 2_000_000, wl.iterations)
    assert max(single) < TOL_STEP, single
    assert max(free) < TOL_FREE, free


def test_config2_full_size_against_fp64():
    torch = pytest.importorskip("torch")
    wl = WORKLOADS["plain-2mm-20M"]
    ev = wl.events(wl.n_events, device=0)
    cg = capi.Geometry(*wl.geometry_args())
    ev_d = torch.from_numpy(np.ascontiguousarray(ev)).cuda()
    f64, _ = capi.reference_fp64(cg, ev_d, 1)
    del ev_d
    with capi.StripReconstruction(cg) as r:
        r.set_events(ev)
        r.iterate(1)
        got = r.rho
    assert rel_l2(got, f64) < TOL_STEP
