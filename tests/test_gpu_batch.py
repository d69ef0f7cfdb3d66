"""Batched reconstructions (jpet_strip_batch_*): one graph launch per iterate
gives every instance the image of its own single-handle iterations."""
import numpy as np
import pytest

import oracle as O
from jpet_strip import capi, phantom

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1e-5


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _instances(k, seed=100, max_events=60000):
    """k instances of uneven sizes: grids 100..500 x 100..450, pixels 2..5 mm,
    sigma_z in [6, 14], sigma_dl in [30, 60], 1..10 ellipses, log-uniform events."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(k):
        p = float(rng.integers(2, 6))
        n_z = int(rng.integers(100, 501))
        n_y = int(rng.integers(100, 451))
        sz = float(rng.uniform(6, 14))
        sdl = float(rng.uniform(30, 60))
        n = int(np.exp(rng.uniform(np.log(2000), np.log(max_events))))
        hz, hy = min(n_z * p / 2, 500.0), min(n_y * p / 2, 450.0)
        ell = phantom.random_ellipse_phantom(seed + i, n=int(rng.integers(1, 11)), half_z=hz,
                                             half_y=hy, centre_z=0.6 * hz, centre_y=0.6 * hy,
                                             axes=(10.0, 0.8 * min(hz, hy)))
        geom = capi.Geometry(450.0, 1000.0, n_y, n_z, p, sz, sdl)
        ev = capi.generate(ell, n, 450.0, 1000.0, sz, sdl, seed=seed + i)
        out.append((geom, ev))
    return out


def _single(geom, ev, n_iter, **opts):
    with capi.StripReconstruction(geom, **opts) as r:
        r.set_events(ev)
        r.iterate(n_iter)
        return r.rho, r.counters()


def test_batch_matches_single_handles_over_odd_and_even_iterations():
    inst = _instances(9)
    with capi.StripBatch([g for g, _ in inst]) as b:
        for i, (_, ev) in enumerate(inst):
            b.set_events(i, ev)
        b.iterate(1)  # odd: images swap inside every handle
        b.iterate(2)
        assert b.launches_per_iteration() >= 2
        for i, (g, ev) in enumerate(inst):
            want, cnt = _single(g, ev, 3)
            got = b.instance(i).rho
            assert rel_l2(got, want) < TOL, i
            c = b.instance(i).counters()
            assert c["n_kernel_calls"] == cnt["n_kernel_calls"], i
            assert c["n_contributing"] == cnt["n_contributing"], i
            assert c["iterations_done"] == 3


def test_batch_against_the_oracle_and_device_events():
    inst = _instances(3, seed=7, max_events=8000)
    with capi.StripBatch([g for g, _ in inst]) as b:
        for i, (_, ev) in enumerate(inst):
            b.set_events(i, torch.from_numpy(ev).cuda())  # device-resident input
        b.iterate(2)
        for i, (g, ev) in enumerate(inst):
            og = O.Geometry(g.radius, g.length, g.n_y, g.n_z, g.pixel, g.sigma_z, g.sigma_dl)
            want, _ = O.mlem_f(og, ev, 2, threads=8)
            assert rel_l2(b.instance(i).rho, want) < 1e-4, i


def test_tuned_batch_keeps_results_and_reports_plans():
    inst = _instances(6, seed=31)
    with capi.StripBatch([g for g, _ in inst]) as b:
        for i, (_, ev) in enumerate(inst):
            b.set_events(i, ev)
        b.tune(max_events=20000)
        plans = [b.plan(i) for i in range(len(inst))]
        assert all(p["raster_shape"] >= 1 and p["block_threads"] in (128, 256) for p in plans)
        assert sum(p["candidates"] for p in plans) >= 2
        b.iterate(2)
        for i, (g, ev) in enumerate(inst):
            want, _ = _single(g, ev, 2)
            assert rel_l2(b.instance(i).rho, want) < TOL, (i, plans[i])


def test_batch_with_large_box_events():
    # 1 mm pixels and wide kernels: some boxes exceed the tile windows and take
    # the batched large-box kernel
    g = capi.Geometry(450.0, 1000.0, 300, 400, 1.0, 14.0, 60.0)
    ev = capi.generate(phantom.random_ellipse_phantom(4, half_z=200, half_y=150, centre_z=100,
                                                      centre_y=80, axes=(10, 120)),
                       20000, 450.0, 1000.0, 14.0, 60.0, seed=4)
    with capi.StripBatch([g, g]) as b:
        b.set_events(0, ev)
        b.set_events(1, ev[:5000])
        b.iterate(2)
        for i, e in enumerate((ev, ev[:5000])):
            want, cnt = _single(g, e, 2)
            assert rel_l2(b.instance(i).rho, want) < TOL
            assert b.instance(i).counters()["n_oversize"] == cnt["n_oversize"]
        assert b.instance(0).counters()["n_oversize"] > 0


def test_batch_argument_checks():
    g = capi.Geometry(450.0, 1000.0, 90, 100, 10.0, 10.0, 42.0)
    with pytest.raises(capi.StripError):
        capi.StripBatch([g], precision=capi.PRECISION_FIXED)
    with capi.StripBatch([g]) as b:
        with pytest.raises(capi.StripError):
            b.iterate(1)  # events not set
        with pytest.raises(capi.StripError):
            b.set_events(3, np.zeros((1, 3), np.float32))
