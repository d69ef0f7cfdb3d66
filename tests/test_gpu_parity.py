"""Parity of the sm_103a MLEM iteration (through the C ABI) with the CPU oracle.

Tolerances: per-iteration relative L2 <= 1e-5 against the reference float path
(the bar the path is built to), <= 1e-4 after 20 iterations.  Integer outputs
(kernel-call and pixel counters) must be identical.
"""
import numpy as np
import pytest

import oracle as O
from jpet_strip import capi, phantom

pytestmark = pytest.mark.gpu

TOL_ITER = 1e-5
VARIANTS = [capi.VARIANT_FAST, capi.VARIANT_EXACT, capi.VARIANT_WARP, capi.VARIANT_ROWS]


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


def _geoms(c):
    g = c["geometry"]
    args = (g["R"], g["L"], g["n_y"], g["n_z"], g["p"], g["sz"], g["sdl"])
    return capi.Geometry(*args), O.Geometry(*args)


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("case", ["c1", "crop"])
def test_iterations_match_reference_goldens(golden, case, variant):
    manifest, load = golden
    c = manifest[case]
    cg, _ = _geoms(c)
    ev = load(f"{case}_events.npy")
    with capi.StripReconstruction(cg, variant=variant) as rec:
        rec.set_events(ev)
        done = 0
        for it in c["iterations"]:
            rec.iterate(it - done)
            done = it
            got = rec.rho
            want = load(f"{case}_strict_it{it:02d}.npy")
            assert rel_l2(got, want) < TOL_ITER, (case, it, rel_l2(got, want))
        want = load(f"{case}_release_it{done:02d}.npy")
        assert rel_l2(got, want) < TOL_ITER


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("case", ["c1", "crop"])
def test_each_iteration_and_counters_match_oracle(golden, case, variant):
    manifest, load = golden
    c = manifest[case]
    cg, og = _geoms(c)
    ev = load(f"{case}_events.npy")
    with capi.StripReconstruction(cg, variant=variant) as rec:
        rec.set_events(ev)
        rho = None
        for it in range(3):
            rec.iterate(1)
            rho, st = O.mlem_f(og, ev, 1, rho, threads=4)
            got = rec.rho
            assert rel_l2(got, rho) < TOL_ITER, (it, rel_l2(got, rho))
            cnt = rec.counters()
            assert cnt["n_kernel_calls"] == st["n_kernel_calls"]
            assert cnt["n_pixels"] == st["n_pixels"]
            assert cnt["n_contributing"] == st["n_contributing"]
            rec.rho = rho  # continue both from the same image


@pytest.mark.parametrize("variant", VARIANTS)
def test_twenty_iterations_stay_within_1e4(golden, variant):
    manifest, load = golden
    cg, og = _geoms(manifest["c1"])
    ev = load("c1_events.npy")
    with capi.StripReconstruction(cg, variant=variant) as rec:
        rec.set_events(ev)
        rec.iterate(20)
        got = rec.rho
    want, _ = O.mlem_f(og, ev, 20, threads=8)
    assert rel_l2(got, want) < 1e-4


def test_mass_conservation_and_nonnegativity(golden):
    manifest, load = golden
    cg, _ = _geoms(manifest["c1"])
    ev = load("c1_events.npy")
    with capi.StripReconstruction(cg) as rec:
        rec.set_events(ev)
        rec.iterate(2)
        r = rec.rho
        cnt = rec.counters()
    assert (r >= 0).all()
    assert abs(r.astype(np.float64).sum() - cnt["n_contributing"]) < 1e-6 * len(ev) + 1e-2


def test_initial_image_and_set_image_roundtrip():
    g = capi.Geometry(450, 1000, 90, 100, 10, 10, 42)
    with capi.StripReconstruction(g) as rec:
        assert np.array_equal(rec.rho, np.ones((90, 100), np.float32))
        x = np.random.default_rng(0).random((90, 100)).astype(np.float32)
        rec.rho = x
        assert np.array_equal(rec.rho, x)


def test_empty_event_list_and_iterate_before_events():
    g = capi.Geometry(450, 1000, 90, 100, 10, 10, 42)
    with capi.StripReconstruction(g) as rec:
        with pytest.raises(capi.StripError) as e:
            rec.iterate(1)
        assert e.value.code == capi.JPET_ERR_STATE
        rec.set_events(np.zeros((0, 3), np.float32))
        rec.iterate(1)
        assert not rec.rho.any()


@pytest.mark.parametrize("variant", VARIANTS)
def test_edge_events_outside_grid_nan_and_single(golden, variant):
    # events far outside, on the grid corner, NaN and Inf: same result as the oracle
    og = O.Geometry(450, 1000, 90, 100, 5, 10, 42)
    cg = capi.Geometry(450, 1000, 90, 100, 5, 10, 42)
    ev = np.array([
        [0.0, 0.0, 0.0],            # centre
        [240.0, 260.0, 200.0],      # near the grid corner
        [900.0, 900.0, 0.0],        # far outside in z
        [0.0, 0.0, 2000.0],         # far outside in y
        [np.nan, 0.0, 0.0],
        [np.inf, -np.inf, 0.0],
        [1e30, -1e30, 1e30],
        [-249.0, -251.0, -170.0],
    ], np.float32)
    for sl in (slice(0, 1), slice(None)):
        with capi.StripReconstruction(cg, variant=variant) as rec:
            rec.set_events(ev[sl])
            rec.iterate(1)
            got = rec.rho
            cnt = rec.counters()
        want, st = O.mlem_f(og, ev[sl], 1, threads=1)
        assert np.isfinite(got).all()
        assert rel_l2(got, want) < TOL_ITER
        assert cnt["n_kernel_calls"] == st["n_kernel_calls"]


def test_zero_image_gives_zero_without_nan(golden):
    manifest, load = golden
    cg, og = _geoms(manifest["c1"])
    ev = load("c1_events.npy")[:500]
    with capi.StripReconstruction(cg) as rec:
        rec.set_events(ev)
        rec.rho = np.zeros((cg.n_y, cg.n_z), np.float32)
        rec.iterate(1)
        got = rec.rho
        assert rec.counters()["n_contributing"] == 0
    assert not got.any()


def test_sensitivity_maps_match_oracle():
    for g in [(450, 1000, 180, 200, 5, 10, 42), (500, 200, 64, 40, 5, 10, 63)]:
        cg, og = capi.Geometry(*g), O.Geometry(*g)
        with capi.StripReconstruction(cg) as rec:
            for kind in (0, 1):
                got = rec.sensitivity(kind)
                want = O.sensitivity_map(og, kind)
                np.testing.assert_allclose(got, want, rtol=2e-6, atol=1e-7)


def test_gpu_reference_semantics_mode(golden):
    manifest, load = golden
    cg, og = _geoms(manifest["c1"])
    ev = load("c1_events.npy")
    with capi.StripReconstruction(cg, mode=capi.MODE_GPU_REFERENCE) as rec:
        rec.set_events(ev)
        rec.iterate(2)
        got = rec.rho
    want = O.mlem_gpuref(og, ev, 2, threads=4)
    assert rel_l2(got, want) < TOL_ITER


def test_run_callback_protocol(golden):
    manifest, load = golden
    cg, og = _geoms(manifest["c1"])
    ev = load("c1_events.npy")[:3000]
    rho = np.ones((cg.n_y, cg.n_z), np.float32)
    outputs, progress = [], []
    name = capi.run(cg, ev, rho, 2, 3, output=lambda it, img: outputs.append((it, img)),
                    progress=lambda done, fin: progress.append((done, fin)))
    assert name
    # output(-1, sensitivity), then i+1 for i < I-1 in block 0, then block ends
    assert [o[0] for o in outputs] == [-1, 1, 2, 3, 6]
    assert progress[:2] == [(0, False), (0, True)] and progress[-1] == (6, False)
    want, _ = O.mlem_f(og, ev, 6, threads=4)
    assert rel_l2(rho, want) < 1e-5
    assert rel_l2(outputs[-1][1], want) < 1e-5
    np.testing.assert_allclose(outputs[0][1], O.sensitivity_map(og, 1), rtol=2e-6)


@pytest.mark.parametrize("variant", VARIANTS)
def test_tiling_does_not_change_results(golden, variant):
    # results are independent of the tile shape (1x1 tiles: one window per pixel)
    manifest, load = golden
    cg, og = _geoms(manifest["c1"])
    ev = load("c1_events.npy")
    want, st = O.mlem_f(og, ev, 1, threads=4)
    for tw, th in [(1, 1), (8, 32), (64, 16)]:
        with capi.StripReconstruction(cg, tile_w=tw, tile_h=th, variant=variant) as rec:
            rec.set_events(ev)
            rec.iterate(1)
            assert rel_l2(rec.rho, want) < TOL_ITER
            assert rec.counters()["n_kernel_calls"] == st["n_kernel_calls"]


@pytest.mark.parametrize("variant", VARIANTS)
def test_larger_random_phantom_against_oracle(variant):
    # 2 mm grid, 10-ellipse phantom, 30k events
    ell = phantom.random_ellipse_phantom(seed=7)
    ev = phantom.generate_events(ell, 30000, 450.0, 1000.0, 10.0, 42.0, seed=7)
    args = (450.0, 1000.0, 450, 500, 2.0, 10.0, 42.0)
    cg, og = capi.Geometry(*args), O.Geometry(*args)
    with capi.StripReconstruction(cg, variant=variant) as rec:
        rec.set_events(ev)
        rho = None
        for _ in range(2):
            rec.iterate(1)
            rho, st = O.mlem_f(og, ev, 1, rho, threads=8)
            assert rel_l2(rec.rho, rho) < TOL_ITER
            rec.rho = rho
        assert rec.counters()["n_kernel_calls"] == st["n_kernel_calls"]


@pytest.mark.parametrize("sigma", [(5.0, 20.0, 1.0), (14.0, 55.0, 2.0), (10.0, 42.0, 5.0),
                                   (6.0, 60.0, 3.0)])
def test_fast_kernel_register_shapes(sigma):
    # geometries that select each register-cache shape of the fast kernel
    sz, sdl, p = sigma
    n_z, n_y = int(1000 / p), int(900 / p)
    n_z, n_y = min(n_z, 400), min(n_y, 360)
    ell = phantom.random_ellipse_phantom(seed=3)
    ev = phantom.generate_events(ell, 8000, 450.0, 1000.0, sz, sdl, seed=3)
    args = (450.0, 1000.0, n_y, n_z, p, sz, sdl)
    cg, og = capi.Geometry(*args), O.Geometry(*args)
    with capi.StripReconstruction(cg) as rec:
        rec.set_events(ev)
        rec.iterate(2)
        got = rec.rho
        cnt = rec.counters()
    want, st = O.mlem_f(og, ev, 2, threads=8)
    assert rel_l2(got, want) < TOL_ITER
    assert cnt["n_kernel_calls"] == st["n_kernel_calls"]


@pytest.mark.parametrize("threads", [128, 256])
@pytest.mark.parametrize("precision", [capi.PRECISION_FP32, capi.PRECISION_FIXED,
                                       capi.PRECISION_COMPENSATED, capi.PRECISION_FP64_DEN])
@pytest.mark.parametrize("shape", sorted(capi.RASTER_SHAPES))
def test_row_owned_kernel_every_shape(shape, precision, threads):
    """Every register shape of the row-owned kernel, forced, on 2 mm events whose
    boxes (64 rows, 22 columns) overflow the small shapes: those events take
    the queued exact path, the rest the register path; both give the
    reference's image and counters."""
    ell = phantom.random_ellipse_phantom(seed=5)
    ev = phantom.generate_events(ell, 6000, 450.0, 1000.0, 10.0, 42.0, seed=5)
    args = (450.0, 1000.0, 450, 500, 2.0, 10.0, 42.0)
    cg, og = capi.Geometry(*args), O.Geometry(*args)
    want, st = O.mlem_f(og, ev, 1, threads=8)
    with capi.StripReconstruction(cg, precision=precision, block_threads=threads,
                                  raster_shape=capi.RASTER_SHAPES[shape],
                                  variant=capi.VARIANT_ROWS) as rec:
        rec.set_events(ev)
        rec.iterate(1)
        got = rec.rho
        cnt = rec.counters()
    # fixed-point tiles round every contribution to 2^-22 of an event: with
    # 6000 events on 225000 pixels (about 1e-3 of an event per contribution,
    # ~50 per pixel) that alone is ~1e-5 relative
    tol = 3e-5 if precision == capi.PRECISION_FIXED else TOL_ITER
    assert rel_l2(got, want) < tol
    assert cnt["n_kernel_calls"] == st["n_kernel_calls"]
    assert cnt["n_contributing"] == st["n_contributing"]
    small = shape in ("8x1x1", "8x1x2", "4x1x2")
    assert (cnt["n_exact_path"] > 0) == small, cnt


@pytest.mark.parametrize("precision", [capi.PRECISION_COMPENSATED, capi.PRECISION_FP64_DEN,
                                       capi.PRECISION_FIXED])
def test_compensated_precision_modes(golden, precision):
    manifest, load = golden
    cg, og = _geoms(manifest["c1"])
    ev = load("c1_events.npy")
    f64 = load("c1_fp64_it03.npy")
    with capi.StripReconstruction(cg, precision=precision) as rec:
        rec.set_events(ev)
        rho = None
        for it in range(3):
            rec.iterate(1)
            rho, st = O.mlem_f(og, ev, 1, rho, threads=4)
            assert rel_l2(rec.rho, rho) < TOL_ITER
            cnt = rec.counters()
            assert cnt["n_kernel_calls"] == st["n_kernel_calls"]
            assert cnt["n_contributing"] == st["n_contributing"]
            rec.rho = rho
    with capi.StripReconstruction(cg, precision=precision) as rec, \
            capi.StripReconstruction(cg) as plain:
        rec.set_events(ev)
        plain.set_events(ev)
        rec.iterate(3)
        plain.iterate(3)
        e_comp = rel_l2(rec.rho, f64)
        e_plain = rel_l2(plain.rho, f64)
    # error against the FP64 reference template: compensated tiles are not worse
    # than plain FP32; fixed-point tiles are quantized to 2^-22 of an event
    if precision == capi.PRECISION_FIXED:
        assert e_comp < 1e-5, e_comp
    else:
        assert e_comp <= 1.05 * e_plain + 1e-9, (e_comp, e_plain)


@pytest.mark.parametrize("threads", [128, 256])
@pytest.mark.parametrize("precision", [capi.PRECISION_FP32, capi.PRECISION_FIXED,
                                       capi.PRECISION_COMPENSATED, capi.PRECISION_FP64_DEN])
def test_batch_union_kernel_every_precision_mode(precision, threads):
    """The default (FAST) kernel in every accumulation mode on 2 mm events, where
    it takes the chain form of the exponent (two ex2 per event, row and lane,
    the further pixel pairs stepped by a constant ratio): each image matches
    the reference float path and the counters match exactly; the fixed-point
    image is the same bit for bit on a second run."""
    ell = phantom.random_ellipse_phantom(seed=9)
    ev = phantom.generate_events(ell, 8000, 450.0, 1000.0, 10.0, 42.0, seed=9)
    args = (450.0, 1000.0, 450, 500, 2.0, 10.0, 42.0)
    cg, og = capi.Geometry(*args), O.Geometry(*args)
    want, st = O.mlem_f(og, ev, 2, threads=8)
    imgs = []
    for _ in range(2 if precision == capi.PRECISION_FIXED else 1):
        with capi.StripReconstruction(cg, precision=precision, block_threads=threads) as rec:
            rec.set_events(ev)
            rec.iterate(2)
            imgs.append(rec.rho.copy())
            cnt = rec.counters()
    # fixed point: one rounding to 2^-22 of an event per batch and pixel
    tol = 3e-5 if precision == capi.PRECISION_FIXED else TOL_ITER
    assert rel_l2(imgs[0], want) < tol
    assert cnt["n_kernel_calls"] == st["n_kernel_calls"]
    assert cnt["n_contributing"] == st["n_contributing"]
    assert cnt["n_exact_path"] == 0 and cnt["n_oversize"] == 0, cnt
    if precision == capi.PRECISION_FIXED:
        assert np.array_equal(imgs[0], imgs[1])


def test_precision_mode_argument_checks():
    g = capi.Geometry(450, 1000, 90, 100, 10, 10, 42)
    with pytest.raises(capi.StripError) as e:
        capi.StripReconstruction(g, precision=7)
    assert e.value.code == capi.JPET_ERR_ARGUMENT
    with pytest.raises(capi.StripError) as e:
        capi.StripReconstruction(g, precision=capi.PRECISION_COMPENSATED,
                                 variant=capi.VARIANT_EXACT)
    assert e.value.code == capi.JPET_ERR_UNSUPPORTED


def test_fp64_reference_iteration_matches_fp64_oracle(golden):
    """jpet_strip_reference_fp64 is the reference template at double: it matches
    the FP64 oracle (and so the reference's own double instantiation) to
    summation-order rounding, with the same counters."""
    manifest, load = golden
    cg, og = _geoms(manifest["c1"])
    ev = load("c1_events.npy")
    got, cnt = capi.reference_fp64(cg, ev, 3)
    want = load("c1_fp64_it03.npy")
    assert rel_l2(got, want) < 1e-12
    _, st = O.mlem_f(og, ev, 1, threads=4)
    assert cnt["n_kernel_calls"] == st["n_kernel_calls"]
    # and on the cropped 2 mm case (clamped boxes) against the oracle at double
    cg2, og2 = _geoms(manifest["crop"])
    ev2 = load("crop_events.npy")
    got2, _ = capi.reference_fp64(cg2, ev2, 2)
    want2 = O.mlem_d(og2, ev2, 2, threads=4)
    assert rel_l2(got2, want2) < 1e-12


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("grid", [(12, 16, 5.0, 5.0), (90, 120, 2.0, 3.0), (300, 200, 4.0, 2.5),
                                  (7, 500, 2.0, 2.0)])
def test_small_and_non_square_grids(grid, variant):
    """Tiny grids (windows narrower than the widest sweep), rows taller or
    shorter than the columns are wide, and a grid a few rows high: every kernel
    against the oracle (the reference's Scanner keeps pixel_width and
    pixel_height apart, scanner.h:39-67)."""
    n_y, n_z, pw, ph = grid
    ell = phantom.random_ellipse_phantom(seed=9, half_z=min(500.0, n_z * pw / 2),
                                         half_y=min(450.0, n_y * ph / 2), centre_z=20.0,
                                         centre_y=10.0, axes=(5.0, 200.0))
    ev = phantom.generate_events(ell, 5000, 450.0, 1000.0, 10.0, 42.0, seed=9)
    args = (450.0, 1000.0, n_y, n_z, pw, 10.0, 42.0)
    cg = capi.Geometry(*args, pixel_height=ph)
    og = O.Geometry(*args, pixel_height=ph)
    want, st = O.mlem_f(og, ev, 2, threads=8)
    with capi.StripReconstruction(cg, variant=variant) as rec:
        rec.set_events(ev)
        rec.iterate(2)
        got = rec.rho
        cnt = rec.counters()
    assert rel_l2(got, want) < TOL_ITER
    assert cnt["n_kernel_calls"] == st["n_kernel_calls"]


def test_upload_paths_agree(golden):
    """Host AoS (one contiguous copy read with stride 3), host SoA and device SoA
    uploads prepare the same events: the same image and counters, repeated
    uploads of different sizes included (the staging buffer is reused)."""
    import ctypes as C

    import torch

    manifest, load = golden
    cg, og = _geoms(manifest["c1"])
    ev = load("c1_events.npy")
    want, st = O.mlem_f(og, ev, 1, threads=4)
    soa = np.ascontiguousarray(ev.T)
    dev = torch.from_numpy(soa).to("cuda:0")
    imgs, cnts = [], []
    with capi.StripReconstruction(cg) as rec:
        for how in ("aos_small", "aos", "soa", "device", "aos"):
            if how == "aos_small":
                rec.set_events(ev[:1000])
            elif how == "aos":
                rec.set_events(ev)
            elif how == "soa":
                L = capi.lib()
                rc = L.jpet_strip_set_events_soa(rec._h, soa[0].ctypes.data, soa[1].ctypes.data,
                                                 soa[2].ctypes.data, len(ev))
                assert rc == capi.JPET_OK
            else:
                rec.set_events_device(dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(),
                                      len(ev))
            rec.rho = np.ones((cg.n_y, cg.n_z), np.float32)
            rec.iterate(1)
            if how != "aos_small":
                imgs.append(rec.rho)
                c = rec.counters()
                c.pop("iterations_done")
                cnts.append(c)
    for img, c in zip(imgs, cnts):
        assert rel_l2(img, want) < TOL_ITER
        assert c == cnts[0] and c["n_kernel_calls"] == st["n_kernel_calls"]


@pytest.mark.parametrize("variant", VARIANTS)
def test_fine_pixels_with_boxes_beyond_every_shape(variant):
    """0.5 mm pixels with sigma 10/42: boxes of ~250 x 85 pixels exceed every
    register shape and most exceed the shared-memory window, so the events take
    the queued reference-order path and the global large-box path; the image
    and counters are still the reference's."""
    ell = phantom.random_ellipse_phantom(seed=12, half_z=120.0, half_y=90.0, centre_z=60.0,
                                         centre_y=50.0, axes=(5.0, 60.0))
    ev = phantom.generate_events(ell, 1500, 450.0, 1000.0, 10.0, 42.0, seed=12)
    args = (450.0, 1000.0, 400, 500, 0.5, 10.0, 42.0)
    cg, og = capi.Geometry(*args), O.Geometry(*args)
    want, st = O.mlem_f(og, ev, 2, threads=8)
    with capi.StripReconstruction(cg, variant=variant) as rec:
        rec.set_events(ev)
        rec.iterate(2)
        got = rec.rho
        cnt = rec.counters()
    assert rel_l2(got, want) < TOL_ITER
    assert cnt["n_kernel_calls"] == st["n_kernel_calls"]
    assert cnt["n_contributing"] == st["n_contributing"]
    if variant != capi.VARIANT_EXACT:
        assert cnt["n_oversize"] + cnt["n_exact_path"] > 0, cnt


def test_fixed_point_mode_is_deterministic(golden):
    """Fixed-point tiles summed into the 64-bit integer image: two runs give the
    same image bit for bit (integer sums do not depend on their order)."""
    manifest, load = golden
    cg, _ = _geoms(manifest["c1"])
    ev = load("c1_events.npy")
    imgs = []
    for _ in range(2):
        with capi.StripReconstruction(cg, precision=capi.PRECISION_FIXED) as rec:
            rec.set_events(ev)
            rec.iterate(3)
            assert rec.counters()["n_exact_path"] == 0 and rec.counters()["n_oversize"] == 0
            imgs.append(rec.rho.copy())
    assert np.array_equal(imgs[0], imgs[1])
