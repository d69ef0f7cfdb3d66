"""GPU event generator (jpet_strip_generate) against the reference's own
2d_strip_phantom output and the generator's semantics."""
import json
import math
import os

import numpy as np
import pytest

from jpet_strip import capi, phantom

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
stats = pytest.importorskip("scipy.stats")

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
R, L = 450.0, 1000.0


def _emission_points(ev):
    """Inverse projection of exact responses (src/2d/strip/response.h:13-37)."""
    ev = ev.astype(np.float64)
    t = (ev[:, 0] - ev[:, 1]) / (2 * R)
    y = -0.5 * ev[:, 2] / np.sqrt(1 + t * t)
    z = 0.5 * (ev[:, 0] + ev[:, 1] + 2 * y * t)
    return z, y, t


def test_deterministic_for_a_seed():
    ell = phantom.three_ellipse_phantom()
    a = capi.generate(ell, 300000, R, L, 10.0, 42.0, seed=5)
    b = capi.generate(ell, 300000, R, L, 10.0, 42.0, seed=5)
    c = capi.generate(ell, 300000, R, L, 10.0, 42.0, seed=6)
    assert a.shape == (300000, 3) and np.isfinite(a).all()
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c)
    # a shorter request is a prefix of the longer stream
    d = capi.generate(ell, 1000, R, L, 10.0, 42.0, seed=5)
    assert np.array_equal(d, a[:1000])


def test_distribution_matches_reference_phantom_tool():
    ref = np.load(os.path.join(GOLDEN, "phantom_ref_events.npy"))
    ev = capi.generate(phantom.three_ellipse_phantom(), 200000, R, L, 10.0, 42.0, seed=21)
    for k in range(3):
        assert stats.ks_2samp(ref[:, k], ev[:, k]).pvalue > 1e-4, k
    t_ref = (ref[:, 0] - ref[:, 1]) / (2 * R)
    t_gpu = (ev[:, 0] - ev[:, 1]) / (2 * R)
    assert stats.ks_2samp(t_ref, t_gpu).pvalue > 1e-4


def test_detected_fraction_of_emissions_matches_reference():
    meta = json.load(open(os.path.join(GOLDEN, "phantom_ref.json")))
    p_ref = meta["detected"] / meta["emissions"]
    n = 10_000_000
    ev = capi.generate_device(phantom.three_ellipse_phantom(), n, R, L, 10.0, 42.0, seed=3,
                              detected=False)
    p = ev.shape[0] / n
    sig = math.sqrt(p_ref * (1 - p_ref) / meta["emissions"] + p * (1 - p) / n)
    assert abs(p - p_ref) < 5 * sig, (p, p_ref, sig)


def test_exact_responses_lie_in_the_regions_with_reference_weights():
    ell = phantom.three_ellipse_phantom()
    ev = capi.generate(ell, 200000, R, L, 0.0, 0.0, seed=8)
    assert (np.abs(ev[:, :2]) < L / 2).all()
    z, y, _ = _emission_points(ev)
    member = np.full(len(z), -1)
    for i in range(len(ell) - 1, -1, -1):
        inside = ell[i].contains(z, y * (1 - 1e-6))  # float32 responses: tiny slack
        member[inside] = i
    assert (member >= 0).mean() > 0.9999
    # region shares among detected events: same as the CPU generator's
    ev2 = phantom.generate_events(ell, 200000, R, L, 0.0, 0.0, seed=8)
    z2, y2, _ = _emission_points(ev2)
    member2 = np.full(len(z2), -1)
    for i in range(len(ell) - 1, -1, -1):
        member2[ell[i].contains(z2, y2)] = i
    for i in range(len(ell)):
        p1, p2 = (member == i).mean(), (member2 == i).mean()
        sig = math.sqrt(p1 * (1 - p1) / len(z) + p2 * (1 - p2) / len(z2))
        assert abs(p1 - p2) < 5 * sig + 1e-4, (i, p1, p2)


def test_point_and_rectangle_regions_and_additive_flag():
    pts = [(capi.REGION_POINT, 30.0, -20.0, 0, 0, 0, 1.0)]
    ev = capi.generate(pts, 20000, R, L, 0.0, 0.0, seed=2)
    z, y, _ = _emission_points(ev)
    assert np.abs(z - 30.0).max() < 1e-2 and np.abs(y + 20.0).max() < 1e-2
    rect = [(capi.REGION_RECTANGLE, -50.0, 40.0, 20.0, 10.0, 0, 1.0)]
    ev = capi.generate(rect, 50000, R, L, 0.0, 0.0, seed=2)
    z, y, _ = _emission_points(ev)
    assert (np.abs(z + 50.0) <= 20.0 + 1e-2).all() and (np.abs(y - 40.0) <= 10.0 + 1e-2).all()
    # an inner disc listed first masks the outer one (disjunctive) unless additive
    inner = phantom.Ellipse(0.0, 0.0, 50.0, 50.0, 0.0, 1.0)
    outer = phantom.Ellipse(0.0, 0.0, 100.0, 100.0, 0.0, 1.0)
    frac = []
    for additive in (False, True):
        ev = capi.generate([inner, outer], 200000, R, L, 0.0, 0.0, seed=4, additive=additive)
        z, y, _ = _emission_points(ev)
        frac.append((z * z + y * y < 50.0 ** 2).mean())
    # uniform density: the inner disc holds ~1/4 of the emissions; additive: 2/5
    assert 0.2 < frac[0] < 0.3 and 0.35 < frac[1] < 0.45, frac


@pytest.mark.parametrize("detected", [True, False])
def test_count_images_and_tan_map_match_the_oracle_binning(detected):
    """Count images of the phantom tool: the naive image and the tangent-binned
    map of the returned responses equal the oracle's float binning exactly
    (shifted grid origin included); every detected emission point is also an
    emitted one; emissions inside the grid are all counted."""
    import oracle as O

    ell = phantom.three_ellipse_phantom()
    geom = capi.Geometry(R, L, 180, 200, 5.0, 10.0, 42.0)
    og = O.Geometry(R, L, 180, 200, 5.0, 10.0, 42.0)
    origin = (7.5, -3.0)
    ev, im = capi.generate_with_images(ell, 300000, geom, seed=3, detected=detected,
                                       origin=origin, tan_bins=12)
    naive, tan = O.naive_bins(og, ev, origin=origin, tan_bins=12)
    assert np.array_equal(im["naive"], naive)
    assert np.array_equal(im["tan_map"], tan)
    assert (im["emitted"] >= im["detected"]).all()
    assert im["detected"].sum() == len(ev)  # the phantom lies inside the grid
    if not detected:
        assert im["emitted"].sum() == 300000
    assert 0 < tan.sum() <= naive.sum() <= len(ev)
    # the same events as without images
    plain = capi.generate(ell, 300000, R, L, 10.0, 42.0, seed=3, detected=detected)
    assert np.array_equal(plain, ev)


@pytest.mark.parametrize("divide", [False, True])
def test_tan_kernel_map_matches_the_oracle(divide):
    """The --tan-bins kernel map against the oracle's float restatement of the
    reference loop: the same float operations in the same order, with CUDA's
    expf/atanf for the C library's (a few ulp)."""
    import oracle as O

    geom = capi.Geometry(R, L, 90, 100, 10.0, 10.0, 42.0)
    og = O.Geometry(R, L, 90, 100, 10.0, 10.0, 42.0)
    kp, origin = (20.0, -10.0), (5.0, 0.0)
    got = capi.tan_kernel_map(geom, 16, kp, origin=origin, divide_by_sensitivity=divide)
    want = O.tan_kernel_map(og, 16, kp, origin=origin, divide_by_sensitivity=divide)
    assert got.shape == (16, 90, 100) and np.isfinite(got).all()
    scale = float(want.max())
    assert scale > 0
    assert float(np.max(np.abs(got - want))) <= 2e-6 * scale
    big = want > 1e-3 * scale
    np.testing.assert_allclose(got[big], want[big], rtol=2e-6)


def test_full_outputs_are_the_exact_projection_of_the_emission_events():
    """--full outputs: each emission event (x, y, sin phi, cos phi) projects to
    its exact response (scanner.h:107-113), which lies on the scintillators
    (scanner.h:208-213); the written response is that response plus the
    Gaussian smearing (sigma_z, sigma_dl); the events and responses keep the
    order and count of the plain stream."""
    ell = phantom.three_ellipse_phantom()
    geom = capi.Geometry(R, L, 180, 200, 5.0, 10.0, 42.0)
    ev, im = capi.generate_with_images(ell, 200000, geom, seed=4, full=True)
    ex, evs = im["exact"].astype(np.float64), im["events"].astype(np.float64)
    assert ex.shape == (len(ev), 3) and evs.shape == (len(ev), 4)
    x, y, sx, cx = evs.T
    assert np.allclose(sx * sx + cx * cx, 1.0, atol=1e-6)
    t = sx / cx
    np.testing.assert_allclose(ex[:, 0], x + (R - y) * t, rtol=1e-5, atol=2e-3)
    np.testing.assert_allclose(ex[:, 1], x - (R + y) * t, rtol=1e-5, atol=2e-3)
    np.testing.assert_allclose(ex[:, 2], -2 * y * np.sqrt(t * t + 1), rtol=1e-5, atol=2e-3)
    assert np.all(np.abs(ex[:, :2]) < L / 2)
    d = ev.astype(np.float64) - ex
    assert abs(d[:, 0].std() - 10.0) < 0.1 and abs(d[:, 1].std() - 10.0) < 0.1
    assert abs(d[:, 2].std() - 42.0) < 0.4 and abs(d.mean(0)).max() < 0.3
    plain = capi.generate(ell, 200000, R, L, 10.0, 42.0, seed=4)
    assert np.array_equal(plain, ev)
