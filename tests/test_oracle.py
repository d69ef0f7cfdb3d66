"""Pins the CPU oracle (oracle/strip_oracle.c) to the reference.

1. Known-answer values from the reference's own unit tests (the numbers are
   copied from the cited test files; their Catch harness is not buildable here).
2. Golden images written by the reference's own CPU tool (tests/golden/,
   generated by tests/golden/make_golden.py from oracle/_ref builds).
3. Invariants of the MLEM update.
"""
import math

import numpy as np
import pytest

import oracle as O


def _approx(got, want, eps):
    # Catch's Approx: |a - b| < eps * (1 + max(|a|, |b|))
    return abs(got - want) < eps * (1.0 + max(abs(got), abs(want)))


# src/2d/strip/gaussian_kernel_test.cpp:11-51 (F = float, sigma 0.01 / 0.04, R 0.35)
@pytest.mark.parametrize(
    "angle,y,dz,dy,want",
    [
        (math.pi / 6, 0.1, 0.0, 0.0, 184.304974530866),
        (math.pi / 6, 0.1, 0.05, 0.1, 5.272096361578383e-6),
        (math.pi / 6, 0.1, -0.05, -0.05, 0.0338473429952690),
        (math.pi / 4, -0.3, 0.0, 0.0, 95.87658397191050),
        (math.pi / 4, -0.3, 0.05, 0.1, 0.0),
        (math.pi / 4, -0.3, -0.05, -0.05, 0.1719727908599724),
    ],
)
def test_gaussian_kernel_known_answers(angle, y, dz, dy, want):
    a = np.float32(angle)
    sec = np.float32(1) / np.cos(a)
    tan = np.tan(a)
    got = O.gaussian_kernel_f(0.01, 0.04, y, float(tan), float(sec), 0.35, dz, dy)
    assert _approx(got, want, 1e-6), (got, want)


# src/2d/strip/kernel_test.cpp:31-49 (Scanner<double, short>, rel 1e-13)
@pytest.mark.parametrize(
    "R,L,z,y,want",
    [
        (500, 1000, 0, 0, 0.5),
        (500, 1000, 50, 0, 0.46652458328685176),
        (500, 1000, -50, 100, 0.4410019151324715),
        (500, 1000, -450, -200, 0.07526632771111386),
        (450, 200, 0, 0, 0.1392089745461279),
        (450, 200, 50, 0, 0.07044657495455454),
        (450, 200, -50, 100, 0.07402517367717103),
        (450, 200, -70, -200, 0.05269621503719814),
    ],
)
def test_sensitivity_known_answers(R, L, z, y, want):
    g = O.Geometry(R, L, 200, 200, 5, 10, 63)
    got = O.lib().orc_sensitivity_d(g.c(), z, y)
    assert _approx(got, want, 1e-13)


# src/2d/strip/kernel_test.cpp:81-112 (sigma_z 10, sigma_dl 63, rel 1e-4)
@pytest.mark.parametrize(
    "angle,bby,bbz",
    [
        (0.0470448, 94.3954, 21.6737),
        (-0.594145, 78.3053, 56.9959),
        (0.20029, 92.6108, 28.3458),
        (-0.571667, 79.4745, 55.3539),
        (-0.420542, 86.266, 44.0276),
    ],
)
def test_bbox_known_answers(angle, bby, bbz):
    ipd = 1.0 / (63.0 * 63.0)
    ipz = 1.0 / (10.0 * 10.0)
    A = (4.0 / (math.cos(angle) ** 2)) * ipd + 2.0 * math.tan(angle) ** 2 * ipz
    B = -4.0 * math.tan(angle) * ipz
    C = 2.0 * ipz
    B_2 = (B / 2.0) ** 2
    assert _approx(O.lib().orc_bb_y_dd(A, C, B_2), bby, 1e-4)
    assert _approx(O.lib().orc_bb_z_dd(A, C, B_2), bbz, 1e-4)


# src/2d/strip/response_test.cpp:11-55 (rel 1e-13)
@pytest.mark.parametrize(
    "y,z,deg,tan,zu,zd,dl",
    [
        (10.0, 20.0, 7.0, 0.1227845609029046, 74.02520679727803, -36.480898015336116,
         -20.15019650917697),
        (-10.0, 37.0, -5.0, -0.08748866352592401, -3.244785221925042, 75.49501195140655,
         20.076396750866948),
    ],
)
def test_projection_conversions(y, z, deg, tan, zu, zd, dl):
    import ctypes as C

    phi = deg * math.pi / 180.0
    t = math.sin(phi) / math.cos(phi)  # ImageSpaceEventAngle::to_tan (strip/event.h:25-28)
    assert _approx(t, tan, 1e-13)
    out = [C.c_double() for _ in range(3)]
    O.lib().orc_to_projection_space_tan_d(450.0, y, z, t, *[C.byref(v) for v in out])
    assert _approx(out[0].value, zu, 1e-13)
    assert _approx(out[1].value, zd, 1e-13)
    assert _approx(out[2].value, dl, 1e-13)
    # round trip through Response::calculate_tan_y_z in double
    R = 450.0
    t2 = (out[0].value - out[1].value) / (2 * R)
    y2 = -0.5 * (out[2].value / math.sqrt(1 + t2 * t2))
    z2 = 0.5 * (out[0].value + out[1].value + 2 * y2 * t2)
    assert _approx(y2, y, 1e-13) and _approx(z2, z, 1e-13)


# src/2d/strip/scanner_test.cpp:15-66
def test_pixel_at_and_center():
    import ctypes as C

    g = O.Geometry(500, 1000, 200, 200, 5, 10, 63).c()

    def at(z, y):
        px, py = C.c_int32(), C.c_int32()
        O.lib().orc_pixel_at_d(g, z, y, C.byref(px), C.byref(py))
        return px.value, py.value

    def center(gg, x, y):
        z, yy = C.c_double(), C.c_double()
        O.lib().orc_pixel_center_d(gg, x, y, C.byref(z), C.byref(yy))
        return z.value, yy.value

    assert at(0.0, 0.0) == (100, 100)
    assert at(-0.00001, 0.00001) == (99, 99)
    assert at(-500.0, 500.0) == (0, 0)
    assert at(500.0, 500.0) == (200, 0)
    assert at(-500.0, -500.0) == (0, 200)
    assert at(500.0, -500.0) == (200, 200)
    assert at(-499.99999, 499.99999) == (0, 0)
    assert at(499.99999, 499.99999) == (199, 0)
    assert at(-499.99999, -499.99999) == (0, 199)
    assert at(499.99999, -499.99999) == (199, 199)
    # Scanner(100, 200, 200, 200, 10, 63): pixel size 2R/n_y = L/n_z = 1
    g1 = O.Geometry(100, 200, 200, 200, 1.0, 10, 63).c()
    assert center(g1, 100, 100) == (0.5, -0.5)
    assert center(g1, 99, 99) == (-0.5, 0.5)
    assert center(g1, 0, 0) == (-99.5, 99.5)
    for z, y, want in [(0.0, 0.0, (2.5, -2.5)), (-6.0, 3.0, (-7.5, 2.5)), (6.0, 3.0, (7.5, 2.5)),
                       (-6.0, -3.0, (-7.5, -2.5)), (6.0, -3.0, (7.5, -2.5))]:
        assert center(g, *at(z, y)) == want


def _geom(c):
    g = c["geometry"]
    return O.Geometry(g["R"], g["L"], g["n_y"], g["n_z"], g["p"], g["sz"], g["sdl"])


@pytest.mark.parametrize("case", ["c1", "crop"])
def test_oracle_bit_exact_vs_reference_strict_build(golden, case):
    manifest, load = golden
    c = manifest[case]
    geom = _geom(c)
    ev = load(f"{case}_events.npy")
    rho = None
    done = 0
    for it in c["iterations"]:
        rho, _ = O.mlem_f(geom, ev, it - done, rho, threads=1)
        done = it
        want = load(f"{case}_strict_it{it:02d}.npy")
        assert np.array_equal(rho.view(np.uint32), want.view(np.uint32)), f"iteration {it}"


@pytest.mark.parametrize("case", ["c1", "crop"])
def test_oracle_vs_reference_release_build(golden, case):
    # the release build may contract a*b+c into FMA; the difference is rounding only
    manifest, load = golden
    c = manifest[case]
    it = c["iterations"][-1]
    rho, _ = O.mlem_f(_geom(c), load(f"{case}_events.npy"), it, threads=1)
    want = load(f"{case}_release_it{it:02d}.npy")
    rel = np.linalg.norm(rho - want) / np.linalg.norm(want)
    assert rel < 2e-6, rel


def test_oracle_fp64_vs_reference_template(golden):
    manifest, load = golden
    c = manifest["c1"]
    rho = O.mlem_d(_geom(c), load("c1_events.npy"), 3, threads=2)
    want = load("c1_fp64_it03.npy")
    rel = np.linalg.norm(rho - want) / np.linalg.norm(want)
    assert rel < 1e-12, rel


def test_mass_conservation_and_threads(golden):
    # sum(rho) after an iteration = number of events with a positive denominator
    manifest, load = golden
    c = manifest["c1"]
    ev = load("c1_events.npy")
    r1, st = O.mlem_f(_geom(c), ev, 1, threads=1)
    r4, _ = O.mlem_f(_geom(c), ev, 1, threads=4)
    assert st["n_contributing"] == len(ev)
    assert abs(float(r1.astype(np.float64).sum()) - st["n_contributing"]) < 1e-3
    assert np.linalg.norm(r1 - r4) / np.linalg.norm(r1) < 1e-6
    assert (r1 >= 0).all()


def test_gpuref_restatement_basic(golden):
    manifest, load = golden
    c = manifest["c1"]
    ev = load("c1_events.npy")[:2000]
    r = O.mlem_gpuref(_geom(c), ev, 1, threads=2)
    # each contributing event distributes exactly one unit (weights s only in den)
    # so the sum is below the event count by the sensitivity weighting
    assert np.isfinite(r).all() and (r >= 0).all()
    assert r.sum() > 0


def test_nll_gradient_matches_finite_differences(golden):
    manifest, load = golden
    c = manifest["c1"]
    g = _geom(c)
    ev = load("c1_events.npy")[:3000]
    rho, _ = O.mlem_f(g, ev, 2, threads=2)
    sup = (g.sigma_z, g.sigma_dl)
    loss, grad_rho, grad_s, skipped = O.nll_grad(g, ev, rho, support_sigma=sup)
    assert skipped == 0
    h = 1e-3
    for k, name in enumerate(("sigma_z", "sigma_dl")):
        gp = O.Geometry(**{**g.__dict__, name: getattr(g, name) + h})
        gm = O.Geometry(**{**g.__dict__, name: getattr(g, name) - h})
        lp = O.nll_grad(gp, ev, rho, support_sigma=sup, want_grad_rho=False)[0]
        lm = O.nll_grad(gm, ev, rho, support_sigma=sup, want_grad_rho=False)[0]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - grad_s[k]) <= 1e-5 * max(1.0, abs(fd)), (name, fd, grad_s[k])
    # d/drho at a few pixels
    rng = np.random.default_rng(0)
    idx = rng.choice(rho.size, 5, replace=False)
    for i in idx:
        hp = max(1e-3 * rho.flat[i], 1e-3)
        rp = rho.copy()
        rp.flat[i] += hp
        rm = rho.copy()
        rm.flat[i] -= hp
        lp = O.nll_grad(g, ev, rp, support_sigma=sup, want_grad_rho=False)[0]
        lm = O.nll_grad(g, ev, rm, support_sigma=sup, want_grad_rho=False)[0]
        fd = (lp - lm) / (2 * hp)
        assert abs(fd - grad_rho.flat[i]) <= 1e-4 * max(1.0, abs(fd)), (i, fd, grad_rho.flat[i])


@pytest.mark.skipif(O.ref_binary("ref_rec_strict") is None, reason="reference tools not built")
def test_oracle_vs_reference_binary_multithreaded(tmp_path, golden):
    import subprocess

    manifest, load = golden
    ev = load("c1_events.npy")
    p = tmp_path / "ev.bin"
    ev.tofile(p)
    subprocess.run([O.ref_binary("ref_rec_strict"), str(p), "-r", "450", "-l", "1000", "-p", "5",
                    "--n-z-pixels", "200", "--n-y-pixels", "180", "--s-z", "10", "--s-dl", "42",
                    "-i", "2", "-I", "1", "-T", "4", "-o", str(tmp_path / "r.bin")], check=True)
    want = np.fromfile(tmp_path / "r_2.bin", np.float32).reshape(180, 200)
    got, _ = O.mlem_f(O.Geometry(450, 1000, 180, 200, 5, 10, 42), ev, 2, threads=4)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-6


def test_point_source_likelihood_peaks_at_true_widths():
    """FP64 likelihood of a centred point source with its image known: the
    maximum over each width lies within 0.25 mm of the simulated (10, 42)."""
    from jpet_strip import phantom

    ev = phantom.generate_events(phantom.point_source(), 20000, 450.0, 1000.0, 10.0, 42.0, seed=5)
    img = phantom.point_image(450, 500, 2.0, [(-1.0, -1.0)]) * np.float32(len(ev))

    def loss(sz, sdl):
        g = O.Geometry(450.0, 1000.0, 450, 500, 2.0, sz, sdl)
        return O.nll_grad(g, ev, img, support_sigma=(14.0, 55.0), want_grad_rho=False)[0]

    for grid, f in (((9.5, 10.0, 10.5), lambda v: loss(v, 42.0)),
                    ((41.0, 42.0, 43.0), lambda v: loss(10.0, v))):
        l0, l1, l2 = (f(v) for v in grid)
        h = grid[1] - grid[0]
        vertex = grid[1] + 0.5 * h * (l0 - l2) / (l0 - 2 * l1 + l2)
        assert l0 - 2 * l1 + l2 > 0
        assert abs(vertex - grid[1]) < 0.25, (grid, l0, l1, l2, vertex)


def test_cpu_generator_matches_reference_phantom_tool():
    """The seeded CPU generator that feeds the parity tests draws from the same
    distribution as the reference's 2d_strip_phantom (two-sample KS against its
    committed events)."""
    import os

    from scipy import stats

    from jpet_strip import phantom

    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", "phantom_ref_events.npy"))
    ev = phantom.generate_events(phantom.three_ellipse_phantom(), 100000, 450.0, 1000.0, 10.0,
                                 42.0, seed=9)
    for k in range(3):
        assert stats.ks_2samp(ref[:, k], ev[:, k]).pvalue > 1e-4, k
    t_ref = (ref[:, 0] - ref[:, 1]) / 900.0
    t = (ev[:, 0] - ev[:, 1]) / 900.0
    assert stats.ks_2samp(t_ref, t).pvalue > 1e-4
