"""The GB300 3D hybrid reconstruction (include/jpet_hybrid.h) against the
reference's own Reconstruction (golden runs in tests/golden/hybrid_ref.npz) and
against the CPU restatement (oracle/hybrid_oracle.inc) on a 96-detector ring.

Tolerances: frame events and given/normalized weights bit-exact (the set-up is
evaluated in the reference's rounding); computed weights and the sensitivity
within 1e-6 relative (the device expf and the host's may differ in the last
bit); each iteration started from the reference's previous image within 1e-5
relative L2 of the reference's next image (float sums in another order, the
exponential by ex2.approx and the frame sensitivity's two arctangents as one
atan2); free-running iterations within 1e-4.
"""
import ctypes as C
import os

import numpy as np
import pytest

import oracle as O
from jpet_strip import hybrid as HY
from jpet_strip import hybrid_workloads as H

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hybrid_ref.npz")
TOL_STEP = 1e-5
TOL_FREE = 1e-4


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def rel_max(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-30)))


@pytest.fixture(scope="module")
def ref():
    return np.load(GOLDEN)


CASES = ["computed", "given", "multiplane", "sens3d"]


def _modes(ref, tag):
    """(weights mode, sensitivity mode, sensitivity map, iterations) of a golden case."""
    gi = ref[tag + "_grid"]
    weights = HY.WEIGHTS_GIVEN if gi[4] else HY.WEIGHTS_COMPUTED
    if tag + "_sens_in" in ref:
        return weights, HY.SENSITIVITY_GIVEN_3D, ref[tag + "_sens_in"], int(gi[6])
    sens = HY.SENSITIVITY_ONE if gi[5] else HY.SENSITIVITY_COMPUTED
    return weights, sens, None, int(gi[6])


@pytest.mark.parametrize("tag", CASES)
def test_golden_setup_and_frame_events(ref, tag):
    g = H.from_arrays(ref, tag + "_")
    weights, sens, smap, _ = _modes(ref, tag)
    with HY.HybridReconstruction(g, weights, sens, smap) as r:
        w = r.weights
        if weights == HY.WEIGHTS_GIVEN:
            assert np.array_equal(w, ref[tag + "_weights"])
        else:
            assert rel_max(w, ref[tag + "_weights"]) < 1e-6
        assert rel_max(r.sensitivity[ref[tag + "_sens"] > 0],
                       ref[tag + "_sens"][ref[tag + "_sens"] > 0]) < 1e-6
        r << ref[tag + "_responses"]
        fr = r.frame_events()
        want = ref[tag + "_frame"]
        assert fr.shape == want.shape
        for name in want.dtype.names:
            assert np.array_equal(fr[name], want[name]), name
        st = r.statistics()
        assert [st["used_events"], st["used_pixels"], st["used_voxels"]] == list(
            ref[tag + "_stats"][0])


@pytest.mark.parametrize("tag", CASES)
def test_golden_iterations(ref, tag):
    g = H.from_arrays(ref, tag + "_")
    weights, sens, smap, n_iter = _modes(ref, tag)
    rhos = ref[tag + "_rho"]
    with HY.HybridReconstruction(g, weights, sens, smap) as step, \
            HY.HybridReconstruction(g, weights, sens, smap) as run:
        step << ref[tag + "_responses"]
        run << ref[tag + "_responses"]
        for it in range(n_iter):
            if it > 0:
                step.rho = rhos[it - 1]
            step(1)
            assert rel_l2(step.rho, rhos[it]) < TOL_STEP, it
            run(1)
            assert rel_l2(run.rho, rhos[it]) < TOL_FREE, it
        assert step.statistics()["contributing"] == ref[tag + "_frame"].shape[0]


@pytest.fixture(scope="module")
def ring96():
    g, n, n_iter = H.workload("hybrid-96")
    resp = H.responses(g, n, seed=11)
    w, s = O.hybrid_setup(g)
    frames = O.hybrid_translate(g, w, resp)
    return g, resp, w, s, frames, n_iter


def test_ring96_against_oracle(ring96):
    g, resp, w, s, frames, n_iter = ring96
    threads = os.cpu_count() or 1
    with HY.HybridReconstruction(g) as step, HY.HybridReconstruction(g) as run:
        assert rel_max(step.weights, w) < 1e-6
        assert rel_max(step.sensitivity[s > 0], s[s > 0]) < 1e-6
        step << resp
        run << resp
        fr = step.frame_events()
        for name in frames.dtype.names:
            assert np.array_equal(fr[name], frames[name]), name
        rho = None
        single, free = [], []
        for it in range(n_iter):
            nxt, cnt = O.hybrid_mlem(g, w, s, frames, 1, rho, threads=threads)
            if rho is not None:
                step.rho = rho
            step(1)
            single.append(rel_l2(step.rho, nxt))
            run(1)
            free.append(rel_l2(run.rho, nxt))
            st = step.statistics()
            assert [st["used_events"], st["used_pixels"], st["used_voxels"]] == list(cnt[:3])
            assert st["contributing"] == cnt[3]
            rho = nxt
    assert max(single) < TOL_STEP, single
    assert max(free) < TOL_FREE, free


@pytest.mark.parametrize("form", ["multiplane", "sens3d"])
def test_ring96_multiplane_and_3d_sensitivity_against_oracle(form):
    """The multi-plane form (one system matrix per plane half, 3D sensitivity
    computed per plane half) and the external 3D sensitivity on the 96-detector
    ring, events at every plane including plane 0 (where both sides clamp the
    plane the reference would read one past its arrays)."""
    g, _, _ = H.workload("hybrid-96", weights="given")
    smap = None
    if form == "multiplane":
        g = H.multiplane_weights(g, g.n_planes // 2, seed=21)
        mode = HY.SENSITIVITY_COMPUTED
    else:
        smap = np.random.default_rng(22).uniform(
            0.5, 1.5, (g.n_planes // 2) * g.n_columns * g.n_rows).astype(np.float32)
        mode = HY.SENSITIVITY_GIVEN_3D
    resp = H.responses(g, 40_000, seed=23)
    # a thousand of them moved to the grid's first planes
    resp["z_up"][:1000] = resp["z_dn"][:1000] = g.z_left + 1.5 * g.pixel_size
    w, s = O.hybrid_setup(g, weights_given=True, sens_given=smap)
    frames = O.hybrid_translate(g, w, resp)
    assert np.any(frames["plane_begin"] == 0)
    threads = os.cpu_count() or 1
    with HY.HybridReconstruction(g, HY.WEIGHTS_GIVEN, mode, smap) as r:
        assert np.array_equal(r.weights, w) if form == "sens3d" else rel_max(r.weights, w) < 1e-6
        assert rel_max(r.sensitivity[s > 0], s[s > 0]) < 1e-6
        r << resp
        rho = None
        for it in range(2):
            nxt, cnt = O.hybrid_mlem(g, w, s, frames, 1, rho, threads=threads)
            if rho is not None:
                r.rho = rho
            r(1)
            assert rel_l2(r.rho, nxt) < TOL_STEP, it
            st = r.statistics()
            assert [st["used_events"], st["used_pixels"], st["used_voxels"]] == list(cnt[:3])
            assert st["contributing"] == cnt[3]
            rho = nxt


def test_run_entry_point_schedule_and_result(ring96):
    """jpet_hybrid_run with normalized weights and a given sensitivity, as the
    reference's GPU run receives them: outputs at the reference's iterations,
    progress around each, result equal to the handle API's."""
    g, resp, w, s, frames, _ = ring96
    outs, prog = [], []
    rho0 = np.ones(g.n_voxels, np.float32)
    res, name = HY.run(g, w, s, frames, rho0, 2, 4, output=lambda i, img: outs.append(
        (i, float(img.sum()))), progress=lambda d, f: prog.append((d, f)))
    assert name
    # first block: after iterations 1, 2, 3 (i < n_in_block - 1); then after each block
    assert [i for i, _ in outs] == [1, 2, 3, 4, 8]
    assert prog[:2] == [(0, False), (0, True)] and prog[-1] == (8, False)
    # normalized weights are taken as they are
    gw = H.HybridGeometry(**{**g.__dict__, "weights": w})
    with HY.HybridReconstruction(gw, HY.WEIGHTS_NORMALIZED, HY.SENSITIVITY_GIVEN, s) as r:
        assert np.array_equal(r.weights, w)
        r.set_frame_events(frames)
        r(8)
        assert rel_l2(res, r.rho) < 1e-6


def test_rejects_bad_frame_events(ring96):
    g = ring96[0]
    frames = ring96[4][:16].copy()
    with HY.HybridReconstruction(g) as r:
        bad = frames.copy()
        bad["info_end"][3] = g.n_pixel_infos + 5
        with pytest.raises(HY.HybridError, match="outside the geometry"):
            r.set_frame_events(bad)
        bad = frames.copy()
        bad["plane_end"][2] = g.n_planes + 1
        with pytest.raises(HY.HybridError):
            r.set_frame_events(bad)
        bad = frames.copy()
        bad["first"][0] = 32000
        with pytest.raises(HY.HybridError):
            r.set_frame_events(bad)
        r.set_frame_events(frames)
        assert r.n_events == 16


def test_last_lor_range_is_clamped(ring96):
    """An event on the last LOR with pixel infos whose range would end one past
    the geometry's last info: the range is clamped (the reference would read past
    its arrays) and the iteration matches the oracle, which clamps the same way."""
    g, _, w, s, _, _ = ring96
    last = int(np.nonzero(g.info_end > g.info_begin)[0][-1])  # last LOR with pixel infos
    assert g.info_end[last] == g.n_pixel_infos
    first = int((np.sqrt(8 * last + 1) - 1) // 2)
    second = last - first * (first + 1) // 2
    seg = g.segments[last]
    R = float(seg["length"]) / 2
    r = np.zeros(4, H.RESPONSE_DTYPE)
    r["first"], r["second"] = first, second
    r["z_up"], r["z_dn"] = [0.0, 0.01, -0.02, 0.05], [0.0, 0.01, -0.02, 0.05]
    # the LOR's infos end inside the grid: events whose range reaches past them
    t_last = float(g.positions[g.n_pixel_infos - 1])
    up = (2 * t_last - 1) * R + np.array([-0.02, -0.01, 0.0, 0.01])
    r["dl"] = -2 * up
    frames = O.hybrid_translate(g, w, r)
    assert frames.shape[0] > 0 and np.all(frames["info_end"] <= g.n_pixel_infos)
    assert np.any(frames["info_end"] == g.n_pixel_infos)
    with HY.HybridReconstruction(g) as h:
        h << r
        fr = h.frame_events()
        for name in frames.dtype.names:
            assert np.array_equal(fr[name], frames[name]), name
        h(1)
        want, _ = O.hybrid_mlem(g, w, s, frames, 1)
        assert rel_l2(h.rho, want) < TOL_STEP


def test_create_rejects_pixels_outside_grid(ring96):
    g = ring96[0]
    bad = H.HybridGeometry(**{**g.__dict__, "pixels": g.pixels.copy()})
    bad.pixels["x"][7] = g.n_columns
    with pytest.raises(HY.HybridError, match="outside the pixel grid"):
        HY.HybridReconstruction(bad)


def test_create_rejects_a_lor_listing_a_pixel_twice(ring96):
    g = ring96[0]
    px = g.pixels.copy()
    l = 500
    b = int(g.info_begin[l])
    assert g.info_end[l] - b > 3
    px[b + 2] = px[b]
    bad = H.HybridGeometry(**{**g.__dict__, "pixels": px})
    with pytest.raises(HY.HybridError, match="same pixel twice"):
        HY.HybridReconstruction(bad)


def test_events_whose_range_leaves_their_lor_are_rejected(ring96):
    g, frames = ring96[0], ring96[4]
    with HY.HybridReconstruction(g) as r:
        bad = frames[:8].copy()
        f = bad["first"].astype(np.int64)
        lor = f * (f + 1) // 2 + bad["second"]
        bad["info_end"][1] = g.info_end[lor[1]] + 2
        with pytest.raises(HY.HybridError, match="one past its end"):
            r.set_frame_events(bad)
