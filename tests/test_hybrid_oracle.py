"""The CPU restatement of the 3D hybrid reconstruction (oracle/hybrid_oracle.inc)
against the reference's own Reconstruction run on the same inputs
(tests/golden/hybrid_ref.npz, made by make_hybrid_golden.py from the harness
compiled out of src/3d/hybrid/reconstruction.h): weights, sensitivity, frame
events and every iteration's image bit for bit, and the reference's statistics,
in the single-plane form (computed or given weights), the multi-plane form (one
system matrix per plane half, 3D sensitivity) and with an external 3D
sensitivity."""
import os

import numpy as np
import pytest

import oracle as O
from jpet_strip import hybrid_workloads as H

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hybrid_ref.npz")
CASES = ("computed", "given", "multiplane", "sens3d")


def setup(ref, tag, g):
    gi = ref[tag + "_grid"]
    sens_in = ref[tag + "_sens_in"] if tag + "_sens_in" in ref else None
    return O.hybrid_setup(g, bool(gi[4]), bool(gi[5]), sens_given=sens_in)


@pytest.fixture(scope="module")
def ref():
    return np.load(GOLDEN)


@pytest.mark.parametrize("tag", CASES)
def test_setup_and_frame_events_bit_exact(ref, tag):
    g = H.from_arrays(ref, tag + "_")
    w, s = setup(ref, tag, g)
    assert np.array_equal(w, ref[tag + "_weights"])
    assert np.array_equal(s, ref[tag + "_sens"])
    fr = O.hybrid_translate(g, w, ref[tag + "_responses"])
    want = ref[tag + "_frame"]
    assert fr.shape == want.shape
    for name in want.dtype.names:
        assert np.array_equal(fr[name], want[name]), name
    # the golden covers the filter and both ends of the info and plane ranges
    assert fr.shape[0] < ref[tag + "_responses"].shape[0]
    f = fr["first"].astype(np.int64)
    lor = f * (f + 1) // 2 + fr["second"]
    assert np.any(fr["info_end"] == g.info_end[lor] + 1)
    assert np.any(fr["info_begin"] == g.info_begin[lor])
    # (the multi-plane and 3D-sensitivity cases start at plane 1: for plane 0 the
    # reference reads one plane past its weight and sensitivity arrays)
    first = 0 if g.n_planes_half == 1 and tag + "_sens_in" not in ref else 1
    assert np.any(fr["plane_begin"] == first) and np.any(fr["plane_end"] == g.n_planes)


@pytest.mark.parametrize("tag", CASES)
def test_iterations_bit_exact(ref, tag):
    g = H.from_arrays(ref, tag + "_")
    gi = ref[tag + "_grid"]
    w, s = setup(ref, tag, g)
    fr = O.hybrid_translate(g, w, ref[tag + "_responses"])
    rho = None
    for it in range(int(gi[6])):
        rho, cnt = O.hybrid_mlem(g, w, s, fr, 1, rho, threads=1)
        assert np.array_equal(rho, ref[tag + "_rho"][it]), it
        assert list(cnt[:3]) == list(ref[tag + "_stats"][it])


def test_threads_agree_to_rounding(ref):
    g = H.from_arrays(ref, "computed_")
    w, s = O.hybrid_setup(g)
    fr = O.hybrid_translate(g, w, ref["computed_responses"])
    one, _ = O.hybrid_mlem(g, w, s, fr, 2, threads=1)
    four, _ = O.hybrid_mlem(g, w, s, fr, 2, threads=4)
    assert np.linalg.norm(one - four) / np.linalg.norm(one) < 1e-6
