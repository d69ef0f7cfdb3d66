"""Host-side checks of the 3D hybrid C ABI that need no GPU: the geometry is
validated before any device is touched, with status codes and messages."""
import ctypes as C

import numpy as np
import pytest

from jpet_strip import hybrid as HY
from jpet_strip import hybrid_workloads as H


@pytest.fixture(scope="module")
def tiny():
    return H.workload("hybrid-tiny")[0]


def _create(g, opts=None):
    L = HY._lib()
    gs, keep = HY.geom_struct(g)
    h = C.c_void_p()
    rc = L.jpet_hybrid_create(C.byref(gs), C.byref(opts) if opts else None, C.byref(h))
    return rc, L.jpet_hybrid_last_error(None).decode()


def test_struct_layouts_match_the_reference_types():
    # FrameEvent with F = float, S = short, 64-bit size_t; LineSegment<float>; Response
    assert H.FRAME_EVENT_DTYPE.itemsize == 48
    assert H.SEGMENT_DTYPE.itemsize == 48
    assert H.RESPONSE_DTYPE.itemsize == 16
    assert C.sizeof(HY.HybGeom) == 120


def test_rejects_bad_geometry_without_device(tiny):
    bad = H.HybridGeometry(**{**tiny.__dict__, "n_detectors": 0})
    rc, msg = _create(bad)
    assert rc == -1 and "n_detectors" in msg
    bad = H.HybridGeometry(**{**tiny.__dict__, "n_planes": 0})
    rc, msg = _create(bad)
    assert rc == -1 and "grid" in msg
    ib = tiny.info_begin.copy()
    ib[5] = tiny.info_end[5] + 1
    bad = H.HybridGeometry(**{**tiny.__dict__, "info_begin": ib})
    rc, msg = _create(bad)
    assert rc == -1 and "LOR 5" in msg
    bad = H.HybridGeometry(**{**tiny.__dict__, "sigma_z": 0.0})
    rc, msg = _create(bad)
    assert rc == -1 and "positive" in msg


def test_rejects_bad_modes_without_device(tiny):
    o = HY.HybOpts(0, 7, 0, None, 0, 0)
    rc, msg = _create(tiny, o)
    assert rc == -1 and "mode" in msg
    o = HY.HybOpts(0, 0, HY.SENSITIVITY_GIVEN, None, 0, 0)
    rc, msg = _create(tiny, o)
    assert rc == -1 and "sensitivity_map" in msg
    assert HY._lib().jpet_hybrid_destroy(None) == 0


def test_rejects_bad_multiplane_forms_without_device(tiny):
    """One system matrix per plane half needs given weights and a 3D
    sensitivity; n_planes_half may not exceed the planes; an external 3D
    sensitivity needs at least two planes."""
    mp = H.multiplane_weights(tiny, tiny.n_planes // 2, seed=1)
    rc, msg = _create(mp)
    assert rc == -1 and "given weights" in msg
    smap = np.ones(tiny.n_columns * tiny.n_rows, np.float32)
    o = HY.HybOpts(0, HY.WEIGHTS_GIVEN, HY.SENSITIVITY_GIVEN, smap.ctypes.data, 0, 0)
    rc, msg = _create(mp, o)
    assert rc == -1 and "3D sensitivity" in msg
    bad = H.HybridGeometry(**{**mp.__dict__, "n_planes_half": tiny.n_planes + 1})
    o = HY.HybOpts(0, HY.WEIGHTS_GIVEN, HY.SENSITIVITY_ONE, None, 0, 0)
    rc, msg = _create(bad, o)
    assert rc == -1 and "n_planes_half" in msg
    flat = H.HybridGeometry(**{**tiny.__dict__, "n_planes": 1})
    o = HY.HybOpts(0, HY.WEIGHTS_COMPUTED, HY.SENSITIVITY_GIVEN_3D, smap.ctypes.data, 0, 0)
    rc, msg = _create(flat, o)
    assert rc == -1 and "2 planes" in msg
