"""jpet_strip_iterate_noalloc: one MLEM iteration for callers that may not
allocate device memory (its per-event working data live in a fixed array of the
library).  Called through the C ABI on device buffers and compared with the
handle-based entry point, within the per-iteration tolerance of the parity
tests, on two calls in a row (the second reusing the first one's output)."""
import ctypes as C

import numpy as np
import pytest

from jpet_strip import capi

pytestmark = pytest.mark.gpu

TOL_ITER = 1e-5


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_matches_handle_entry_point(golden):
    torch = pytest.importorskip("torch")
    manifest, load = golden
    g = manifest["c1"]["geometry"]
    geom = capi.Geometry(g["R"], g["L"], g["n_y"], g["n_z"], g["p"], g["sz"], g["sdl"])
    ev = load("c1_events.npy")
    L = capi.lib()
    ev_d = torch.from_numpy(np.ascontiguousarray(ev)).cuda()
    img_a = torch.ones((geom.n_y, geom.n_z), dtype=torch.float32, device="cuda")
    img_b = torch.empty_like(img_a)
    stream = torch.cuda.current_stream().cuda_stream
    cg = geom.c()
    with capi.StripReconstruction(geom) as rec:
        rec.set_events(ev)
        src, dst = img_a, img_b
        for call in range(2):
            rc = L.jpet_strip_iterate_noalloc(C.byref(cg), ev_d.data_ptr(), len(ev),
                                              src.data_ptr(), dst.data_ptr(), stream)
            assert rc == capi.JPET_OK, L.jpet_strip_last_error(None)
            torch.cuda.synchronize()
            rec.iterate(1)
            want = rec.rho
            got = dst.cpu().numpy()
            assert rel_l2(got, want) < TOL_ITER, (call, rel_l2(got, want))
            src, dst = dst, src
    # a warm call allocates no device memory: free memory is the same before and after
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    rc = L.jpet_strip_iterate_noalloc(C.byref(cg), ev_d.data_ptr(), len(ev), src.data_ptr(),
                                      dst.data_ptr(), stream)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert rc == capi.JPET_OK
    assert free1 == free0, (free0, free1)


def test_noalloc_rejects_oversized_and_bad_arguments():
    torch = pytest.importorskip("torch")
    L = capi.lib()
    cg = capi.Geometry(450.0, 1000.0, 90, 100, 10.0, 10.0, 42.0).c()
    a = torch.zeros((90, 100), dtype=torch.float32, device="cuda")
    b = torch.zeros_like(a)
    ev = torch.zeros((4, 3), dtype=torch.float32, device="cuda")
    rc = L.jpet_strip_iterate_noalloc(C.byref(cg), ev.data_ptr(), (1 << 20) + 1, a.data_ptr(),
                                      b.data_ptr(), None)
    assert rc == capi.JPET_ERR_ARGUMENT
    assert b"at most 1048576" in L.jpet_strip_last_error(None)
    rc = L.jpet_strip_iterate_noalloc(C.byref(cg), ev.data_ptr(), 4, a.data_ptr(), a.data_ptr(),
                                      None)
    assert rc == capi.JPET_ERR_ARGUMENT
    # partly overlapping images, and an output over the responses
    rc = L.jpet_strip_iterate_noalloc(C.byref(cg), ev.data_ptr(), 4, a.data_ptr(),
                                      a.data_ptr() + 4 * 100, None)
    assert rc == capi.JPET_ERR_ARGUMENT
    assert b"overlaps" in L.jpet_strip_last_error(None)
    rc = L.jpet_strip_iterate_noalloc(C.byref(cg), a.data_ptr(), 4, b.data_ptr(), a.data_ptr(),
                                      None)
    assert rc == capi.JPET_ERR_ARGUMENT
