"""C-ABI checks that need no GPU: the library builds, loads and exports every
symbol include/jpet_strip.h declares; argument errors are reported as status
codes without touching a device."""
import ctypes as C
import os
import re

import pytest

from jpet_strip import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))
           if f.endswith(".h")]


def _declared():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(jpet_\w+)\s*\(", text):
            names.add(m.group(1))
        for m in re.finditer(r"typedef\s+\w+\s*\(\*\s*(jpet_\w+)\)", text):
            names.discard(m.group(1))
    return sorted(names)


def test_header_declares_and_library_exports_every_symbol():
    L = capi.lib()
    declared = _declared()
    assert declared, "no declarations found"
    missing = [n for n in declared if not hasattr(L, n)]
    assert not missing, missing
    assert set(capi.EXPORTED) >= set(n for n in declared if n.startswith("jpet_strip"))


def test_abi_version_and_defaults():
    L = capi.lib()
    assert L.jpet_strip_abi_version() == 1
    o = capi.make_opts()
    assert o.mode == capi.MODE_CPU_REFERENCE and o.precision == capi.PRECISION_FP32
    assert all(v == 0 for v in o.reserved)


def test_create_rejects_bad_geometry_without_device():
    L = capi.lib()
    h = C.c_void_p()
    g = capi.Geometry(450, 1000, 0, 200, 5, 10, 42).c()
    rc = L.jpet_strip_create(C.byref(g), None, C.byref(h))
    assert rc == capi.JPET_ERR_ARGUMENT
    assert b"n_y_pixels" in L.jpet_strip_last_error(None)
    g = capi.Geometry(450, 1000, 180, 200, -5, 10, 42).c()
    assert L.jpet_strip_create(C.byref(g), None, C.byref(h)) == capi.JPET_ERR_ARGUMENT
    # the reference's pixel indices are short (scanner.h:142-144): at most 32767
    g = capi.Geometry(450, 1000, 10, 32768, 5, 10, 42).c()
    assert L.jpet_strip_create(C.byref(g), None, C.byref(h)) == capi.JPET_ERR_ARGUMENT
    assert b"32767" in L.jpet_strip_last_error(None)
    assert L.jpet_strip_create(C.byref(g), None, None) == capi.JPET_ERR_ARGUMENT
    assert L.jpet_strip_destroy(None) == 0


def test_null_handle_calls_are_argument_errors():
    L = capi.lib()
    for fn, args in [(L.jpet_strip_iterate, (None, 1)), (L.jpet_strip_get_image, (None, None)),
                     (L.jpet_strip_set_events, (None, None, 0)),
                     (L.jpet_strip_synchronize, (None,))]:
        assert fn(*args) == capi.JPET_ERR_ARGUMENT


def test_no_device_is_a_status_not_an_abort():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = capi.lib()
    h = C.c_void_p()
    g = capi.Geometry(450, 1000, 180, 200, 5, 10, 42).c()
    rc = L.jpet_strip_create(C.byref(g), None, C.byref(h))
    assert rc == capi.JPET_ERR_CUDA
    assert not h.value


def test_generator_argument_checks_need_no_device():
    import ctypes as C

    L = capi.lib()
    g = capi.Geom(450.0, 1000.0, 1, 1, 1.0, 1.0, 10.0, 42.0)
    regs = capi._regions([phantom_ellipse()])
    n = C.c_int64(0)
    # NULL output with n > 0, zero regions, negative n, bad kind
    assert L.jpet_strip_generate(C.byref(g), regs, 1, 10, 1, 1, None, 10, C.byref(n), None, None) \
        == capi.JPET_ERR_ARGUMENT
    assert L.jpet_strip_generate(C.byref(g), regs, 0, 0, 1, 1, None, 0, C.byref(n), None, None) \
        == capi.JPET_ERR_ARGUMENT
    assert L.jpet_strip_generate(C.byref(g), regs, 1, -1, 1, 1, None, 0, C.byref(n), None, None) \
        == capi.JPET_ERR_ARGUMENT
    bad = capi._regions([(7, 0.0, 0.0, 1.0, 1.0, 0.0, 1.0)])
    assert L.jpet_strip_generate(C.byref(g), bad, 1, 0, 1, 1, None, 0, C.byref(n), None, None) \
        == capi.JPET_ERR_ARGUMENT
    assert b"region" in L.jpet_strip_last_error(None)
    # zero events: validated and returns without touching a device
    assert L.jpet_strip_generate(C.byref(g), regs, 1, 0, 1, 1, None, 0, C.byref(n), None, None) \
        == capi.JPET_OK


def phantom_ellipse():
    from jpet_strip import phantom

    return phantom.Ellipse(0.0, 0.0, 100.0, 80.0, 10.0, 1.0)


def test_binding_fails_loudly_without_the_library(monkeypatch, tmp_path):
    """The product has no CPU fallback: with libjpet_strip.so missing the
    binding raises instead of computing anything."""
    monkeypatch.setattr(capi, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(capi, "_lib", None)
    with pytest.raises(ImportError):
        capi.lib()
    with pytest.raises(ImportError):
        capi.StripReconstruction(capi.Geometry(450, 1000, 90, 100, 10, 10, 42))


def test_batch_create_rejects_unsupported_options_without_device():
    import ctypes as C

    L = capi.lib()
    g = capi.Geometry(450, 1000, 90, 100, 10, 10, 42).c()
    arr = (capi.Geom * 1)(g)
    b = C.c_void_p()
    o = capi.make_opts(precision=capi.PRECISION_FIXED)
    assert L.jpet_strip_batch_create(1, arr, C.byref(o), C.byref(b)) == capi.JPET_ERR_UNSUPPORTED
    assert L.jpet_strip_batch_create(0, arr, None, C.byref(b)) == capi.JPET_ERR_ARGUMENT
    assert L.jpet_strip_batch_destroy(None) == capi.JPET_OK


def test_tan_map_and_kernel_map_argument_checks_need_no_device():
    L = capi.lib()
    g = capi.Geom(450.0, 1000.0, 18, 20, 5.0, 5.0, 10.0, 42.0)
    regs = capi._regions([phantom_ellipse()])
    n = C.c_int64(0)
    out = (C.c_float * 30)()
    # a map without planes, planes without a map
    for bins, ptr in [(0, C.cast(out, C.c_void_p)), (4, None), (-1, None)]:
        im = capi.GenImages(None, None, None, 0.0, 0.0, bins, 0, ptr)
        assert L.jpet_strip_generate(C.byref(g), regs, 1, 10, 1, 1, C.cast(out, C.c_void_p), 10,
                                     C.byref(n), C.byref(im), None) == capi.JPET_ERR_ARGUMENT
        assert b"tan_map" in L.jpet_strip_last_error(None)
    buf = (C.c_float * (18 * 20 * 2))()
    assert L.jpet_strip_tan_kernel_map(C.byref(g), 0, 0.0, 0.0, 0.0, 0.0, 0, buf, 0) \
        == capi.JPET_ERR_ARGUMENT
    assert L.jpet_strip_tan_kernel_map(C.byref(g), 2, 0.0, 0.0, 0.0, 0.0, 0, None, 0) \
        == capi.JPET_ERR_ARGUMENT
    bad = capi.Geom(450.0, 1000.0, 18, 20, 5.0, 5.0, 0.0, 42.0)
    assert L.jpet_strip_tan_kernel_map(C.byref(bad), 2, 0.0, 0.0, 0.0, 0.0, 0, buf, 0) \
        == capi.JPET_ERR_ARGUMENT


def test_oracle_tan_maps_are_consistent():
    """The oracle's tangent map refines its naive image (planes sum to at most
    the image), and its kernel map is finite, non-negative and peaks near the
    kernel point."""
    import numpy as np

    import oracle as O

    og = O.Geometry(450.0, 1000.0, 90, 100, 10.0, 10.0, 42.0)
    ev = np.load(os.path.join(ROOT, "tests", "golden", "c1_events.npy"))[:20000]
    naive, tan = O.naive_bins(og, ev, tan_bins=8)
    assert naive.sum() > 0 and (tan.sum(0) <= naive).all() and tan.sum() > 0.9 * naive.sum()
    m = O.tan_kernel_map(og, 8, (20.0, -10.0))
    assert np.isfinite(m).all() and (m >= 0).all()
    _, row, col = np.unravel_index(np.argmax(m), m.shape)
    # grid row 0 is the lowest y: pixel centre -450 + 10 (row + 0.5)
    assert abs(-500 + 10 * (col + 0.5) - 20.0) <= 10 and abs(-450 + 10 * (row + 0.5) + 10.0) <= 10


def test_header_compiles_as_c99_and_cxx11(tmp_path):
    """include/jpet_strip.h is a plain C header (what cgo, JNI or a C caller
    includes) and also valid C++11 (the reference's language level)."""
    import shutil
    import subprocess

    src = tmp_path / "use.c"
    src.write_text('#include <string.h>\n#include "jpet_strip.h"\n'
                   "int main(void) {\n"
                   "  jpet_strip_opts o; jpet_strip_default_opts(&o);\n"
                   "  jpet_strip_gen_images im; memset(&im, 0, sizeof im);\n"
                   "  return o.mode + im.tan_bins;\n}\n")
    inc = os.path.join(ROOT, "include")
    for cc, std, lang in (("gcc", "-std=c99", "c"), ("g++", "-std=c++11", "c++")):
        if not shutil.which(cc):
            pytest.skip(f"{cc} not available")
        r = subprocess.run([cc, std, "-Wall", "-Wextra", "-Werror", "-x", lang, "-I", inc, "-c",
                            str(src), "-o", str(tmp_path / f"use_{lang}.o")],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
