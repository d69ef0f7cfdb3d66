"""ctypes loader for the CPU restatement (liboracle_strip.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` -- never by the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle_strip.so")
# the same restatement built with FP contraction allowed: the CPU baseline's timing build
RELEASE_LIB_PATH = os.path.join(HERE, "liboracle_strip_release.so")
REF_DIR = os.path.join(HERE, "_ref")


class OrcGeom(C.Structure):
    _fields_ = [
        ("radius", C.c_double),
        ("scintillator_length", C.c_double),
        ("n_y_pixels", C.c_int32),
        ("n_z_pixels", C.c_int32),
        ("pixel_height", C.c_double),
        ("pixel_width", C.c_double),
        ("sigma_z", C.c_double),
        ("sigma_dl", C.c_double),
    ]


class OrcStats(C.Structure):
    _fields_ = [
        ("n_events", C.c_int64),
        ("n_pixels", C.c_int64),
        ("n_kernel_calls", C.c_int64),
        ("n_contributing", C.c_int64),
    ]


@dataclass
class Geometry:
    radius: float
    length: float
    n_y: int
    n_z: int
    pixel: float
    sigma_z: float
    sigma_dl: float
    pixel_height: float | None = None  # rows' height when it differs from the width

    def c(self) -> OrcGeom:
        ph = self.pixel if self.pixel_height is None else self.pixel_height
        return OrcGeom(self.radius, self.length, self.n_y, self.n_z, ph, self.pixel,
                       self.sigma_z, self.sigma_dl)


def build() -> str:
    """Compiles the restatement with make (seconds); returns the library path."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_libs = {}


def lib(release: bool = False):
    """The parity oracle, or with release=True its timing build (FMA contraction
    allowed, so results differ from the strict one by rounding)."""
    path = RELEASE_LIB_PATH if release else LIB_PATH
    if path not in _libs:
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        gp = C.POINTER(OrcGeom)
        fp = C.POINTER(C.c_float)
        L.orc_mlem_f.argtypes = [gp, f32p, C.c_int64, f32p, C.c_int, C.c_int, C.POINTER(OrcStats)]
        L.orc_mlem_d.argtypes = [gp, f32p, C.c_int64, f64p, C.c_int, C.c_int, C.POINTER(OrcStats)]
        L.orc_mlem_gpuref.argtypes = [gp, f32p, C.c_int64, f32p, C.c_int, C.c_int, C.c_void_p]
        L.orc_sensitivity_map_f.argtypes = [gp, C.c_int, f32p]
        L.orc_naive_bins_f.argtypes = [gp, f32p, C.c_int64, C.c_double, C.c_double, C.c_int32,
                                       C.c_void_p, C.c_void_p]
        L.orc_tan_kernel_map_f.argtypes = [gp, C.c_int32, C.c_double, C.c_double, C.c_double,
                                           C.c_double, C.c_int32, f32p]
        L.orc_nll_grad.argtypes = [gp, C.c_double, C.c_double, f32p, C.c_int64, f32p,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                   C.POINTER(C.c_int64)]
        L.orc_nll_grad.restype = C.c_double
        L.orc_gaussian_kernel_f.argtypes = [C.c_float] * 8
        L.orc_gaussian_kernel_f.restype = C.c_float
        L.orc_gaussian_kernel_d.argtypes = [C.c_double] * 8
        L.orc_gaussian_kernel_d.restype = C.c_double
        L.orc_analytic_kernel_d.argtypes = [C.c_double] * 8
        L.orc_analytic_kernel_d.restype = C.c_double
        L.orc_analytic_kernel_f.argtypes = [C.c_float] * 8
        L.orc_analytic_kernel_f.restype = C.c_float
        L.orc_bb_y_dd.argtypes = [C.c_double] * 3
        L.orc_bb_y_dd.restype = C.c_double
        L.orc_bb_z_dd.argtypes = [C.c_double] * 3
        L.orc_bb_z_dd.restype = C.c_double
        L.orc_sensitivity_d.argtypes = [gp, C.c_double, C.c_double]
        L.orc_sensitivity_d.restype = C.c_double
        L.orc_pixel_at_d.argtypes = [gp, C.c_double, C.c_double, C.POINTER(C.c_int32),
                                     C.POINTER(C.c_int32)]
        L.orc_pixel_center_d.argtypes = [gp, C.c_int32, C.c_int32, C.POINTER(C.c_double),
                                         C.POINTER(C.c_double)]
        L.orc_response_tan_y_z_f.argtypes = [C.c_float] * 4 + [fp] * 3
        L.orc_ellipse_bb_f.argtypes = [C.c_float] * 3 + [fp] * 6
        L.orc_event_box_f.argtypes = [gp, C.c_float, C.c_float, C.c_float] + [C.POINTER(C.c_int32)] * 4
        L.orc_event_box_f.restype = C.c_int32
        L.orc_to_projection_space_tan_d.argtypes = [C.c_double] * 4 + [C.POINTER(C.c_double)] * 3
        _libs[path] = L
    return _libs[path]


def _events(ev) -> np.ndarray:
    ev = np.ascontiguousarray(ev, dtype=np.float32).reshape(-1, 3)
    return ev


def mlem_f(geom: Geometry, events, n_iterations: int, rho=None, threads: int = 1,
           release: bool = False):
    """Reference CPU float path: returns (rho float32[n_y, n_z], stats dict).
    release=True runs the timing build (FMA contraction allowed)."""
    ev = _events(events)
    r = (np.ones(geom.n_y * geom.n_z, np.float32) if rho is None
         else np.ascontiguousarray(rho, np.float32).reshape(-1).copy())
    st = OrcStats()
    g = geom.c()
    rc = lib(release).orc_mlem_f(C.byref(g), ev.reshape(-1), len(ev), r, n_iterations, threads,
                                 C.byref(st))
    if rc != 0:
        raise RuntimeError("orc_mlem_f failed")
    return r.reshape(geom.n_y, geom.n_z), dict(
        n_events=st.n_events, n_pixels=st.n_pixels, n_kernel_calls=st.n_kernel_calls,
        n_contributing=st.n_contributing)


def mlem_d(geom: Geometry, events, n_iterations: int, rho=None, threads: int = 0):
    """FP64 instantiation of the same algorithm; returns float64[n_y, n_z]."""
    ev = _events(events)
    r = (np.ones(geom.n_y * geom.n_z, np.float64) if rho is None
         else np.ascontiguousarray(rho, np.float64).reshape(-1).copy())
    st = OrcStats()
    g = geom.c()
    rc = lib().orc_mlem_d(C.byref(g), ev.reshape(-1), len(ev), r, n_iterations, threads,
                          C.byref(st))
    if rc != 0:
        raise RuntimeError("orc_mlem_d failed")
    return r.reshape(geom.n_y, geom.n_z)


def mlem_gpuref(geom: Geometry, events, n_iterations: int, rho=None, threads: int = 0):
    """Reference GPU-kernel semantics (analytic kernel, sensitivity-weighted denominator)."""
    ev = _events(events)
    r = (np.ones(geom.n_y * geom.n_z, np.float32) if rho is None
         else np.ascontiguousarray(rho, np.float32).reshape(-1).copy())
    g = geom.c()
    rc = lib().orc_mlem_gpuref(C.byref(g), ev.reshape(-1), len(ev), r, n_iterations,
                               threads, None)
    if rc != 0:
        raise RuntimeError("orc_mlem_gpuref failed")
    return r.reshape(geom.n_y, geom.n_z)


def sensitivity_map(geom: Geometry, kind: int = 0) -> np.ndarray:
    out = np.empty(geom.n_y * geom.n_z, np.float32)
    g = geom.c()
    lib().orc_sensitivity_map_f(C.byref(g), kind, out)
    return out.reshape(geom.n_y, geom.n_z)


def nll_grad(geom: Geometry, events, rho, support_sigma=None, s=None, threads: int = 0,
             want_grad_rho: bool = True):
    """FP64 NLL, dL/drho (float64 image) and dL/dsigma (float64[2])."""
    ev = _events(events)
    r = np.ascontiguousarray(rho, np.float32).reshape(-1)
    g = geom.c()
    ssz, ssdl = support_sigma if support_sigma is not None else (geom.sigma_z, geom.sigma_dl)
    gr = np.zeros(r.size, np.float64) if want_grad_rho else None
    gs = np.zeros(2, np.float64)
    s_arr = None if s is None else np.ascontiguousarray(s, np.float32).reshape(-1)
    skipped = C.c_int64(0)
    loss = lib().orc_nll_grad(
        C.byref(g), ssz, ssdl, ev.reshape(-1), len(ev), r,
        None if s_arr is None else s_arr.ctypes.data,
        None if gr is None else gr.ctypes.data, gs.ctypes.data, threads, C.byref(skipped))
    return loss, (None if gr is None else gr.reshape(geom.n_y, geom.n_z)), gs, skipped.value


def gaussian_kernel_f(sz, sdl, y, tan, sec, R, dz, dy) -> float:
    return lib().orc_gaussian_kernel_f(sz, sdl, y, tan, sec, R, dz, dy)


def gaussian_kernel_d(sz, sdl, y, tan, sec, R, dz, dy) -> float:
    return lib().orc_gaussian_kernel_d(sz, sdl, y, tan, sec, R, dz, dy)


def analytic_kernel_d(sz, sdl, y, tan, sec, R, dz, dy) -> float:
    return lib().orc_analytic_kernel_d(sz, sdl, y, tan, sec, R, dz, dy)


def naive_bins(geom: Geometry, events, origin=(0.0, 0.0), tan_bins: int = 0):
    """The phantom tool's naive image int32[n_y, n_z] and, with tan_bins > 0,
    its tangent-binned map int32[tan_bins, n_y, n_z] of smeared responses
    (phantom_cmd.cpp:339-352; float, reference order)."""
    ev = _events(events)
    g = geom.c()
    naive = np.zeros((geom.n_y, geom.n_z), np.int32)
    tan = np.zeros((max(tan_bins, 1), geom.n_y, geom.n_z), np.int32)
    lib().orc_naive_bins_f(C.byref(g), ev, len(ev),
                           float(origin[0]), float(origin[1]), int(tan_bins),
                           naive.ctypes.data, tan.ctypes.data if tan_bins > 0 else None)
    return naive, (tan if tan_bins > 0 else None)


def tan_kernel_map(geom: Geometry, tan_bins: int, kernel_point=(0.0, 0.0), origin=(0.0, 0.0),
                   divide_by_sensitivity: bool = False) -> np.ndarray:
    """The phantom tool's --tan-bins kernel map float32[tan_bins, n_y, n_z]
    (phantom_cmd.cpp:396-430; float, reference order)."""
    g = geom.c()
    out = np.zeros((tan_bins, geom.n_y, geom.n_z), np.float32)
    lib().orc_tan_kernel_map_f(C.byref(g), int(tan_bins), float(kernel_point[0]),
                               float(kernel_point[1]), float(origin[0]), float(origin[1]),
                               int(bool(divide_by_sensitivity)), out)
    return out


def event_box(geom: Geometry, z_u, z_d, dl):
    vals = [C.c_int32() for _ in range(4)]
    g = geom.c()
    cnt = lib().orc_event_box_f(C.byref(g), z_u, z_d, dl, *[C.byref(v) for v in vals])
    return tuple(v.value for v in vals), cnt


def ref_binary(name: str) -> str | None:
    """Path of a reference tool built by build_ref.sh, if present on this host."""
    p = os.path.join(REF_DIR, name)
    return p if os.path.exists(p) and os.access(p, os.X_OK) else None


# ---- 3D hybrid reconstruction (src/3d/hybrid/reconstruction.h) -----------------

class OrcHybrid(C.Structure):
    _fields_ = [
        ("n_detectors", C.c_int32),
        ("n_pixel_infos", C.c_int64),
        ("segments", C.c_void_p),
        ("lor_widths", C.c_void_p),
        ("pixels", C.c_void_p),
        ("positions", C.c_void_p),
        ("info_begin", C.c_void_p),
        ("info_end", C.c_void_p),
        ("n_columns", C.c_int32),
        ("n_rows", C.c_int32),
        ("n_planes", C.c_int32),
        ("pixel_size", C.c_float),
        ("lower_left_x", C.c_float),
        ("lower_left_y", C.c_float),
        ("z_left", C.c_float),
        ("sigma_z", C.c_float),
        ("sigma_dl", C.c_float),
        ("length", C.c_float),
        ("n_planes_half", C.c_int32),
        ("sens_depth", C.c_int32),
    ]


def _hyb_lib(release: bool = False):
    L = lib(release)
    if not hasattr(L, "_hyb_ready"):
        hp = C.POINTER(OrcHybrid)
        vp = C.c_void_p
        L.orc_hybrid_calculate_weight.argtypes = [hp, vp]
        L.orc_hybrid_calculate_sensitivity.argtypes = [hp, vp, vp]
        L.orc_hybrid_normalize.argtypes = [hp, vp, vp]
        L.orc_hybrid_translate_all.argtypes = [hp, vp, C.c_int64, vp, vp]
        L.orc_hybrid_translate_all.restype = C.c_int64
        L.orc_hybrid_mlem.argtypes = [hp, vp, vp, vp, C.c_int64, vp, C.c_int, C.c_int, vp]
        L.orc_hybrid_mlem.restype = C.c_int
        L._hyb_ready = True
    return L


def _ptr(a) -> int:
    return a.ctypes.data if a.size else 0


def hybrid_sens_depth(g, sens_given_3d: bool = False) -> int:
    """Depth of the reconstruction's sensitivity image (reconstruction.h:80-85):
    n_planes_half for a multi-plane geometry, n_planes / 2 with an external 3D
    sensitivity, else 1."""
    h = getattr(g, "n_planes_half", 1)
    return h if h > 1 else (g.n_planes // 2 if sens_given_3d else 1)


def hybrid_struct(g, sens_depth: int | None = None) -> tuple[OrcHybrid, list]:
    """orc_hybrid view of a HybridGeometry (arrays kept alive by the returned list)."""
    keep = [np.ascontiguousarray(a) for a in (g.segments, g.widths, g.pixels, g.positions,
                                               g.info_begin, g.info_end)]
    h = getattr(g, "n_planes_half", 1)
    d = hybrid_sens_depth(g) if sens_depth is None else sens_depth
    s = OrcHybrid(g.n_detectors, g.n_pixel_infos, *[_ptr(a) for a in keep], g.n_columns,
                  g.n_rows, g.n_planes, g.pixel_size, g.lower_left_x, g.lower_left_y, g.z_left,
                  g.sigma_z, g.sigma_dl, g.length, h, d)
    return s, keep


def hybrid_setup(g, weights_given: bool = False, sens_to_one: bool = False,
                 sens_given=None):
    """calculate_weight (unless given), calculate_sensitivity, ones, or the given
    3D sensitivity (float32[depth * n_rows * n_columns], the --sensitivity
    image, depth n_planes / 2 or n_planes_half), then normalize_geometry_weights:
    (normalized weights [n_planes_half * n_infos], raw sensitivity
    [depth * n_rows * n_columns])."""
    L = _hyb_lib()
    depth = hybrid_sens_depth(g, sens_given is not None)
    s, keep = hybrid_struct(g, depth)
    w = np.array(g.weights, np.float32, copy=True).reshape(-1)
    if not weights_given:
        L.orc_hybrid_calculate_weight(C.byref(s), _ptr(w))
    n_sens = depth * g.n_columns * g.n_rows
    if sens_given is not None:
        sens = np.array(sens_given, np.float32, copy=True).reshape(-1)
        assert sens.size == n_sens
    else:
        sens = np.ones(n_sens, np.float32)
        if not sens_to_one:
            L.orc_hybrid_calculate_sensitivity(C.byref(s), _ptr(w), _ptr(sens))
    L.orc_hybrid_normalize(C.byref(s), _ptr(w), _ptr(sens))
    return w, sens


def hybrid_translate(g, weights, responses):
    """Frame events of the kept responses (translate_to_frame + bounding-box filter)."""
    L = _hyb_lib()
    s, keep = hybrid_struct(g)
    r = np.ascontiguousarray(responses)
    out = np.zeros(r.shape[0], dtype=_frame_dtype())
    w = np.ascontiguousarray(weights, np.float32)
    n = L.orc_hybrid_translate_all(C.byref(s), _ptr(r), r.shape[0], _ptr(w), _ptr(out))
    return out[:n].copy()


def _frame_dtype():
    return np.dtype({
        "names": ["first", "second", "up", "right", "tan", "sec", "info_begin", "info_end",
                  "plane_begin", "plane_end"],
        "formats": ["<i2", "<i2", "<f4", "<f4", "<f4", "<f4", "<u8", "<u8", "<i2", "<i2"],
        "offsets": [0, 2, 4, 8, 12, 16, 24, 32, 40, 42],
        "itemsize": 48})


def hybrid_mlem(g, weights, sens, events, n_iterations: int, rho=None, threads: int = 1,
                release: bool = False):
    """n_iterations of Reconstruction::operator(); returns (rho float32[n_voxels],
    counters int64[4]: used_events, used_pixels, used_voxels, positive denominators).
    release=True runs the timing build (FMA contraction allowed)."""
    L = _hyb_lib(release)
    sn = np.ascontiguousarray(sens, np.float32).reshape(-1)
    s, keep = hybrid_struct(g, sn.size // (g.n_columns * g.n_rows))
    rho = (np.ones(g.n_voxels, np.float32) if rho is None
           else np.array(rho, np.float32, copy=True).reshape(-1))
    ev = np.ascontiguousarray(events)
    w = np.ascontiguousarray(weights, np.float32)
    cnt = np.zeros(4, np.int64)
    rc = L.orc_hybrid_mlem(C.byref(s), _ptr(w), _ptr(sn), _ptr(ev), ev.shape[0], _ptr(rho),
                           n_iterations, threads, _ptr(cnt))
    if rc != 0:
        raise MemoryError("orc_hybrid_mlem")
    return rho, cnt
