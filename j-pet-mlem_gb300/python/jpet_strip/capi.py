"""ctypes binding of the C ABI in include/jpet_strip.h (libjpet_strip.so).

This is the Python-side mirror of the reference's strip reconstruction API: a
``StripReconstruction`` object owns one library handle and offers the members
of ``PET2D::Strip::Reconstruction`` (src/2d/strip/reconstruction.h:57-213):
``rho``, ``sensitivity``, ``responses`` loading and ``__call__(n_iterations)``.

There is no fallback: if the compiled library is missing this module raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

_PKG_ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
LIB_PATH = os.environ.get("JPET_STRIP_LIB", os.path.join(_PKG_ROOT, "lib", "libjpet_strip.so"))

JPET_OK = 0
JPET_ERR_ARGUMENT = -1
JPET_ERR_CUDA = -2
JPET_ERR_MEMORY = -3
JPET_ERR_STATE = -4
JPET_ERR_TIMEOUT = -5
JPET_ERR_UNSUPPORTED = -6

MODE_CPU_REFERENCE = 0
MODE_GPU_REFERENCE = 1
PRECISION_FP32 = 0
PRECISION_COMPENSATED = 1
PRECISION_FP64_DEN = 2
PRECISION_FIXED = 3
VARIANT_FAST = 0
VARIANT_EXACT = 1
VARIANT_WARP = 2
VARIANT_ROWS = 3
RASTER_AUTO = 0
RASTER_SHAPES = {"8x1x1": 1, "8x1x2": 2, "4x1x2": 3, "4x1x3": 4, "4x1x4": 5, "4x2x4": 6,
                 "2x1x6": 7}

# every symbol include/jpet_strip.h declares
EXPORTED = [
    "jpet_strip_abi_version", "jpet_strip_default_opts", "jpet_strip_create",
    "jpet_strip_destroy", "jpet_strip_last_error", "jpet_strip_set_stream",
    "jpet_strip_set_events", "jpet_strip_set_events_soa", "jpet_strip_set_events_device",
    "jpet_strip_set_image", "jpet_strip_set_image_device", "jpet_strip_iterate",
    "jpet_strip_get_image", "jpet_strip_image_device", "jpet_strip_get_sensitivity",
    "jpet_strip_get_counters", "jpet_strip_synchronize", "jpet_strip_run",
    "jpet_strip_nll_grad", "jpet_strip_iterate_noalloc", "jpet_strip_generate",
    "jpet_strip_generate_host", "jpet_strip_batch_create", "jpet_strip_batch_destroy",
    "jpet_strip_batch_last_error", "jpet_strip_batch_size", "jpet_strip_batch_instance",
    "jpet_strip_batch_set_events", "jpet_strip_batch_tune", "jpet_strip_batch_plan_of",
    "jpet_strip_batch_iterate", "jpet_strip_batch_launches_per_iteration",
    "jpet_strip_reference_fp64", "jpet_strip_tan_kernel_map",
]


class StripError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"jpet_strip error {code}: {message}")
        self.code = code


class GenImages(C.Structure):
    _fields_ = [
        ("emitted", C.c_void_p),
        ("detected", C.c_void_p),
        ("naive", C.c_void_p),
        ("origin_x", C.c_double),
        ("origin_y", C.c_double),
        ("tan_bins", C.c_int32),
        ("reserved", C.c_int32),
        ("tan_map", C.c_void_p),
        ("exact_responses", C.c_void_p),
        ("events", C.c_void_p),
    ]


class Geom(C.Structure):
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


class Opts(C.Structure):
    _fields_ = [
        ("device", C.c_int32),
        ("mode", C.c_int32),
        ("precision", C.c_int32),
        ("tile_w", C.c_int32),
        ("tile_h", C.c_int32),
        ("block_threads", C.c_int32),
        ("variant", C.c_int32),
        ("raster_shape", C.c_int32),
        ("reserved", C.c_int32 * 8),
    ]


class Region(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("reserved", C.c_int32),
        ("x", C.c_double),
        ("y", C.c_double),
        ("a", C.c_double),
        ("b", C.c_double),
        ("angle_deg", C.c_double),
        ("intensity", C.c_double),
    ]


REGION_ELLIPSE, REGION_RECTANGLE, REGION_POINT = 0, 1, 2
GEN_DETECTED, GEN_ADDITIVE = 1, 2


class BatchPlan(C.Structure):
    _fields_ = [
        ("raster_shape", C.c_int32),
        ("block_threads", C.c_int32),
        ("tuned_ms_per_iteration", C.c_double),
        ("tuned_events", C.c_int64),
        ("candidates", C.c_int32),
        ("tile", C.c_int32),
    ]


class Counters(C.Structure):
    _fields_ = [
        ("n_events", C.c_int64),
        ("n_pixels", C.c_int64),
        ("n_kernel_calls", C.c_int64),
        ("n_contributing", C.c_int64),
        ("n_oversize", C.c_int64),
        ("n_tiles", C.c_int64),
        ("n_chunks", C.c_int64),
        ("iterations_done", C.c_int64),
        ("n_exact_path", C.c_int64),
    ]


OUTPUT_FN = C.CFUNCTYPE(None, C.c_int, C.POINTER(C.c_float), C.c_int, C.c_int, C.c_void_p)
PROGRESS_FN = C.CFUNCTYPE(None, C.c_int, C.c_int, C.c_void_p)

_lib = None


def lib() -> C.CDLL:
    """Loads libjpet_strip.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libjpet_strip.so not built at {LIB_PATH}; run build()")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.jpet_strip_abi_version.restype = C.c_int
        L.jpet_strip_default_opts.argtypes = [C.POINTER(Opts)]
        L.jpet_strip_default_opts.restype = None
        L.jpet_strip_create.argtypes = [C.POINTER(Geom), C.POINTER(Opts), C.POINTER(vp)]
        L.jpet_strip_destroy.argtypes = [vp]
        L.jpet_strip_last_error.argtypes = [vp]
        L.jpet_strip_last_error.restype = C.c_char_p
        L.jpet_strip_set_stream.argtypes = [vp, vp]
        L.jpet_strip_set_events.argtypes = [vp, vp, C.c_int64]
        L.jpet_strip_set_events_soa.argtypes = [vp, vp, vp, vp, C.c_int64]
        L.jpet_strip_set_events_device.argtypes = [vp, vp, vp, vp, C.c_int64]
        L.jpet_strip_set_image.argtypes = [vp, vp]
        L.jpet_strip_set_image_device.argtypes = [vp, vp]
        L.jpet_strip_iterate.argtypes = [vp, C.c_int]
        L.jpet_strip_get_image.argtypes = [vp, vp]
        L.jpet_strip_image_device.argtypes = [vp, C.POINTER(vp)]
        L.jpet_strip_get_sensitivity.argtypes = [vp, C.c_int, vp]
        L.jpet_strip_get_counters.argtypes = [vp, C.POINTER(Counters)]
        L.jpet_strip_synchronize.argtypes = [vp]
        L.jpet_strip_nll_grad.argtypes = [vp, C.c_double, C.c_double, vp, vp,
                                          C.POINTER(C.c_double), vp, C.POINTER(C.c_double),
                                          C.POINTER(C.c_int64)]
        L.jpet_strip_iterate_noalloc.argtypes = [C.POINTER(Geom), vp, C.c_int64, vp, vp, vp]
        L.jpet_strip_generate.argtypes = [C.POINTER(Geom), C.POINTER(Region), C.c_int32,
                                          C.c_int64, C.c_uint64, C.c_int32, vp, C.c_int64,
                                          C.POINTER(C.c_int64), vp, vp]
        L.jpet_strip_generate_host.argtypes = [C.POINTER(Geom), C.POINTER(Region), C.c_int32,
                                               C.c_int64, C.c_uint64, C.c_int32, vp, C.c_int64,
                                               C.POINTER(C.c_int64), vp, C.c_int32]
        L.jpet_strip_tan_kernel_map.argtypes = [C.POINTER(Geom), C.c_int32, C.c_double,
                                                C.c_double, C.c_double, C.c_double, C.c_int32,
                                                vp, C.c_int32]
        L.jpet_strip_batch_create.argtypes = [C.c_int32, C.POINTER(Geom), C.POINTER(Opts),
                                              C.POINTER(vp)]
        L.jpet_strip_batch_destroy.argtypes = [vp]
        L.jpet_strip_batch_last_error.argtypes = [vp]
        L.jpet_strip_batch_last_error.restype = C.c_char_p
        L.jpet_strip_batch_size.argtypes = [vp]
        L.jpet_strip_batch_instance.argtypes = [vp, C.c_int32, C.POINTER(vp)]
        L.jpet_strip_batch_set_events.argtypes = [vp, C.c_int32, vp, C.c_int64, C.c_int32]
        L.jpet_strip_batch_tune.argtypes = [vp, C.c_int64]
        L.jpet_strip_batch_plan_of.argtypes = [vp, C.c_int32, C.POINTER(BatchPlan)]
        L.jpet_strip_batch_iterate.argtypes = [vp, C.c_int32]
        L.jpet_strip_batch_launches_per_iteration.argtypes = [vp]
        L.jpet_strip_reference_fp64.argtypes = [C.POINTER(Geom), vp, C.c_int64, vp, vp, C.c_int32,
                                                C.POINTER(C.c_int64), C.POINTER(C.c_int64), vp]
        L.jpet_strip_run.argtypes = [C.POINTER(Geom), C.POINTER(Opts), vp, C.c_int64, vp, C.c_int,
                                     C.c_int, OUTPUT_FN, PROGRESS_FN, vp, C.c_char_p, C.c_size_t]
        for name in EXPORTED:
            if name not in ("jpet_strip_last_error", "jpet_strip_default_opts",
                            "jpet_strip_abi_version", "jpet_strip_batch_last_error"):
                getattr(L, name).restype = C.c_int
        _lib = L
    return _lib


@dataclass
class Geometry:
    """Scanner geometry in the reference's option units (mm in its examples)."""

    radius: float
    length: float
    n_y: int
    n_z: int
    pixel: float
    sigma_z: float
    sigma_dl: float
    pixel_height: float | None = None  # rows' height when it differs from the width

    def c(self) -> Geom:
        ph = self.pixel if self.pixel_height is None else self.pixel_height
        return Geom(self.radius, self.length, self.n_y, self.n_z, ph, self.pixel,
                    self.sigma_z, self.sigma_dl)


def make_opts(device=0, mode=MODE_CPU_REFERENCE, precision=PRECISION_FP32, tile_w=0,
              tile_h=0, block_threads=0, variant=VARIANT_FAST, raster_shape=RASTER_AUTO) -> Opts:
    o = Opts()
    lib().jpet_strip_default_opts(C.byref(o))
    o.device, o.mode, o.precision = device, mode, precision
    o.tile_w, o.tile_h, o.block_threads = tile_w, tile_h, block_threads
    o.variant = variant
    o.raster_shape = raster_shape
    return o


def _check(rc: int, h=None):
    if rc != JPET_OK:
        msg = lib().jpet_strip_last_error(h)
        raise StripError(rc, msg.decode() if msg else "?")


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _regions(regions) -> "C.Array":
    """Regions as jpet_strip_region: phantom.Ellipse objects or tuples
    (kind, x, y, a, b, angle_deg, intensity)."""
    arr = (Region * len(regions))()
    for i, r in enumerate(regions):
        if hasattr(r, "angle_deg"):
            arr[i] = Region(REGION_ELLIPSE, 0, r.z, r.y, r.a, r.b, r.angle_deg, r.intensity)
        else:
            kind, x, y, a, b, ang, inten = r
            arr[i] = Region(int(kind), 0, x, y, a, b, ang, inten)
    return arr


def generate_device(regions, n: int, radius: float, length: float, sigma_z: float,
                    sigma_dl: float, seed: int, detected: bool = True, additive: bool = False,
                    device: int = 0):
    """Events of the phantom regions on the GPU: a torch float32[k, 3] device
    tensor of (z_u, z_d, dl), k = n with ``detected`` (n detected events), else
    the detected among n emissions."""
    import torch

    g = Geom(radius, length, 1, 1, 1.0, 1.0, sigma_z, sigma_dl)
    regs = _regions(regions)
    out = torch.empty((max(n, 1), 3), dtype=torch.float32, device=f"cuda:{device}")
    written = C.c_int64(0)
    flags = (GEN_DETECTED if detected else 0) | (GEN_ADDITIVE if additive else 0)
    with torch.cuda.device(device):
        stream = torch.cuda.current_stream().cuda_stream
        _check(lib().jpet_strip_generate(C.byref(g), regs, len(regions), n, seed, flags,
                                         out.data_ptr(), n, C.byref(written), None, stream))
    return out[: written.value]


def generate(regions, n: int, radius: float, length: float, sigma_z: float, sigma_dl: float,
             seed: int, detected: bool = True, additive: bool = False, device: int = 0) -> np.ndarray:
    """As generate_device, copied to a host float32[k, 3] array."""
    return generate_device(regions, n, radius, length, sigma_z, sigma_dl, seed, detected,
                           additive, device).cpu().numpy()


def generate_with_images(regions, n: int, geom: "Geometry", seed: int, detected: bool = True,
                         additive: bool = False, origin=(0.0, 0.0), tan_bins: int = 0,
                         full: bool = False, device: int = 0):
    """The phantom tool's outputs through jpet_strip_generate_host: the events
    (float32[k, 3]) and the int32 count images on geom's grid (emitted,
    detected, naive: [n_y, n_z], row 0 the lowest y; tan_map:
    [tan_bins, n_y, n_z] when tan_bins > 0); with ``full`` also the exact
    responses (float32[k, 3]) and emission events (float32[k, 4]: x, y, sin
    phi, cos phi) of the returned events."""
    g = geom.c()
    regs = _regions(regions)
    shape = (geom.n_y, geom.n_z)
    imgs = {k: np.zeros(shape, np.int32) for k in ("emitted", "detected", "naive")}
    if tan_bins > 0:
        imgs["tan_map"] = np.zeros((tan_bins,) + shape, np.int32)
    out = np.zeros((max(n, 1), 3), np.float32)
    if full:
        imgs["exact"] = np.zeros((max(n, 1), 3), np.float32)
        imgs["events"] = np.zeros((max(n, 1), 4), np.float32)
    im = GenImages(_ptr(imgs["emitted"]), _ptr(imgs["detected"]), _ptr(imgs["naive"]),
                   float(origin[0]), float(origin[1]), int(tan_bins), 0,
                   _ptr(imgs["tan_map"]) if tan_bins > 0 else None,
                   _ptr(imgs["exact"]) if full else None,
                   _ptr(imgs["events"]) if full else None)
    written = C.c_int64(0)
    flags = (GEN_DETECTED if detected else 0) | (GEN_ADDITIVE if additive else 0)
    _check(lib().jpet_strip_generate_host(C.byref(g), regs, len(regions), n, seed, flags,
                                          _ptr(out), n, C.byref(written), C.byref(im), device))
    if full:
        imgs["exact"] = imgs["exact"][: written.value]
        imgs["events"] = imgs["events"][: written.value]
    return out[: written.value], imgs


def tan_kernel_map(geom: "Geometry", tan_bins: int, kernel_point=(0.0, 0.0),
                   origin=(0.0, 0.0), divide_by_sensitivity: bool = False,
                   device: int = 0) -> np.ndarray:
    """The phantom tool's --tan-bins kernel map, float32[tan_bins, n_y, n_z]."""
    g = geom.c()
    out = np.zeros((tan_bins, geom.n_y, geom.n_z), np.float32)
    _check(lib().jpet_strip_tan_kernel_map(C.byref(g), tan_bins, float(kernel_point[0]),
                                           float(kernel_point[1]), float(origin[0]),
                                           float(origin[1]), int(bool(divide_by_sensitivity)),
                                           _ptr(out), device))
    return out


def reference_fp64(geom: Geometry, events, n_iterations: int, rho=None, device: int = 0):
    """The reference iteration at double on the GPU.  events: float32[n, 3]
    (host array or CUDA tensor).  Returns (float64[n_y, n_z] image, counters)."""
    import torch

    dev = f"cuda:{device}"
    ev = events if (hasattr(events, "is_cuda") and events.is_cuda) else \
        torch.from_numpy(np.ascontiguousarray(events, np.float32).reshape(-1, 3))
    ev = ev.to(dev).contiguous()
    r = torch.ones((geom.n_y, geom.n_z), dtype=torch.float64, device=dev) if rho is None else \
        torch.as_tensor(np.asarray(rho, np.float64)).to(dev).contiguous()
    work = torch.empty_like(r)
    calls, contrib = C.c_int64(0), C.c_int64(0)
    g = geom.c()
    with torch.cuda.device(device):
        stream = torch.cuda.current_stream().cuda_stream
        _check(lib().jpet_strip_reference_fp64(C.byref(g), ev.data_ptr(), ev.shape[0],
                                               r.data_ptr(), work.data_ptr(), n_iterations,
                                               C.byref(calls), C.byref(contrib), stream))
    return r.cpu().numpy(), {"n_kernel_calls": calls.value, "n_contributing": contrib.value}


class StripBatch:
    """Many reconstructions iterated together (one graph launch per iterate)."""

    def __init__(self, geoms, **opts):
        arr = (Geom * len(geoms))(*[g.c() for g in geoms])
        o = make_opts(**opts)
        self._b = C.c_void_p()
        _check(lib().jpet_strip_batch_create(len(geoms), arr, C.byref(o), C.byref(self._b)), None)
        self.geoms = list(geoms)
        self._views = {}

    def _ck(self, rc):
        if rc != JPET_OK:
            msg = lib().jpet_strip_batch_last_error(self._b)
            raise StripError(rc, msg.decode() if msg else "?")

    def close(self):
        if self._b:
            lib().jpet_strip_batch_destroy(self._b)
            self._b = C.c_void_p()
            self._views = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self):
        return len(self.geoms)

    def set_events(self, i: int, events):
        """events: float32[n, 3] host array, or a CUDA tensor of that shape."""
        if hasattr(events, "is_cuda") and events.is_cuda:
            ev = events.contiguous()
            self._ck(lib().jpet_strip_batch_set_events(self._b, i, ev.data_ptr(), ev.shape[0], 1))
        else:
            ev = np.ascontiguousarray(events, dtype=np.float32).reshape(-1, 3)
            self._ck(lib().jpet_strip_batch_set_events(self._b, i, _ptr(ev) if len(ev) else None,
                                                       len(ev), 0))

    def tune(self, max_events: int = 0):
        self._ck(lib().jpet_strip_batch_tune(self._b, max_events))

    def plan(self, i: int) -> dict:
        p = BatchPlan()
        self._ck(lib().jpet_strip_batch_plan_of(self._b, i, C.byref(p)))
        return {f: getattr(p, f) for f, _ in BatchPlan._fields_}

    def iterate(self, n: int = 1):
        self._ck(lib().jpet_strip_batch_iterate(self._b, n))

    def launches_per_iteration(self) -> int:
        return lib().jpet_strip_batch_launches_per_iteration(self._b)

    def instance(self, i: int) -> "StripReconstruction":
        """The instance's handle (owned by the batch)."""
        if i not in self._views:
            h = C.c_void_p()
            self._ck(lib().jpet_strip_batch_instance(self._b, i, C.byref(h)))
            v = StripReconstruction.__new__(StripReconstruction)
            v.geom = self.geoms[i]
            v._h = h
            v.n_events = 0
            v._borrowed = True
            self._views[i] = v
        return self._views[i]


class StripReconstruction:
    """One reconstruction on the GPU, mirroring PET2D::Strip::Reconstruction."""

    def __init__(self, geom: Geometry, **opts):
        self.geom = geom
        self._h = C.c_void_p()
        g = geom.c()
        o = make_opts(**opts)
        _check(lib().jpet_strip_create(C.byref(g), C.byref(o), C.byref(self._h)), None)
        self.n_events = 0

    def close(self):
        if self._h and not getattr(self, "_borrowed", False):
            lib().jpet_strip_destroy(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def set_events(self, responses: np.ndarray):
        """responses: float32[n, 3] (z_u, z_d, dl), the reference Response layout."""
        ev = np.ascontiguousarray(responses, dtype=np.float32).reshape(-1, 3)
        _check(lib().jpet_strip_set_events(self._h, _ptr(ev) if len(ev) else None, len(ev)),
               self._h)
        self.n_events = len(ev)

    def set_events_device(self, z_u_ptr: int, z_d_ptr: int, dl_ptr: int, n: int):
        _check(lib().jpet_strip_set_events_device(self._h, z_u_ptr, z_d_ptr, dl_ptr, n), self._h)
        self.n_events = n

    @property
    def rho(self) -> np.ndarray:
        out = np.empty((self.geom.n_y, self.geom.n_z), np.float32)
        _check(lib().jpet_strip_get_image(self._h, _ptr(out)), self._h)
        return out

    @rho.setter
    def rho(self, value: np.ndarray):
        v = np.ascontiguousarray(value, dtype=np.float32).reshape(self.geom.n_y, self.geom.n_z)
        _check(lib().jpet_strip_set_image(self._h, _ptr(v)), self._h)

    def set_image_device(self, ptr: int):
        _check(lib().jpet_strip_set_image_device(self._h, ptr), self._h)

    def image_device_ptr(self) -> int:
        p = C.c_void_p()
        _check(lib().jpet_strip_image_device(self._h, C.byref(p)), self._h)
        return p.value or 0

    def sensitivity(self, kind: int = 0) -> np.ndarray:
        out = np.empty((self.geom.n_y, self.geom.n_z), np.float32)
        _check(lib().jpet_strip_get_sensitivity(self._h, kind, _ptr(out)), self._h)
        return out

    def iterate(self, n: int = 1):
        _check(lib().jpet_strip_iterate(self._h, n), self._h)

    __call__ = iterate

    def synchronize(self):
        _check(lib().jpet_strip_synchronize(self._h), self._h)

    def set_stream(self, stream_ptr: int | None):
        _check(lib().jpet_strip_set_stream(self._h, stream_ptr), self._h)

    def nll_grad(self, sigma_z: float, sigma_dl: float, rho_ptr: int | None = None,
                 sens_ptr: int | None = None, grad_ptr: int | None = None):
        """Device pointers in, (loss, (dL/dsigma_z, dL/dsigma_dl), n_skipped) out;
        dL/drho is written to grad_ptr when given."""
        loss = C.c_double()
        gs = (C.c_double * 2)()
        sk = C.c_int64()
        _check(lib().jpet_strip_nll_grad(self._h, sigma_z, sigma_dl, rho_ptr, sens_ptr,
                                         C.byref(loss), grad_ptr, gs, C.byref(sk)), self._h)
        return loss.value, (gs[0], gs[1]), sk.value

    def counters(self) -> dict:
        c = Counters()
        _check(lib().jpet_strip_get_counters(self._h, C.byref(c)), self._h)
        return {name: getattr(c, name) for name, _ in Counters._fields_}


def run(geom: Geometry, responses: np.ndarray, rho: np.ndarray, n_blocks: int,
        n_iterations_in_block: int, output=None, progress=None, **opts):
    """The reference GPU entry point GPU::Reconstruction::run
    (src/2d/strip/cuda/reconstruction.h:32-44) over host buffers.  ``rho`` is
    updated in place; output(iteration, image) and progress(completed, finished)
    follow the reference's callback protocol.  Returns the device name."""
    ev = np.ascontiguousarray(responses, dtype=np.float32).reshape(-1, 3)
    assert rho.dtype == np.float32 and rho.flags.c_contiguous
    g = geom.c()
    o = make_opts(**opts)

    def _out(it, img, n_z, n_y, _user):
        if output is not None:
            arr = np.ctypeslib.as_array(img, shape=(n_y, n_z)).copy()
            output(it, arr)

    def _prog(done, finished, _user):
        if progress is not None:
            progress(done, bool(finished))

    out_cb = OUTPUT_FN(_out)
    prog_cb = PROGRESS_FN(_prog)
    name = C.create_string_buffer(256)
    _check(lib().jpet_strip_run(C.byref(g), C.byref(o), _ptr(ev) if len(ev) else None, len(ev),
                                _ptr(rho), n_blocks, n_iterations_in_block, out_cb, prog_cb,
                                None, name, 256), None)
    return name.value.decode()
