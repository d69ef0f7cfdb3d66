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

# every symbol include/jpet_strip.h declares
EXPORTED = [
    "jpet_strip_abi_version", "jpet_strip_default_opts", "jpet_strip_create",
    "jpet_strip_destroy", "jpet_strip_last_error", "jpet_strip_set_stream",
    "jpet_strip_set_events", "jpet_strip_set_events_soa", "jpet_strip_set_events_device",
    "jpet_strip_set_image", "jpet_strip_set_image_device", "jpet_strip_iterate",
    "jpet_strip_get_image", "jpet_strip_image_device", "jpet_strip_get_sensitivity",
    "jpet_strip_get_counters", "jpet_strip_synchronize", "jpet_strip_run",
    "jpet_strip_nll_grad", "jpet_strip_iterate_noalloc",
]


class StripError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"jpet_strip error {code}: {message}")
        self.code = code


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
        ("reserved", C.c_int32 * 9),
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
        L.jpet_strip_run.argtypes = [C.POINTER(Geom), C.POINTER(Opts), vp, C.c_int64, vp, C.c_int,
                                     C.c_int, OUTPUT_FN, PROGRESS_FN, vp, C.c_char_p, C.c_size_t]
        for name in EXPORTED:
            if name not in ("jpet_strip_last_error", "jpet_strip_default_opts",
                            "jpet_strip_abi_version"):
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

    def c(self) -> Geom:
        return Geom(self.radius, self.length, self.n_y, self.n_z, self.pixel, self.pixel,
                    self.sigma_z, self.sigma_dl)


def make_opts(device=0, mode=MODE_CPU_REFERENCE, precision=PRECISION_FP32, tile_w=0,
              tile_h=0, block_threads=0, variant=VARIANT_FAST) -> Opts:
    o = Opts()
    lib().jpet_strip_default_opts(C.byref(o))
    o.device, o.mode, o.precision = device, mode, precision
    o.tile_w, o.tile_h, o.block_threads = tile_w, tile_h, block_threads
    o.variant = variant
    return o


def _check(rc: int, h=None):
    if rc != JPET_OK:
        msg = lib().jpet_strip_last_error(h)
        raise StripError(rc, msg.decode() if msg else "?")


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


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
        if self._h:
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
