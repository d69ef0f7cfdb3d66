"""ctypes binding of the 3D hybrid C ABI (include/jpet_hybrid.h, libjpet_strip.so).

``HybridReconstruction`` mirrors PET3D::Hybrid::Reconstruction
(src/3d/hybrid/reconstruction.h): it owns one library handle whose set-up runs
calculate_weight / calculate_sensitivity / normalize_geometry_weights as the
reference command does (reconstruction_cmd.cpp:462-522), loads responses
(``<<``, translate_to_frame plus the bounding-box filter) and runs iterations
(``__call__``, Reconstruction::operator()).  ``rho`` and ``sensitivity`` are in
the reference's own layouts.  There is no fallback: without the compiled
library this module raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .hybrid_workloads import FRAME_EVENT_DTYPE, RESPONSE_DTYPE, HybridGeometry

WEIGHTS_COMPUTED, WEIGHTS_GIVEN, WEIGHTS_NORMALIZED = 0, 1, 2
SENSITIVITY_COMPUTED, SENSITIVITY_ONE, SENSITIVITY_GIVEN, SENSITIVITY_GIVEN_3D = 0, 1, 2, 3


class HybGeom(C.Structure):
    _fields_ = [
        ("n_detectors", C.c_int32),
        ("n_pixel_infos", C.c_int64),
        ("lor_segments", C.c_void_p),
        ("lor_widths", C.c_void_p),
        ("pixels", C.c_void_p),
        ("pixel_positions", C.c_void_p),
        ("pixel_weights", C.c_void_p),
        ("lor_pixel_info_begin", C.c_void_p),
        ("lor_pixel_info_end", C.c_void_p),
        ("n_columns", C.c_int32),
        ("n_rows", C.c_int32),
        ("pixel_size", C.c_float),
        ("lower_left_x", C.c_float),
        ("lower_left_y", C.c_float),
        ("n_planes", C.c_int32),
        ("z_left", C.c_float),
        ("sigma_z", C.c_float),
        ("sigma_dl", C.c_float),
        ("length", C.c_float),
        ("n_planes_half", C.c_int32),
    ]


class HybOpts(C.Structure):
    _fields_ = [
        ("device", C.c_int32),
        ("weights", C.c_int32),
        ("sensitivity", C.c_int32),
        ("sensitivity_map", C.c_void_p),
        ("block_threads", C.c_int32),
        ("reserved", C.c_int32),
    ]


class HybCounters(C.Structure):
    _fields_ = [
        ("used_events", C.c_int64),
        ("used_pixels", C.c_int64),
        ("used_voxels", C.c_int64),
        ("contributing", C.c_int64),
    ]


EXPORTED = [
    "jpet_hybrid_default_opts", "jpet_hybrid_create", "jpet_hybrid_destroy",
    "jpet_hybrid_last_error", "jpet_hybrid_set_stream", "jpet_hybrid_set_responses",
    "jpet_hybrid_set_responses_device", "jpet_hybrid_set_frame_events",
    "jpet_hybrid_get_frame_events", "jpet_hybrid_set_image", "jpet_hybrid_get_image",
    "jpet_hybrid_get_sensitivity", "jpet_hybrid_get_weights", "jpet_hybrid_iterate",
    "jpet_hybrid_get_counters", "jpet_hybrid_synchronize", "jpet_hybrid_run",
]


def _ptr(a) -> int | None:
    return a.ctypes.data if a is not None and a.size else None


def _lib():
    L = capi.lib()
    if not getattr(L, "_hybrid_ready", False):
        vp = C.c_void_p
        L.jpet_hybrid_create.argtypes = [C.POINTER(HybGeom), C.POINTER(HybOpts),
                                         C.POINTER(vp)]
        L.jpet_hybrid_destroy.argtypes = [vp]
        L.jpet_hybrid_last_error.argtypes = [vp]
        L.jpet_hybrid_last_error.restype = C.c_char_p
        L.jpet_hybrid_set_stream.argtypes = [vp, vp]
        L.jpet_hybrid_set_responses.argtypes = [vp, vp, C.c_int64]
        L.jpet_hybrid_set_responses_device.argtypes = [vp, vp, C.c_int64]
        L.jpet_hybrid_set_frame_events.argtypes = [vp, vp, C.c_int64]
        L.jpet_hybrid_get_frame_events.argtypes = [vp, vp, C.POINTER(C.c_int64)]
        L.jpet_hybrid_set_image.argtypes = [vp, vp]
        L.jpet_hybrid_get_image.argtypes = [vp, vp]
        L.jpet_hybrid_get_sensitivity.argtypes = [vp, vp]
        L.jpet_hybrid_get_weights.argtypes = [vp, vp]
        L.jpet_hybrid_iterate.argtypes = [vp, C.c_int]
        L.jpet_hybrid_get_counters.argtypes = [vp, C.POINTER(HybCounters)]
        L.jpet_hybrid_synchronize.argtypes = [vp]
        L.jpet_hybrid_run.argtypes = [C.POINTER(HybGeom), vp, vp, C.c_int64, vp, C.c_int,
                                      C.c_int, C.c_int, vp, vp, vp, C.c_int, C.c_char_p,
                                      C.c_size_t]
        L._hybrid_ready = True
    return L


def geom_struct(g: HybridGeometry, weights=None) -> tuple[HybGeom, list]:
    """jpet_hybrid_geom view of a HybridGeometry (arrays kept alive by the list)."""
    w = g.weights if weights is None else weights
    keep = [np.ascontiguousarray(a) for a in (g.segments, g.widths, g.pixels, g.positions,
                                               np.asarray(w, np.float32), g.info_begin,
                                               g.info_end)]
    s = HybGeom(g.n_detectors, g.n_pixel_infos, *[_ptr(a) for a in keep], g.n_columns,
                g.n_rows, g.pixel_size, g.lower_left_x, g.lower_left_y, g.n_planes, g.z_left,
                g.sigma_z, g.sigma_dl, g.length, g.n_planes_half)
    return s, keep


class HybridError(RuntimeError):
    pass


class HybridReconstruction:
    """One reconstruction on one device (the reference's Reconstruction object).
    A geometry with n_planes_half > 1 (one system matrix per plane half) has a
    3D sensitivity of that depth; SENSITIVITY_GIVEN_3D takes the external 3D
    sensitivity (depth n_planes / 2 for one plane half)."""

    def __init__(self, g: HybridGeometry, weights: int = WEIGHTS_COMPUTED,
                 sensitivity: int = SENSITIVITY_COMPUTED, sensitivity_map=None, device: int = 0):
        self.g = g
        self.sens_depth = (g.n_planes_half if g.n_planes_half > 1
                           else (g.n_planes // 2 if sensitivity == SENSITIVITY_GIVEN_3D else 1))
        L = _lib()
        gs, self._keep = geom_struct(g)
        smap = None if sensitivity_map is None else np.ascontiguousarray(sensitivity_map,
                                                                         np.float32)
        self._keep.append(smap)
        o = HybOpts(device, weights, sensitivity, _ptr(smap), 0, 0)
        h = C.c_void_p()
        rc = L.jpet_hybrid_create(C.byref(gs), C.byref(o), C.byref(h))
        if rc != 0:
            raise HybridError(f"jpet_hybrid_create {rc}: "
                              f"{L.jpet_hybrid_last_error(None).decode()}")
        self.h = h

    def _check(self, rc, what):
        if rc != 0:
            msg = _lib().jpet_hybrid_last_error(self.h).decode()
            raise HybridError(f"{what} {rc}: {msg}")

    def close(self):
        if getattr(self, "h", None):
            _lib().jpet_hybrid_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        self.close()

    # --- events ---
    def set_responses(self, responses):
        r = np.ascontiguousarray(responses, RESPONSE_DTYPE)
        self._check(_lib().jpet_hybrid_set_responses(self.h, _ptr(r), r.shape[0]),
                    "set_responses")
        return self

    __lshift__ = set_responses

    def set_responses_device(self, ptr: int, n: int):
        self._check(_lib().jpet_hybrid_set_responses_device(self.h, ptr, n),
                    "set_responses_device")

    def set_frame_events(self, events):
        e = np.ascontiguousarray(events, FRAME_EVENT_DTYPE)
        self._check(_lib().jpet_hybrid_set_frame_events(self.h, _ptr(e), e.shape[0]),
                    "set_frame_events")

    def frame_events(self) -> np.ndarray:
        n = C.c_int64()
        L = _lib()
        self._check(L.jpet_hybrid_get_frame_events(self.h, None, C.byref(n)), "get_frame_events")
        out = np.zeros(n.value, FRAME_EVENT_DTYPE)
        if n.value:
            self._check(L.jpet_hybrid_get_frame_events(self.h, _ptr(out), C.byref(n)),
                        "get_frame_events")
        return out

    @property
    def n_events(self) -> int:
        n = C.c_int64()
        self._check(_lib().jpet_hybrid_get_frame_events(self.h, None, C.byref(n)),
                    "get_frame_events")
        return n.value

    # --- images ---
    @property
    def rho(self) -> np.ndarray:
        out = np.empty(self.g.n_voxels, np.float32)
        self._check(_lib().jpet_hybrid_get_image(self.h, _ptr(out)), "get_image")
        return out

    @rho.setter
    def rho(self, v):
        a = np.ascontiguousarray(v, np.float32).reshape(-1)
        assert a.size == self.g.n_voxels
        self._check(_lib().jpet_hybrid_set_image(self.h, _ptr(a)), "set_image")

    @property
    def sensitivity(self) -> np.ndarray:
        out = np.empty(self.sens_depth * self.g.n_columns * self.g.n_rows, np.float32)
        self._check(_lib().jpet_hybrid_get_sensitivity(self.h, _ptr(out)), "get_sensitivity")
        return out

    @property
    def weights(self) -> np.ndarray:
        out = np.empty(self.g.n_planes_half * self.g.n_pixel_infos, np.float32)
        self._check(_lib().jpet_hybrid_get_weights(self.h, _ptr(out)), "get_weights")
        return out

    # --- iterations ---
    def __call__(self, n_iterations: int = 1):
        self._check(_lib().jpet_hybrid_iterate(self.h, n_iterations), "iterate")
        return self

    iterate = __call__

    def synchronize(self):
        self._check(_lib().jpet_hybrid_synchronize(self.h), "synchronize")

    def set_stream(self, stream_ptr: int | None):
        self._check(_lib().jpet_hybrid_set_stream(self.h, stream_ptr), "set_stream")

    def statistics(self) -> dict:
        c = HybCounters()
        self._check(_lib().jpet_hybrid_get_counters(self.h, C.byref(c)), "get_counters")
        return {"used_events": c.used_events, "used_pixels": c.used_pixels,
                "used_voxels": c.used_voxels, "contributing": c.contributing}


OUTPUT_FN = C.CFUNCTYPE(None, C.c_int, C.POINTER(C.c_float), C.c_void_p)
PROGRESS_FN = C.CFUNCTYPE(None, C.c_int, C.c_int, C.c_void_p)


def run(g: HybridGeometry, normalized_weights, sensitivity, frame_events, rho, n_blocks: int,
        n_iterations_in_block: int, start_iteration: int = 0, output=None, progress=None,
        device: int = 0):
    """jpet_hybrid_run: the reference GPU entry point over host buffers.  Returns
    (rho, device name); output(iteration, image) and progress(completed,
    finished) are called as the reference calls its delegates."""
    L = _lib()
    gs, keep = geom_struct(g, normalized_weights)
    sens = np.ascontiguousarray(sensitivity, np.float32)
    ev = np.ascontiguousarray(frame_events, FRAME_EVENT_DTYPE)
    r = np.array(rho, np.float32, copy=True).reshape(-1)
    n_vox = g.n_voxels

    def _out(it, img, _u):
        if output:
            output(it, np.ctypeslib.as_array(img, (n_vox,)).copy())

    def _prog(done, fin, _u):
        if progress:
            progress(done, bool(fin))

    ocb, pcb = OUTPUT_FN(_out), PROGRESS_FN(_prog)
    name = C.create_string_buffer(256)
    rc = L.jpet_hybrid_run(C.byref(gs), _ptr(sens), _ptr(ev), ev.shape[0], _ptr(r), n_blocks,
                           n_iterations_in_block, start_iteration,
                           C.cast(ocb, C.c_void_p), C.cast(pcb, C.c_void_p), None, device, name,
                           256)
    if rc != 0:
        raise HybridError(f"jpet_hybrid_run {rc}: {L.jpet_hybrid_last_error(None).decode()}")
    return r, name.value.decode()
