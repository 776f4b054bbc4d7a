"""ctypes access to the CPU oracle (test infrastructure only).

``port`` is the C++ restatement (oracle/asuna_oracle.cpp); ``ref`` is the
reference's own shader source compiled as host C++ (built where the reference
checkout, or an earlier translation of it, is present).  Both take the same asuna_scene_desc / asuna_shot as
the library.  Imported only by tests, the smoke check and the benchmark's CPU
baseline.
"""
import ctypes as C
import os
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(_HERE))
from asuna_gb300 import _abi as A  # noqa: E402

from . import build_oracle  # noqa: E402


class OracleStats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("extend_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("nodes_visited", C.c_uint64), ("tris_tested", C.c_uint64), ("seconds", C.c_double),
                ("threads", C.c_int)]


_port = None
_ref = None


def port():
    global _port
    if _port is None:
        L = C.CDLL(build_oracle.build_port())
        L.oracle_scene_create.argtypes = [C.POINTER(A.SceneDesc), C.POINTER(C.c_void_p)]
        L.oracle_scene_destroy.argtypes = [C.c_void_p]
        L.oracle_render.argtypes = [C.c_void_p, C.POINTER(A.Shot), C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                                    C.c_int, C.c_int, C.POINTER(OracleStats)]
        L.oracle_render_pixels_f64.argtypes = [C.c_void_p, C.POINTER(A.Shot), C.c_void_p, C.c_uint32, C.c_int,
                                               C.c_void_p, C.c_void_p, C.POINTER(OracleStats)]
        L.oracle_xxhash32.restype = C.c_uint32
        L.oracle_xxhash32.argtypes = [C.c_uint32] * 3
        L.oracle_pcg.restype = C.c_uint32
        L.oracle_pcg.argtypes = [C.POINTER(C.c_uint32)]
        L.oracle_rand.restype = C.c_float
        L.oracle_rand.argtypes = [C.POINTER(C.c_uint32)]
        L.oracle_trace.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_float,
                                   C.POINTER(C.c_float), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                   C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.oracle_occluded.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_float]
        L.oracle_math.restype = C.c_float
        L.oracle_math.argtypes = [C.c_int, C.c_float, C.c_float]
        L.oracle_envmap_tables.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_tonemap.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]
        L.oracle_diffuse_fresnel.restype = C.c_float
        L.oracle_diffuse_fresnel.argtypes = [C.c_float, C.c_int]
        L.oracle_camera_perspective.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_float, C.c_float,
                                                C.c_uint32, C.c_uint32, C.POINTER(A.Camera)]
        _port = L
    return _port


def ref():
    """The reference-shader library, or None where the reference tree is absent."""
    global _ref
    if _ref is None:
        path = build_oracle.build_ref()
        if path is None:
            return None
        L = C.CDLL(path)
        L.ref_render.argtypes = [C.POINTER(A.SceneDesc), C.POINTER(A.Shot), C.c_void_p, C.c_void_p, C.c_int]
        L.ref_xxhash32.restype = C.c_uint32
        L.ref_xxhash32.argtypes = [C.c_uint32] * 3
        L.ref_rand.restype = C.c_float
        L.ref_rand.argtypes = [C.POINTER(C.c_uint32)]
        L.ref_sample_begin.restype = C.c_void_p
        L.ref_sample_begin.argtypes = [C.POINTER(A.SceneDesc), C.POINTER(A.Shot), C.c_void_p]
        L.ref_sample_run.argtypes = [C.c_void_p, C.POINTER(A.Shot), C.c_void_p, C.c_uint32, C.c_int,
                                     C.POINTER(OracleStats)]
        L.ref_sample_end.argtypes = [C.c_void_p]
        _ref = L
    return _ref


class OracleScene:
    def __init__(self, desc):
        self.L = port()
        h = C.c_void_p()
        rc = self.L.oracle_scene_create(desc.ptr, C.byref(h))
        if rc:
            raise RuntimeError(f"oracle_scene_create failed: {rc}")
        self.h = h
        self._desc = desc

    def render(self, shot, film=None, records=True, pixels=None, threads=0, precision=32):
        npix = shot.width * shot.height if pixels is None else len(pixels)
        if film is None:
            film = np.zeros((A.NUM_OUTPUT_IMAGES, shot.height, shot.width, 4), np.float32)
        rec = np.zeros(shot.frames * npix, A.PATH_RECORD_DTYPE) if records else None
        px = None if pixels is None else np.ascontiguousarray(pixels, np.uint32)
        st = OracleStats()
        rc = self.L.oracle_render(self.h, C.byref(shot), film.ctypes.data, None if rec is None else rec.ctypes.data,
                                  None if px is None else px.ctypes.data, npix, threads, precision, C.byref(st))
        if rc:
            raise RuntimeError(f"oracle_render failed: {rc}")
        return film, rec, {k: getattr(st, k) for k, _ in OracleStats._fields_}

    def pixels_f64(self, shot, pixels, threads=0, variance=False):
        """FP64 render of the listed pixels: (mean rgb [n, 3], stats), or
        (mean, variance of the mean, stats) with `variance`."""
        px = np.ascontiguousarray(pixels, np.uint32)
        out = np.zeros((len(px), 3), np.float64)
        var = np.zeros((len(px), 3), np.float64) if variance else None
        st = OracleStats()
        rc = self.L.oracle_render_pixels_f64(self.h, C.byref(shot), px.ctypes.data, len(px), threads,
                                             out.ctypes.data, None if var is None else var.ctypes.data,
                                             C.byref(st))
        if rc:
            raise RuntimeError(f"oracle_render_pixels_f64 failed: {rc}")
        stats = {k: getattr(st, k) for k, _ in OracleStats._fields_}
        return (out, var, stats) if variance else (out, stats)

    def trace(self, o, d, tmin=1e-5, tmax=1e10):
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        t, u, v = C.c_float(), C.c_float(), C.c_float()
        inst, prim = C.c_uint32(), C.c_uint32()
        hit = self.L.oracle_trace(self.h, o.ctypes.data, d.ctypes.data, tmin, tmax, C.byref(t), C.byref(inst),
                                  C.byref(prim), C.byref(u), C.byref(v))
        return (t.value, inst.value, prim.value, u.value, v.value) if hit else None

    def occluded(self, o, d, tmin, tmax):
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        return bool(self.L.oracle_occluded(self.h, o.ctypes.data, d.ctypes.data, tmin, tmax))

    def close(self):
        if self.h:
            self.L.oracle_scene_destroy(self.h)
            self.h = None

    __del__ = close


def ref_render(desc, shot, threads=0):
    """Film and per-path records from the reference's own shader code."""
    L = ref()
    if L is None:
        raise RuntimeError("reference tree not available")
    film = np.zeros((A.NUM_OUTPUT_IMAGES, shot.height, shot.width, 4), np.float32)
    rec = np.zeros(shot.frames * shot.width * shot.height, A.PATH_RECORD_DTYPE)
    rc = L.ref_render(desc.ptr, C.byref(shot), film.ctypes.data, rec.ctypes.data, threads)
    if rc:
        raise RuntimeError(f"ref_render failed: {rc}")
    return film, rec


class OracleHelpers:
    """The oracle's restatements of the host preprocessing a scene
    description needs (asuna_gb300.scene.host_helpers), so that a process
    timing only reference code builds its workload without the library."""

    @staticmethod
    def diffuse_fresnel(ior):
        return port().oracle_diffuse_fresnel(C.c_float(ior), 1000)

    @staticmethod
    def camera_perspective(e, l, u, fov, aperture, focal_distance, width, height, cam):
        rc = port().oracle_camera_perspective(e.ctypes.data, l.ctypes.data, u.ctypes.data, fov, aperture,
                                              focal_distance, width, height, C.byref(cam))
        if rc:
            raise RuntimeError(f"oracle_camera_perspective failed: {rc}")


class RefSampler:
    """The reference's own shader code over pixel samples of one shot size
    (one session at a time): run(shot, pixels) -> stats of the rays traced."""

    def __init__(self, desc, shot):
        self.L = ref()
        if self.L is None:
            raise RuntimeError("reference shader library not available")
        self.film = np.zeros((A.NUM_OUTPUT_IMAGES, shot.height, shot.width, 4), np.float32)
        self._desc = desc
        self.h = self.L.ref_sample_begin(desc.ptr, C.byref(shot), self.film.ctypes.data)
        if not self.h:
            raise RuntimeError("ref_sample_begin failed")

    def run(self, shot, pixels, threads=0):
        px = np.ascontiguousarray(pixels, np.uint32)
        st = OracleStats()
        rc = self.L.ref_sample_run(self.h, C.byref(shot), px.ctypes.data, len(px), threads, C.byref(st))
        if rc:
            raise RuntimeError(f"ref_sample_run failed: {rc}")
        return {k: getattr(st, k) for k, _ in OracleStats._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.L.ref_sample_end(self.h)
            self.h = None

    __del__ = close
