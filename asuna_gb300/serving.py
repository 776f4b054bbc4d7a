"""Python side of the render server (continuous batching, include/asuna_rt.h).

``Server`` wraps asuna_server_*; ``poisson_load`` drives it with requests
arriving as a Poisson process on wall-clock time and reports latency
percentiles, throughput and the rejection rate.
"""
import ctypes as C
import time

import numpy as np

from . import _abi as A
from ._abi import check, lib


class ServerOpts(C.Structure):
    _fields_ = [("device", C.c_int32), ("slots", C.c_uint32), ("frames_per_chunk", C.c_uint32),
                ("max_batch", C.c_uint32), ("max_queue", C.c_uint32), ("reserved", C.c_uint32),
                ("memory_budget", C.c_uint64), ("path_budget", C.c_uint64)]


REQUEST_DENOISE = 1


class Request(C.Structure):
    _fields_ = [("scene", C.c_uint32), ("flags", C.c_uint32), ("shot", A.Shot)]


class RequestResult(C.Structure):
    _fields_ = [("id", C.c_uint64), ("status", C.c_int32), ("scene", C.c_uint32), ("arrival_s", C.c_double),
                ("start_s", C.c_double), ("finish_s", C.c_double), ("samples", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [("admitted", C.c_uint64), ("rejected", C.c_uint64), ("pending", C.c_uint64),
                ("samples", C.c_uint64), ("memory_used", C.c_uint64), ("elapsed_s", C.c_double),
                ("scenes_built", C.c_uint64), ("scenes_evicted", C.c_uint64), ("denoised", C.c_uint64),
                ("scene_bytes", C.c_uint64)]


_SIGS = [
    ("asuna_server_create", [C.POINTER(ServerOpts), C.POINTER(C.c_void_p)]),
    ("asuna_server_add_scene", [C.c_void_p, C.POINTER(A.SceneDesc), C.POINTER(C.c_uint32)]),
    ("asuna_server_register_scene", [C.c_void_p, C.POINTER(A.SceneDesc), C.POINTER(C.c_uint32)]),
    ("asuna_server_set_denoiser", [C.c_void_p, C.POINTER(A.DenoiserOpts), C.c_void_p, C.c_uint64]),
    ("asuna_server_submit", [C.c_void_p, C.POINTER(Request), C.POINTER(C.c_uint64)]),
    ("asuna_server_poll", [C.c_void_p, C.POINTER(RequestResult), C.c_uint32, C.POINTER(C.c_uint32)]),
    ("asuna_server_read", [C.c_void_p, C.c_uint64, C.c_int, C.c_void_p]),
    ("asuna_server_release", [C.c_void_p, C.c_uint64]),
    ("asuna_server_drain", [C.c_void_p, C.c_double]),
    ("asuna_server_get_stats", [C.c_void_p, C.POINTER(ServerStats)]),
    ("asuna_server_destroy", [C.c_void_p]),
]


def _bind():
    L = lib()
    for name, args in _SIGS:
        f = getattr(L, name)
        f.restype = C.c_int
        f.argtypes = args
    return L


class Server:
    def __init__(self, device=0, slots=3, frames_per_chunk=16, max_batch=8, max_queue=0, memory_budget=150 << 30,
                 path_budget=0):
        self.L = _bind()
        o = ServerOpts(device, slots, frames_per_chunk, max_batch, max_queue, 0, memory_budget, path_budget)
        self._keep = []
        h = C.c_void_p()
        check(self.L.asuna_server_create(C.byref(o), C.byref(h)))
        self.h = h

    def add_scene(self, desc):
        """Builds the scene now; it stays resident."""
        sid = C.c_uint32()
        check(self.L.asuna_server_add_scene(self.h, desc.ptr, C.byref(sid)))
        return sid.value

    def register_scene(self, desc):
        """Registers a scene the server builds when its first request is
        admitted and may drop when idle (keep `desc` alive)."""
        sid = C.c_uint32()
        check(self.L.asuna_server_register_scene(self.h, desc.ptr, C.byref(sid)))
        self._keep.append(desc)
        return sid.value

    def set_denoiser(self, params, max_pixels=1088 * 1920, channels=(32, 48, 64, 96, 128)):
        """Trained denoiser parameters (Denoiser.get_params) for denoised requests."""
        o = A.DenoiserOpts()
        o.levels = len(channels)
        for k, c in enumerate(channels):
            o.channels[k] = c
        o.max_pixels = max_pixels
        o.tensor_memory = 1
        p = np.ascontiguousarray(params, np.float32)
        check(self.L.asuna_server_set_denoiser(self.h, C.byref(o), p.ctypes.data, p.size))

    def submit(self, scene, shot, denoise=False):
        r = Request(scene, REQUEST_DENOISE if denoise else 0, shot)
        rid = C.c_uint64()
        check(self.L.asuna_server_submit(self.h, C.byref(r), C.byref(rid)))
        return rid.value

    def poll(self, max_n=256):
        buf = (RequestResult * max_n)()
        n = C.c_uint32()
        check(self.L.asuna_server_poll(self.h, buf, max_n, C.byref(n)))
        return [{k: getattr(buf[i], k) for k, _ in RequestResult._fields_} for i in range(n.value)]

    def read(self, rid, width, height, image=0):
        out = np.empty((height, width, 4), np.float32)
        check(self.L.asuna_server_read(self.h, rid, image, out.ctypes.data))
        return out

    def release(self, rid):
        check(self.L.asuna_server_release(self.h, rid))

    def drain(self, timeout_s=600.0):
        check(self.L.asuna_server_drain(self.h, timeout_s))

    def stats(self):
        s = ServerStats()
        check(self.L.asuna_server_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.L.asuna_server_destroy(self.h)
            self.h = None

    __del__ = close


def poisson_load(server, requests, rate_hz, seed=0, keep=None, timeout_s=1800.0, denoise=None):
    """Submits (scene, shot) pairs at Poisson arrival times (rate_hz per second
    of wall-clock time; `denoise[k]` sets request k's denoise flag), collects
    every result, releases films as they finish (except requests listed in
    `keep` by index, whose image 0 is read first) and returns a summary with
    latency percentiles."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, size=len(requests))
    t0 = time.perf_counter()
    due = t0 + np.cumsum(gaps)
    ids, results, kept = [], {}, {}
    keep = set(keep or [])
    idx_of = {}
    def collect():
        # finished requests: read what is kept, release every film at once
        for r in server.poll():
            results[r["id"]] = r
            if r["status"] == A.OK:
                k = idx_of[r["id"]]
                if k in keep:
                    shot = requests[k][1]
                    kept[k] = server.read(r["id"], shot.width, shot.height, 0)
            server.release(r["id"])

    for k, (scene, shot) in enumerate(requests):
        while time.perf_counter() < due[k]:
            collect()
            time.sleep(min(0.002, max(0.0, due[k] - time.perf_counter())))
        rid = server.submit(scene, shot, denoise=bool(denoise[k]) if denoise is not None else False)
        ids.append(rid)
        idx_of[rid] = k
    deadline = time.perf_counter() + timeout_s
    while len(results) < len(ids) and time.perf_counter() < deadline:
        collect()
        time.sleep(0.002)
    ok = [r for r in results.values() if r["status"] == A.OK]
    lat = np.array([r["finish_s"] - r["arrival_s"] for r in ok]) if ok else np.zeros(1)
    wait = np.array([r["start_s"] - r["arrival_s"] for r in ok]) if ok else np.zeros(1)
    span = (max(r["finish_s"] for r in ok) - min(r["arrival_s"] for r in ok)) if ok else 1.0
    rejected = sum(1 for r in results.values() if r["status"] != A.OK)
    return {
        "requests": len(ids), "completed": len(ok), "rejected": rejected,
        "rejection_rate": rejected / max(len(ids), 1), "missing": len(ids) - len(results),
        "p50_s": float(np.percentile(lat, 50)), "p95_s": float(np.percentile(lat, 95)),
        "p99_s": float(np.percentile(lat, 99)), "mean_queue_wait_s": float(wait.mean()),
        "queued_frac": float(np.mean(wait > 0.01)),
        "msamples_per_s": sum(r["samples"] for r in ok) / max(span, 1e-9) / 1e6,
        "rate_hz": rate_hz, "films": kept,
    }
