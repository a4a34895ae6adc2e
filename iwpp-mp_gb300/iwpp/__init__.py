"""Host-side mirror of the reference's reconstruction interface over libiwpp.so.

The reference exposes one synchronous C++ entry point per queue variant
(``IWPP MP/include/MorphologicalReconstruction.cuh:45-46``)::

    void MorphologicalReconstruction(unsigned char* marker, unsigned char* mask,
                                     size_t pitchMarker, size_t pitchMask, int size);

plus the ``clipImage`` precondition kernel (``MR.cu:827-836``) and
``configureHeapSize`` (``IWPP MP/src/globalQueue.cu:3-6``).  This module binds
the same names (raw device pointers, same argument meaning) and a general
form over PyTorch CUDA tensors, which are only used as device buffers.  Every
call goes through the C ABI in ``include/iwpp.h``; there is no CPU fallback:
if the library is missing or no GB300 is present the call raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import Optional, Sequence

from . import _build

U8, U16, I32 = 0, 1, 2
MUTEX, DOUBLE, UNIQUE, ASYNC, DEFAULT = 0, 1, 2, 3, -1
VARIANTS = {"mutex": MUTEX, "mp": MUTEX, "double": DOUBLE, "dq": DOUBLE, "unique": UNIQUE, "uq": UNIQUE,
            "async": ASYNC, "default": DEFAULT}

STATUS = {0: "ok", 1: "invalid argument", 2: "out of device memory", 3: "timeout", 4: "CUDA error",
          5: "queue overflow restarts exhausted", 6: "no sm_103 device", 7: "busy / not finished",
          8: "too large for the scratch or the server budget"}


class IwppError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__(f"{what}: iwpp status {status} ({STATUS.get(status, '?')})")


class Config(ctypes.Structure):
    _fields_ = [("tile_rows", ctypes.c_int), ("queue_capacity", ctypes.c_longlong),
                ("init_passes", ctypes.c_int), ("grid_ctas", ctypes.c_int), ("max_restarts", ctypes.c_int),
                ("timeout_ms", ctypes.c_int), ("clip_marker", ctypes.c_int), ("plain_loads", ctypes.c_int),
                ("solver", ctypes.c_int), ("front_passes", ctypes.c_int), ("phantom_work", ctypes.c_int)]

    @classmethod
    def make(cls, tile_rows=0, queue_capacity=0, init_passes=-1, grid_ctas=0, max_restarts=0, timeout_ms=0,
             clip_marker=0, plain_loads=0, solver=0, front_passes=0, phantom_work=0):
        return cls(tile_rows, queue_capacity, init_passes, grid_ctas, max_restarts, timeout_ms, clip_marker,
                   plain_loads, solver, front_passes, phantom_work)


class Stats(ctypes.Structure):
    _fields_ = [("tiles", ctypes.c_longlong), ("visits", ctypes.c_longlong), ("sweeps", ctypes.c_longlong),
                ("pushes", ctypes.c_longlong), ("rounds", ctypes.c_int), ("restarts", ctypes.c_int),
                ("status", ctypes.c_int), ("variant", ctypes.c_int), ("device_ms", ctypes.c_double),
                ("row_steps", ctypes.c_longlong), ("phase_cycles", ctypes.c_longlong * 5),
                ("launches", ctypes.c_longlong), ("top_pixels", ctypes.c_longlong),
                ("front_stage", ctypes.c_longlong)]

    PHASES = ("queue_read", "fetch", "processing", "dump", "queue_write")

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "phase_cycles"}
        d["phase_cycles"] = dict(zip(self.PHASES, list(self.phase_cycles)))
        return d


class Image(ctypes.Structure):
    _fields_ = [("marker", ctypes.c_void_p), ("mask", ctypes.c_void_p), ("pitch_marker", ctypes.c_size_t),
                ("pitch_mask", ctypes.c_size_t), ("width", ctypes.c_int), ("height", ctypes.c_int),
                ("dtype", ctypes.c_int), ("connectivity", ctypes.c_int)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("lanes", ctypes.c_int), ("max_batch", ctypes.c_int), ("max_pending", ctypes.c_int),
                ("variant", ctypes.c_int), ("tile_rows", ctypes.c_int), ("lane_ctas", ctypes.c_int),
                ("timeout_ms", ctypes.c_int), ("memory_budget", ctypes.c_longlong),
                ("memory_headroom", ctypes.c_longlong)]


class RequestResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("lane", ctypes.c_int), ("batch_size", ctypes.c_int),
                ("reserved", ctypes.c_int), ("latency_us", ctypes.c_double), ("queue_us", ctypes.c_double),
                ("service_us", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class ServerStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_longlong) for k in ("submitted", "completed", "failed", "rejected", "batches",
                                                 "largest_batch", "pixels", "bytes_in_use", "bytes_peak",
                                                 "memory_budget", "held_back")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class TuneResult(ctypes.Structure):
    _fields_ = [("best", Config), ("best_ms", ctypes.c_double), ("default_ms", ctypes.c_double),
                ("candidates", ctypes.c_int), ("reserved", ctypes.c_int)]


class QueueTestResult(ctypes.Structure):
    _fields_ = [("entries", ctypes.c_longlong), ("expected", ctypes.c_longlong), ("mismatched", ctypes.c_longlong),
                ("first_bad", ctypes.c_longlong), ("status", ctypes.c_int), ("variant", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# Every symbol include/iwpp.h declares, with its ctypes signature.
_SIGS = {
    "iwpp_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "iwpp_version": (ctypes.c_int, []),
    "iwpp_handle_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]),
    "iwpp_handle_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "iwpp_workspace_bytes": (ctypes.c_longlong, [ctypes.c_longlong, ctypes.c_int, ctypes.c_longlong]),
    "iwpp_tile_count": (ctypes.c_longlong, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "iwpp_reconstruct": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                        ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.POINTER(Config), ctypes.c_void_p,
                                        ctypes.POINTER(Stats)]),
    "iwpp_reconstruct_async": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                              ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_int, ctypes.c_int, ctypes.POINTER(Config),
                                              ctypes.c_void_p]),
    "iwpp_handle_sync": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Stats)]),
    "iwpp_reconstruct_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Image), ctypes.c_int, ctypes.c_int,
                                              ctypes.POINTER(Config), ctypes.c_void_p, ctypes.POINTER(Stats)]),
    "iwpp_reconstruct_batch_async": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Image), ctypes.c_int,
                                                    ctypes.c_int, ctypes.POINTER(Config), ctypes.c_void_p]),
    "iwpp_plan_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.POINTER(Image),
                                        ctypes.c_int, ctypes.c_int, ctypes.POINTER(Config)]),
    "iwpp_plan_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "iwpp_plan_sync": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Stats)]),
    "iwpp_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "iwpp_clip": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    "iwpp_sweep": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    "iwpp_sweep_timing": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_float)]),
    "iwpp_reconstruct_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                                ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_void_p]),
    "iwpp_fixed_point_violations": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                   ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                   ctypes.c_int, ctypes.c_void_p,
                                                   ctypes.POINTER(ctypes.c_ulonglong)]),
    "iwpp_queue_selftest": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.POINTER(QueueTestResult)]),
    "iwpp_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Image), ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(TuneResult)]),
    "iwpp_tune_save": (ctypes.c_int, [ctypes.c_char_p]),
    "iwpp_tune_load": (ctypes.c_int, [ctypes.c_char_p]),
    "iwpp_tune_clear": (ctypes.c_int, []),
    "iwpp_tune_entries": (ctypes.c_int, []),
    "iwpp_tune_lookup": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_longlong, ctypes.c_int,
                                        ctypes.POINTER(Config)]),
    "iwpp_server_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                          ctypes.POINTER(ServerConfig)]),
    "iwpp_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_ulonglong)]),
    "iwpp_server_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_int,
                                        ctypes.POINTER(RequestResult)]),
    "iwpp_server_stats_get": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ServerStats)]),
    "iwpp_server_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "MorphologicalReconstruction": (None, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                           ctypes.c_int]),
    "configureHeapSize": (None, []),
    "iwpp_last_status": (ctypes.c_int, []),
}

_lib: Optional[ctypes.CDLL] = None


def library_path() -> str:
    return _build.LIBIWPP


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Loads libiwpp.so (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIBIWPP
    if build_if_missing:
        _build.build_iwpp()
    if not os.path.exists(path):
        raise ImportError(f"libiwpp.so not built at {path}")
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols() -> list[str]:
    return list(_SIGS)


def status_string(status: int) -> str:
    return load().iwpp_status_string(status).decode()


# ----------------------------------------------------------------- helpers
def _torch():
    import torch
    return torch


def dtype_code(t) -> int:
    torch = _torch()
    if t.dtype == torch.uint8:
        return U8
    if getattr(torch, "uint16", None) is not None and t.dtype == torch.uint16:
        return U16
    if t.dtype == torch.int16:  # raw 16-bit storage holding unsigned values
        return U16
    if t.dtype == torch.int32:
        return I32
    raise TypeError(f"unsupported pixel dtype {t.dtype}")


def _pitch(t) -> int:
    if t.dim() != 2 or t.stride(1) != 1:
        raise ValueError("images must be 2-D with unit column stride")
    return t.stride(0) * t.element_size()


def _check_cuda(t, name):
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor (device memory)")


def _variant(v) -> int:
    if isinstance(v, str):
        return VARIANTS[v.lower()]
    return int(v)


def _stream_ptr(stream) -> Optional[int]:
    if stream is None:
        torch = _torch()
        return torch.cuda.current_stream().cuda_stream
    return getattr(stream, "cuda_stream", stream)


# ----------------------------------------------- reference-compatible names
def MorphologicalReconstruction(marker_ptr: int, mask_ptr: int, pitchMarker: int, pitchMask: int, size: int) -> None:
    """Exactly the reference entry point: uint8, size x size, 4-connected,
    synchronous, in place on the device buffer at ``marker_ptr``."""
    lib = load()
    lib.MorphologicalReconstruction(marker_ptr, mask_ptr, pitchMarker, pitchMask, size)
    st = lib.iwpp_last_status()
    if st != 0:
        raise IwppError(st, "MorphologicalReconstruction")


def clipImage(marker_ptr: int, mask_ptr: int, pitchMarker: int, pitchMask: int, size: int) -> None:
    """The reference's precondition kernel (marker = min(marker, mask)) for a
    size x size uint8 image, on the default stream."""
    lib = load()
    st = lib.iwpp_clip(marker_ptr, mask_ptr, pitchMarker, pitchMask, size, size, U8, None)
    if st != 0:
        raise IwppError(st, "clipImage")


def configureHeapSize() -> None:
    load().configureHeapSize()


# ------------------------------------------------------------ general API
class Handle:
    """Owns a device workspace; calls through one handle are stream-ordered."""

    def __init__(self, device: int = 0):
        self._lib = load()
        h = ctypes.c_void_p()
        st = self._lib.iwpp_handle_create(ctypes.byref(h), device)
        if st != 0:
            raise IwppError(st, "iwpp_handle_create")
        self.ptr = h

    def close(self):
        if self.ptr:
            self._lib.iwpp_handle_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def reconstruct(marker, mask, connectivity: int = 8, variant="default", config: Optional[Config] = None,
                stream=None, handle: Optional[Handle] = None, check: bool = True) -> Stats:
    """In-place reconstruction by dilation of ``marker`` under ``mask`` (2-D CUDA
    tensors of uint8 / uint16 (or int16 storage) / int32).  Synchronous."""
    lib = load()
    _check_cuda(marker, "marker")
    _check_cuda(mask, "mask")
    if marker.shape != mask.shape or marker.dtype != mask.dtype:
        raise ValueError("marker and mask must have the same shape and dtype")
    h, w = marker.shape
    stats = Stats()
    st = lib.iwpp_reconstruct(handle.ptr if handle else None, marker.data_ptr(), mask.data_ptr(), _pitch(marker),
                              _pitch(mask), w, h, dtype_code(marker), connectivity, _variant(variant),
                              ctypes.byref(config) if config is not None else None, _stream_ptr(stream),
                              ctypes.byref(stats))
    if check and st != 0:
        raise IwppError(st, "iwpp_reconstruct")
    stats.status = st
    return stats


def reconstruct_batch(pairs: Sequence, connectivity=None, variant="default", config: Optional[Config] = None,
                      stream=None, handle: Optional[Handle] = None, check: bool = True) -> Stats:
    """All (marker, mask[, connectivity]) pairs in one persistent launch."""
    lib = load()
    arr = (Image * max(len(pairs), 1))()
    for i, p in enumerate(pairs):
        m, k = p[0], p[1]
        conn = p[2] if len(p) > 2 else (connectivity or 8)
        _check_cuda(m, "marker")
        _check_cuda(k, "mask")
        arr[i] = Image(m.data_ptr(), k.data_ptr(), _pitch(m), _pitch(k), m.shape[1], m.shape[0], dtype_code(m), conn)
    stats = Stats()
    st = lib.iwpp_reconstruct_batch(handle.ptr if handle else None, arr, len(pairs), _variant(variant),
                                    ctypes.byref(config) if config is not None else None, _stream_ptr(stream),
                                    ctypes.byref(stats))
    if check and st != 0:
        raise IwppError(st, "iwpp_reconstruct_batch")
    stats.status = st
    return stats


def autotune(pairs: Sequence, variant="default", repeats: int = 0, handle: Optional["Handle"] = None,
             stream=None) -> dict:
    """iwpp_autotune over (marker, mask[, connectivity]) pairs: times the
    candidate configurations, records the fastest in the tuning table and
    leaves the markers reconstructed.  Returns the winner and its timings."""
    lib = load()
    arr = (Image * max(len(pairs), 1))()
    for i, p in enumerate(pairs):
        m, k = p[0], p[1]
        conn = p[2] if len(p) > 2 else 8
        _check_cuda(m, "marker")
        _check_cuda(k, "mask")
        arr[i] = Image(m.data_ptr(), k.data_ptr(), _pitch(m), _pitch(k), m.shape[1], m.shape[0], dtype_code(m), conn)
    res = TuneResult()
    h = handle or Handle(pairs[0][0].device.index or 0)
    st = lib.iwpp_autotune(h.ptr, arr, len(pairs), _variant(variant), repeats, _stream_ptr(stream), ctypes.byref(res))
    if st != 0:
        raise IwppError(st, "iwpp_autotune")
    b = res.best
    return {"tile_rows": b.tile_rows, "solver": b.solver, "init_passes": b.init_passes,
            "front_passes": b.front_passes, "queue_capacity": b.queue_capacity, "best_ms": res.best_ms,
            "default_ms": res.default_ms, "candidates": res.candidates}


def fixed_point_violations(result, mask, connectivity: int = 8, stream=None) -> int:
    """Pixels of `result` (device tensor) that a neighbour could still raise."""
    n = ctypes.c_ulonglong()
    h, w = result.shape
    st = load().iwpp_fixed_point_violations(result.data_ptr(), mask.data_ptr(), _pitch(result), _pitch(mask), w, h,
                                            dtype_code(result), connectivity, _stream_ptr(stream), ctypes.byref(n))
    if st != 0:
        raise IwppError(st, "iwpp_fixed_point_violations")
    return int(n.value)


def queue_selftest(variant="default", grid_side: int = 128, copies: int = 2, device: int = 0) -> dict:
    """iwpp_queue_selftest: the reference's fill / read-back queue check on
    this library's queues.  Raises if the run itself failed."""
    r = QueueTestResult()
    st = load().iwpp_queue_selftest(device, _variant(variant), grid_side, copies, ctypes.byref(r))
    if st != 0:
        raise IwppError(st, "iwpp_queue_selftest")
    return r.as_dict()


def tune_save(path: str) -> None:
    st = load().iwpp_tune_save(os.fsencode(path))
    if st != 0:
        raise IwppError(st, "iwpp_tune_save")


def tune_load(path: str) -> None:
    st = load().iwpp_tune_load(os.fsencode(path))
    if st != 0:
        raise IwppError(st, "iwpp_tune_load")


def tune_clear() -> None:
    load().iwpp_tune_clear()


def tune_entries() -> int:
    return int(load().iwpp_tune_entries())


def tune_lookup(variant, dtype: int, connectivity: int, pixels: int, batch: bool = False) -> Optional[dict]:
    c = Config()
    st = load().iwpp_tune_lookup(_variant(variant), dtype, connectivity, pixels, 1 if batch else 0, ctypes.byref(c))
    if st != 0:
        return None
    return {"tile_rows": c.tile_rows, "solver": c.solver, "init_passes": c.init_passes,
            "front_passes": c.front_passes, "queue_capacity": c.queue_capacity}


class Plan:
    """A batch captured once into a CUDA graph; launch() re-runs it."""

    def __init__(self, handle: Handle, pairs: Sequence, variant="default", config: Optional[Config] = None):
        self._lib = load()
        self.handle = handle
        self._keep = list(pairs)
        arr = (Image * max(len(pairs), 1))()
        for i, p in enumerate(pairs):
            m, k = p[0], p[1]
            conn = p[2] if len(p) > 2 else 8
            arr[i] = Image(m.data_ptr(), k.data_ptr(), _pitch(m), _pitch(k), m.shape[1], m.shape[0], dtype_code(m),
                           conn)
        ptr = ctypes.c_void_p()
        st = self._lib.iwpp_plan_create(ctypes.byref(ptr), handle.ptr, arr, len(pairs), _variant(variant),
                                        ctypes.byref(config) if config is not None else None)
        if st != 0:
            raise IwppError(st, "iwpp_plan_create")
        self.ptr = ptr

    def launch(self, stream=None):
        st = self._lib.iwpp_plan_launch(self.ptr, _stream_ptr(stream))
        if st != 0:
            raise IwppError(st, "iwpp_plan_launch")

    def sync(self) -> Stats:
        stats = Stats()
        st = self._lib.iwpp_plan_sync(self.ptr, ctypes.byref(stats))
        if st != 0:
            raise IwppError(st, "iwpp_plan_sync")
        return stats

    def close(self):
        if self.ptr:
            self._lib.iwpp_plan_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def clip(marker, mask, stream=None) -> None:
    lib = load()
    h, w = marker.shape
    st = lib.iwpp_clip(marker.data_ptr(), mask.data_ptr(), _pitch(marker), _pitch(mask), w, h, dtype_code(marker),
                       _stream_ptr(stream))
    if st != 0:
        raise IwppError(st, "iwpp_clip")


def sweep(marker, mask, direction: int, connectivity: int = 8, stream=None) -> None:
    """One whole-image sweep: 0 = +X, 1 = +Y, 2 = -X, 3 = -Y."""
    lib = load()
    h, w = marker.shape
    st = lib.iwpp_sweep(marker.data_ptr(), mask.data_ptr(), _pitch(marker), _pitch(mask), w, h, dtype_code(marker),
                        connectivity, direction, _stream_ptr(stream))
    if st != 0:
        raise IwppError(st, "iwpp_sweep")


def sweep_timing(marker, mask, connectivity: int = 8) -> list[float]:
    lib = load()
    h, w = marker.shape
    out = (ctypes.c_float * 4)()
    st = lib.iwpp_sweep_timing(marker.data_ptr(), mask.data_ptr(), _pitch(marker), _pitch(mask), w, h,
                               dtype_code(marker), connectivity, out)
    if st != 0:
        raise IwppError(st, "iwpp_sweep_timing")
    return list(out)


def tile_count(width: int, height: int, dtype: int, tile_rows: int = 0) -> int:
    return int(load().iwpp_tile_count(width, height, dtype, tile_rows))


_NP_DTYPES = {"uint8": U8, "uint16": U16, "int32": I32}


class Server:
    """The serving loop (``iwpp_server_*``): host numpy requests admitted by
    a device-memory budget and run in continuous batches over ``lanes``
    streams.  ``submit`` returns a ticket at once; ``wait`` returns the
    reconstruction (a new array, or ``out``) and the request's timings."""

    def __init__(self, device: int = 0, lanes: int = 0, max_batch: int = 0, max_pending: int = 0,
                 variant="default", tile_rows: int = 0, lane_ctas: int = 0, timeout_ms: int = 0,
                 memory_budget: int = 0, memory_headroom: int = 0):
        lib = load()
        cfg = ServerConfig(lanes, max_batch, max_pending, _variant(variant), tile_rows, lane_ctas, timeout_ms,
                           memory_budget, memory_headroom)
        p = ctypes.c_void_p()
        st = lib.iwpp_server_create(ctypes.byref(p), device, ctypes.byref(cfg))
        if st != 0:
            raise IwppError(st, "iwpp_server_create")
        self._p = p
        self._held = {}

    def submit(self, marker, mask, connectivity: int = 8, out=None) -> int:
        import numpy as np
        if marker.shape != mask.shape or marker.dtype != mask.dtype or marker.ndim != 2:
            raise ValueError("marker and mask must be 2-D arrays of one shape and dtype")
        code = _NP_DTYPES.get(str(marker.dtype))
        if code is None:
            raise TypeError(f"unsupported dtype {marker.dtype}")
        if out is None:
            out = np.empty_like(marker)
        if out.shape != marker.shape or out.dtype != marker.dtype:
            raise ValueError("out must match marker")
        for a in (marker, mask, out):
            if a.size and a.strides[1] != a.itemsize:
                raise ValueError("rows must be contiguous")
        h, w = marker.shape
        t = ctypes.c_ulonglong()
        pitches = [a.strides[0] if a.size else w * a.itemsize for a in (marker, mask, out)]
        st = load().iwpp_server_submit(self._p, marker.ctypes.data, mask.ctypes.data, out.ctypes.data,
                                       pitches[0], pitches[1], pitches[2], w, h, code,
                                       connectivity, ctypes.byref(t))
        if st != 0:
            raise IwppError(st, "iwpp_server_submit")
        self._held[t.value] = (marker, mask, out)
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1):
        r = RequestResult()
        r.status = -1  # filled only by the wait that takes the ticket's result
        st = load().iwpp_server_wait(self._p, ticket, timeout_ms, ctypes.byref(r))
        if st == 7:
            raise TimeoutError(f"request {ticket} not finished")
        if r.status == -1:  # unknown ticket, or another waiter took its result
            raise IwppError(st, "iwpp_server_wait")
        held = self._held.pop(ticket, None)
        if st != 0:
            raise IwppError(st, "iwpp_server_wait")
        return held[2], r.as_dict()

    def stats(self) -> dict:
        s = ServerStats()
        st = load().iwpp_server_stats_get(self._p, ctypes.byref(s))
        if st != 0:
            raise IwppError(st, "iwpp_server_stats_get")
        return s.as_dict()

    def close(self):
        if getattr(self, "_p", None):
            load().iwpp_server_destroy(self._p)
            self._p = None
            self._held.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
