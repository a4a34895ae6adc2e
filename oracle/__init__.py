"""CPU oracle for reconstruction by dilation -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this package, and only as the checker.  The product
library (``libiwpp.so``) never calls it.

``iwpp_oracle.c`` restates the reference's propagation rule
(``IWPP MP/src/MorphologicalReconstruction.cu:43-44``), its 4-neighbourhood
(``MR.cu:34-161``, extended to 8 by the standard definition), its border
("outside pixels do not exist", ``MR.cu:252-256``) and its clip
(``MR.cu:827-836``) with three published schedules: Vincent's 1993 hybrid
(raster, anti-raster, FIFO), sequential raster / anti-raster scans to a fixed
point, and the all-pixels-at-once definition.

Parity pinning: the reference has no CPU path and no golden outputs in its
repository; the oracle is pinned against outputs of the reference's own
CUDA kernels (see ``oracle/refrun``) committed as fixtures under
``tests/golden/``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(ORACLE_DIR, "lib", "liboracle.so")
SRC = [os.path.join(ORACLE_DIR, "iwpp_oracle.c")]
DEPS = SRC + [os.path.join(ORACLE_DIR, "iwpp_oracle_impl.inc"), os.path.join(ORACLE_DIR, "iwpp_oracle.h")]

U8, U16, I32 = 0, 1, 2
_lib = None


def build(force: bool = False) -> str:
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    stale = force or not os.path.exists(LIB) or any(os.path.getmtime(d) > os.path.getmtime(LIB) for d in DEPS)
    if stale:
        cc = os.environ.get("CC", "gcc")
        cmd = [cc, "-O2", "-std=gnu11", "-fPIC", "-shared", "-o", LIB] + SRC
        res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if res.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + res.stdout)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        sig = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t,
               ctypes.c_int, ctypes.c_int]
        for name in ("oracle_reconstruct", "oracle_reconstruct_sr", "oracle_reconstruct_jacobi"):
            getattr(lib, name).argtypes = sig
            getattr(lib, name).restype = ctypes.c_int
        lib.oracle_clip.argtypes = sig[:-1]
        lib.oracle_clip.restype = ctypes.c_int
        _lib = lib
    return _lib


def _code(a: np.ndarray) -> int:
    if a.dtype == np.uint8:
        return U8
    if a.dtype == np.uint16:
        return U16
    if a.dtype == np.int32:
        return I32
    raise TypeError(a.dtype)


def _call(name: str, marker: np.ndarray, mask: np.ndarray, connectivity: int) -> np.ndarray:
    if marker.shape != mask.shape or marker.dtype != mask.dtype or marker.ndim != 2:
        raise ValueError("marker / mask must be 2-D arrays of one shape and dtype")
    out = np.ascontiguousarray(marker).copy()
    k = np.ascontiguousarray(mask)
    rc = getattr(load(), name)(out.ctypes.data_as(ctypes.c_void_p), k.ctypes.data_as(ctypes.c_void_p),
                               out.shape[1], out.shape[0], out.strides[0], k.strides[0], _code(out), connectivity)
    if rc != 0:
        raise RuntimeError(f"{name} failed ({rc})")
    return out


def reconstruct(marker: np.ndarray, mask: np.ndarray, connectivity: int = 8) -> np.ndarray:
    """Vincent 1993 hybrid algorithm; returns a new array."""
    return _call("oracle_reconstruct", marker, mask, connectivity)


def reconstruct_sr(marker: np.ndarray, mask: np.ndarray, connectivity: int = 8) -> np.ndarray:
    return _call("oracle_reconstruct_sr", marker, mask, connectivity)


def reconstruct_jacobi(marker: np.ndarray, mask: np.ndarray, connectivity: int = 8) -> np.ndarray:
    return _call("oracle_reconstruct_jacobi", marker, mask, connectivity)


def clip(marker: np.ndarray, mask: np.ndarray) -> np.ndarray:
    out = np.ascontiguousarray(marker).copy()
    k = np.ascontiguousarray(mask)
    load().oracle_clip(out.ctypes.data_as(ctypes.c_void_p), k.ctypes.data_as(ctypes.c_void_p), out.shape[1],
                       out.shape[0], out.strides[0], k.strides[0], _code(out))
    return out


def sweep(marker: np.ndarray, mask: np.ndarray, direction: int, connectivity: int = 8,
          strip_bytes: int = 128) -> np.ndarray:
    """numpy restatement of one whole-image sweep as libiwpp defines it:
    +X / -X propagate along whole rows; +Y / -Y along whole columns, and with
    8-connectivity also from the two diagonal pixels of the previous row that
    lie in the same 128-byte column strip."""
    m = marker.copy()
    k = mask
    H, W = m.shape
    if direction in (0, 2):
        cols = range(1, W) if direction == 0 else range(W - 2, -1, -1)
        step = -1 if direction == 0 else 1
        for x in cols:
            prev = m[:, x + step]
            m[:, x] = np.maximum(m[:, x], np.minimum(prev, k[:, x]))
        return m
    ppstrip = strip_bytes // m.itemsize
    rows = range(1, H) if direction == 1 else range(H - 2, -1, -1)
    step = -1 if direction == 1 else 1
    lo = np.iinfo(m.dtype).min
    for y in rows:
        prev = m[y + step].copy()
        v = prev.copy()
        if connectivity == 8:
            left = np.full_like(prev, lo)
            right = np.full_like(prev, lo)
            left[1:] = prev[:-1]
            right[:-1] = prev[1:]
            xs = np.arange(W)
            left[(xs % ppstrip) == 0] = lo
            right[(xs % ppstrip) == ppstrip - 1] = lo
            v = np.maximum(v, np.maximum(left, right))
        m[y] = np.maximum(m[y], np.minimum(v, k[y]))
    return m
