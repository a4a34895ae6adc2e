"""Seeded synthetic workloads (numpy arrays from libiwpp_synth.so).

The reference's own inputs are JPEG/PGM files that are partly missing and
whose golden outputs live outside its repository, so every workload is
synthesised with the shapes, sizes and value laws of the five benchmark
configurations:

0. 1024^2 uint8, 8-conn, seed 0: smoothed noise (sigma 4) + 200 discs
   (radius 5-40, level 180-255); h-dome marker, h = 40.
1. 4096^2 uint8, 4/8-conn, seed 1, sigma 8, 2000 discs, h in {10, 40, 100}.
2. 16384^2, 8-conn, seed 2: smoothed noise (sigma 16) + a one-pixel square
   spiral corridor of the dtype maximum (arm pitch 256, frozen here); marker =
   dtype minimum except 64 seeds = mask value, the first at the spiral start.
   uint8, uint16 (0-65535) and int32 (full signed range).
3. 64 images, seed 3: width log-uniform in [512, 4096], height in
   [512, 3072], uint8/uint16 and 4/8-conn drawn per image, h-dome markers with
   h uniform in [5, 120]; sigma 4 and disc count proportional to area.
4. Served stream, seed 4: Poisson arrivals (2000 / s), sides log-uniform in
   [256, 8192], uint8 80 % / uint16 20 %, 8-conn, h-dome (h in [5, 120]) or
   sparse-seed (0.01 % of pixels) markers, 50 / 50.

Draws of sizes / kinds use ``random.Random(seed).random()`` only (stable
across Python versions); pixel content comes from the C generator, which is
bit-identical on x86-64 and AArch64.
"""
from __future__ import annotations

import ctypes
import math
import os
import random
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _build

U8, U16, I32 = 0, 1, 2
NP_DTYPE = {U8: np.uint8, U16: np.uint16, I32: np.int32}
SPIRAL_ARM_PITCH = 256

_lib = None


def load():
    global _lib
    if _lib is None:
        _build.build_synth()
        lib = ctypes.CDLL(_build.LIBSYNTH)
        vp, sz, i, u64, d = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint64, ctypes.c_double
        lib.iwpp_synth_noise_mask.argtypes = [vp, i, i, sz, i, u64, d, i, i, i, i, i, i]
        lib.iwpp_synth_hdome_marker.argtypes = [vp, vp, i, i, sz, sz, i, i]
        lib.iwpp_synth_sparse_marker.argtypes = [vp, vp, i, i, sz, sz, i, u64, d]
        lib.iwpp_synth_spiral_corridor.argtypes = [vp, i, i, sz, i, i, ctypes.POINTER(i), ctypes.POINTER(i)]
        lib.iwpp_synth_spiral_corridor.restype = ctypes.c_int64
        lib.iwpp_synth_seed_marker.argtypes = [vp, vp, i, i, sz, sz, i, u64, i, i, i]
        lib.iwpp_synth_uniform_pair.argtypes = [vp, vp, i, i, sz, sz, u64]
        lib.iwpp_synth_scale8.argtypes = [i, i]
        lib.iwpp_synth_scale8.restype = ctypes.c_int64
        lib.iwpp_synth_mt64_nth.argtypes = [u64, u64]
        lib.iwpp_synth_mt64_nth.restype = ctypes.c_uint64
        _lib = lib
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def dtype_code(a: np.ndarray) -> int:
    for code, dt in NP_DTYPE.items():
        if a.dtype == dt:
            return code
    raise TypeError(a.dtype)


def noise_mask(width: int, height: int, dtype: int, seed: int, sigma: float, ndiscs: int, rmin: int = 5,
               rmax: int = 40, vmin8: int = 180, vmax8: int = 255, nthreads: int = 0) -> np.ndarray:
    out = np.empty((height, width), NP_DTYPE[dtype])
    rc = load().iwpp_synth_noise_mask(_ptr(out), width, height, out.strides[0], dtype, seed, float(sigma), ndiscs,
                                      rmin, rmax, vmin8, vmax8, nthreads)
    if rc != 0:
        raise RuntimeError(f"iwpp_synth_noise_mask failed ({rc})")
    return out


def hdome_marker(mask: np.ndarray, h8: int) -> np.ndarray:
    out = np.empty_like(mask)
    load().iwpp_synth_hdome_marker(_ptr(out), _ptr(mask), mask.shape[1], mask.shape[0], out.strides[0],
                                   mask.strides[0], dtype_code(mask), h8)
    return out


def sparse_marker(mask: np.ndarray, seed: int, fraction: float = 1e-4) -> np.ndarray:
    out = np.empty_like(mask)
    load().iwpp_synth_sparse_marker(_ptr(out), _ptr(mask), mask.shape[1], mask.shape[0], out.strides[0],
                                    mask.strides[0], dtype_code(mask), seed, float(fraction))
    return out


def spiral_case(width: int, height: int, dtype: int, seed: int = 2, sigma: float = 16.0,
                arm_pitch: int = SPIRAL_ARM_PITCH, nseeds: int = 64, nthreads: int = 0):
    """Configuration-2 pair: (marker, mask, corridor_pixels)."""
    mask = noise_mask(width, height, dtype, seed, sigma, 0, nthreads=nthreads)
    sx, sy = ctypes.c_int(), ctypes.c_int()
    n = load().iwpp_synth_spiral_corridor(_ptr(mask), width, height, mask.strides[0], dtype, arm_pitch,
                                          ctypes.byref(sx), ctypes.byref(sy))
    marker = np.empty_like(mask)
    load().iwpp_synth_seed_marker(_ptr(marker), _ptr(mask), width, height, marker.strides[0], mask.strides[0], dtype,
                                  seed, nseeds, sx.value, sy.value)
    return marker, mask, int(n)


def uniform_pair(width: int, height: int, seed: int):
    """The reference generator's value law (testCaseGenerator.cu:28-35), uint8."""
    marker = np.empty((height, width), np.uint8)
    mask = np.empty((height, width), np.uint8)
    load().iwpp_synth_uniform_pair(_ptr(marker), _ptr(mask), width, height, marker.strides[0], mask.strides[0], seed)
    return marker, mask


# ------------------------------------------------------------- configurations
def config0():
    mask = noise_mask(1024, 1024, U8, 0, 4.0, 200)
    return hdome_marker(mask, 40), mask


def config1_mask():
    return noise_mask(4096, 4096, U8, 1, 8.0, 2000)


def config1(h: int, mask: Optional[np.ndarray] = None):
    if mask is None:
        mask = config1_mask()
    return hdome_marker(mask, h), mask


CONFIG1_CASES = [(conn, h) for conn in (4, 8) for h in (10, 40, 100)]


def config2(dtype: int, size: int = 16384):
    return spiral_case(size, size, dtype)


@dataclass
class ImageSpec:
    index: int
    width: int
    height: int
    dtype: int
    conn: int
    marker_kind: str  # "hdome" | "sparse"
    h8: int
    seed: int

    @property
    def pixels(self) -> int:
        return self.width * self.height

    @property
    def bpp(self) -> int:
        return {U8: 1, U16: 2, I32: 4}[self.dtype]


def _loguniform_int(r: random.Random, lo: int, hi: int) -> int:
    return int(round(math.exp(math.log(lo) + r.random() * (math.log(hi) - math.log(lo)))))


def config3_specs(n: int = 64, seed: int = 3):
    r = random.Random(seed)
    specs = []
    for i in range(n):
        w = _loguniform_int(r, 512, 4096)
        h = _loguniform_int(r, 512, 3072)
        dt = U8 if r.random() < 0.5 else U16
        conn = 4 if r.random() < 0.5 else 8
        h8 = 5 + int(r.random() * 116)
        specs.append(ImageSpec(i, w, h, dt, conn, "hdome", h8, seed * 1000 + i))
    return specs


def config4_stream(n_requests: int = 4000, pool: int = 128, seed: int = 4, rate: float = 2000.0):
    """(arrival_times_s, request -> spec index, specs).  Requests draw their
    image from a pool of `pool` distinct specs, each with its own seed
    (synthesising and checking thousands of multi-megapixel images per run
    is out of reach on the host: 128 take about half a minute)."""
    r = random.Random(seed)
    specs = []
    for i in range(pool):
        w = _loguniform_int(r, 256, 8192)
        h = _loguniform_int(r, 256, 8192)
        dt = U8 if r.random() < 0.8 else U16
        kind = "hdome" if r.random() < 0.5 else "sparse"
        h8 = 5 + int(r.random() * 116)
        specs.append(ImageSpec(i, w, h, dt, 8, kind, h8, seed * 1000 + i))
    t = 0.0
    times, which = [], []
    for _ in range(n_requests):
        t += -math.log(1.0 - r.random()) / rate
        times.append(t)
        which.append(int(r.random() * pool))
    return times, which, specs


def spec_images(spec: ImageSpec, nthreads: int = 0):
    area = spec.width * spec.height
    ndiscs = max(1, int(round(2000 * area / (4096 * 4096))))
    mask = noise_mask(spec.width, spec.height, spec.dtype, spec.seed, 4.0, ndiscs, nthreads=nthreads)
    if spec.marker_kind == "sparse":
        marker = sparse_marker(mask, spec.seed, 1e-4)
    else:
        marker = hdome_marker(mask, spec.h8)
    return marker, mask
