"""Runs the reference's own CUDA reconstruction -- TEST INFRASTRUCTURE ONLY.

Build recipe (what ``build_if_possible`` does):

* On a machine where the reference sources are present, its DQ and UQ
  variants are compiled unmodified, from the files where they lie, for
  sm_103a as relocatable device code and device-linked with the CUDA device
  runtime into one cubin per variant::

      nvcc -arch=sm_103a -rdc=true -dc -I "<variant>/include" <variant>/src/globalQueue.cu
      nvcc -arch=sm_103a -rdc=true -dc -I "<variant>/include" <variant>/src/MorphologicalReconstruction.cu
      nvcc -arch=sm_103a -dlink -cubin -o oracle/_ref/ref_<dq|uq>.cubin *.o -lcudadevrt

  (main.cu, which needs OpenCV, is not used.)  The cubins hold device code
  only, so they run on any host architecture.
* ``refrun_harness.cpp`` (driver API) is compiled for the machine it runs on
  into ``oracle/_ref/refrun_harness``.

The MP (mutex) variant is not run: its kernel spins without a bound on a
global mutex and updates its active-block counter both atomically and
non-atomically (IWPP MP/src/MorphologicalReconstruction.cu:213 vs
IWPP MP/src/globalQueue.cu:138, :143), which can leave the spin without an
exit.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import tempfile

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(ORACLE_DIR, "_ref")
# where the reference checkout lies: IWPP_REFERENCE_DIR, else the recipe's
# default location
REFERENCE = os.environ.get("IWPP_REFERENCE_DIR", "/root/reference")
VARIANT_DIRS = {"dq": "IWPP MP DQ", "uq": "IWPP MP UQ"}
HARNESS_SRC = os.path.join(ORACLE_DIR, "refrun_harness.cpp")
HARNESS_BIN = os.path.join(REF_OUT, "refrun_harness")


def cubin_path(variant: str) -> str:
    return os.path.join(REF_OUT, f"ref_{variant}.cubin")


def _nvcc() -> str:
    return "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc"


def _run(cmd, cwd=None):
    res = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + res.stdout)


def build_cubins() -> bool:
    """Compiles the reference kernels (needs the reference sources)."""
    if not os.path.isdir(REFERENCE):
        return False
    os.makedirs(REF_OUT, exist_ok=True)
    for variant, d in VARIANT_DIRS.items():
        out = cubin_path(variant)
        src_dir = os.path.join(REFERENCE, d)
        srcs = [os.path.join(src_dir, "src", "globalQueue.cu"),
                os.path.join(src_dir, "src", "MorphologicalReconstruction.cu")]
        if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs):
            continue
        with tempfile.TemporaryDirectory() as tmp:
            objs = []
            for s in srcs:
                o = os.path.join(tmp, os.path.basename(s) + ".o")
                _run([_nvcc(), "-arch=sm_103a", "-rdc=true", "-dc", "-w", "-I", os.path.join(src_dir, "include"),
                      "-o", o, s])
                objs.append(o)
            _run([_nvcc(), "-arch=sm_103a", "-dlink", "-cubin", "-o", out] + objs + ["-lcudadevrt"])
    return True


def build_harness() -> bool:
    os.makedirs(REF_OUT, exist_ok=True)
    if os.path.exists(HARNESS_BIN) and os.path.getmtime(HARNESS_BIN) >= os.path.getmtime(HARNESS_SRC):
        # a binary left by another architecture is rebuilt
        try:
            subprocess.run([HARNESS_BIN], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, timeout=10)
            return True
        except OSError:
            pass
    cxx = os.environ.get("CXX", "g++")
    _run([cxx, "-O2", "-std=c++17", "-I/usr/local/cuda/include", "-o", HARNESS_BIN, HARNESS_SRC,
          "-L/usr/local/cuda/lib64", "-L/usr/local/cuda/lib64/stubs", "-lcuda"])
    return True


def build_if_possible() -> bool:
    ok = build_cubins()
    try:
        build_harness()
    except RuntimeError:
        return False
    return ok


def available() -> bool:
    return all(os.path.exists(cubin_path(v)) for v in VARIANT_DIRS) and os.path.exists(HARNESS_SRC)


def run(variant: str, marker: np.ndarray, mask: np.ndarray, timeout: int = 600):
    """The reference's result for a square uint8 pair (side a multiple of
    512): clipImage, then the variant's MorphologicalReconstruction.
    Returns (result, info dict)."""
    if marker.dtype != np.uint8 or marker.shape != mask.shape or marker.shape[0] != marker.shape[1]:
        raise ValueError("the reference handles square uint8 images only")
    size = marker.shape[0]
    if size % 512:
        raise ValueError("the reference needs a side that is a multiple of 512")
    build_harness()
    with tempfile.TemporaryDirectory() as tmp:
        fm, fk, fo = (os.path.join(tmp, n) for n in ("marker.raw", "mask.raw", "out.raw"))
        np.ascontiguousarray(marker).tofile(fm)
        np.ascontiguousarray(mask).tofile(fk)
        res = subprocess.run([HARNESS_BIN, cubin_path(variant), variant, str(size), fm, fk, fo],
                             stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=timeout)
        if res.returncode != 0:
            raise RuntimeError(f"reference run failed ({res.returncode}): {res.stderr[-2000:]}")
        out = np.fromfile(fo, dtype=np.uint8).reshape(size, size)
        info = json.loads(res.stdout.strip().splitlines()[-1])
    return out, info
