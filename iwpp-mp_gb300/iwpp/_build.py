"""In-tree build of the native libraries (no setuptools, no cmake).

* ``libiwpp.so``        -- CUDA kernels + C ABI (``include/iwpp.h``), sm_103a only.
* ``libiwpp_synth.so``  -- deterministic synthetic inputs (host C).
* ``iwpp_cli``          -- command-line front end with the reference's
  arguments (PGM / TIFF / raw I/O), linked against ``libiwpp.so``.

Object files are compiled in parallel; a library is rebuilt when any of its
sources is newer than it.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
SRC_DIR = os.path.join(os.path.dirname(PKG_DIR), "csrc")
REPO_DIR = os.path.dirname(os.path.dirname(PKG_DIR))
INCLUDE_DIR = os.path.join(REPO_DIR, "include")
LIB_DIR = os.path.join(PKG_DIR, "lib")

CUDA_SOURCES = ["iwpp_engine.cu", "iwpp_sweeps.cu", "iwpp_top.cu", "iwpp_api.cu", "iwpp_noalloc.cu",
                "iwpp_server.cu", "iwpp_tune.cu"]
CUDA_HEADERS = ["iwpp_device.cuh", "iwpp_engine.cuh", "iwpp_top.cuh", "iwpp_tune.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
                     "-I" + INCLUDE_DIR]

LIBIWPP = os.path.join(LIB_DIR, "libiwpp.so")
LIBSYNTH = os.path.join(LIB_DIR, "libiwpp_synth.so")
CLI = os.path.join(LIB_DIR, "iwpp_cli")


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout)


def build_iwpp(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(os.path.join(LIB_DIR, "obj"), exist_ok=True)
    srcs = [os.path.join(SRC_DIR, s) for s in CUDA_SOURCES]
    hdrs = [os.path.join(SRC_DIR, h) for h in CUDA_HEADERS] + [os.path.join(INCLUDE_DIR, "iwpp.h")]
    objs = [os.path.join(LIB_DIR, "obj", os.path.splitext(s)[0] + ".o") for s in CUDA_SOURCES]
    nvcc = _nvcc()
    jobs = []
    for src, obj in zip(srcs, objs):
        if force or _stale(obj, [src] + hdrs):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj])
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for _ in ex.map(_run, jobs):
                pass
    if force or _stale(LIBIWPP, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIBIWPP] + objs + ["-Xlinker", "--exclude-libs,ALL"])
    if verbose:
        print("built", LIBIWPP, file=sys.stderr)
    return LIBIWPP


def build_synth(force: bool = False) -> str:
    os.makedirs(LIB_DIR, exist_ok=True)
    src = os.path.join(SRC_DIR, "iwpp_synth.c")
    hdr = os.path.join(SRC_DIR, "iwpp_synth.h")
    if force or _stale(LIBSYNTH, [src, hdr]):
        cc = os.environ.get("CC", "gcc")
        # -ffp-contract=off: identical roundings on x86-64 and AArch64
        _run([cc, "-O2", "-std=gnu11", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-o", LIBSYNTH, src,
              "-lm"])
    return LIBSYNTH


def build_cli(force: bool = False) -> str:
    """Needs libiwpp.so; found next to the executable at run time."""
    src = os.path.join(SRC_DIR, "iwpp_cli.cpp")
    if force or _stale(CLI, [src, LIBIWPP, os.path.join(INCLUDE_DIR, "iwpp.h")]):
        _run([_nvcc(), "-O2", "-std=c++17", "-I" + INCLUDE_DIR, "-o", CLI, src, "-L" + LIB_DIR, "-liwpp",
              "-Xlinker", "-rpath,$ORIGIN"])
    return CLI


def build_all(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_iwpp, force)
        f2 = ex.submit(build_synth, force)
        f1.result()
        f2.result()
    build_cli(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
