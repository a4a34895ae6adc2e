"""The C-ABI library: it loads, exports every symbol include/iwpp.h declares,
and its host-only functions behave (no GPU needed)."""
import ctypes
import os
import re
import subprocess

import pytest

import iwpp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "iwpp.h")


def _declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"IWPP_API\s+[\w\s\*]+?\b(\w+)\s*\(", text)))


def test_header_declarations_parsed():
    names = _declared()
    assert "iwpp_reconstruct" in names and "MorphologicalReconstruction" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    lib = iwpp.load()
    out = subprocess.run(["nm", "-D", "--defined-only", iwpp.library_path()], stdout=subprocess.PIPE, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    for name in _declared():
        assert name in exported, name
        getattr(lib, name)  # resolvable through ctypes too
    # the Python binding covers exactly the declared surface
    assert sorted(iwpp.exported_symbols()) == _declared()


def test_library_exports_nothing_else():
    out = subprocess.run(["nm", "-D", "--defined-only", iwpp.library_path()], stdout=subprocess.PIPE, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    ours = {n for n in exported if not n.startswith("_")}
    assert ours == set(_declared())


def test_status_strings_and_version():
    lib = iwpp.load()
    assert lib.iwpp_version() == 1
    assert lib.iwpp_status_string(0) == b"ok"
    assert b"timed out" in lib.iwpp_status_string(3)
    assert lib.iwpp_status_string(99) == b"unknown status"


def test_tile_counts():
    lib = iwpp.load()
    # tiles are 128 bytes wide: 128 uint8, 64 uint16, 32 int32 pixels
    assert lib.iwpp_tile_count(4096, 4096, 0, 64) == 32 * 64
    assert lib.iwpp_tile_count(4096, 4096, 1, 64) == 64 * 64
    assert lib.iwpp_tile_count(4096, 4096, 2, 32) == 128 * 128
    assert lib.iwpp_tile_count(129, 65, 0, 64) == 2 * 2
    assert lib.iwpp_tile_count(0, 10, 0, 64) == 0
    assert lib.iwpp_tile_count(10, 10, 7, 64) == -1


def test_default_tile_height_without_a_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("with a device the default follows its resident warps (tests/test_tune.py)")
    lib = iwpp.load()
    # no device to size the grid by: the default is 64 rows
    assert lib.iwpp_tile_count(4096, 4096, 0, 0) == lib.iwpp_tile_count(4096, 4096, 0, 64)
    assert lib.iwpp_tile_count(100, 100, 1, 0) == lib.iwpp_tile_count(100, 100, 1, 64)


def test_workspace_bytes_grow_with_tiles():
    lib = iwpp.load()
    a = lib.iwpp_workspace_bytes(1000, 2, 0)
    b = lib.iwpp_workspace_bytes(100000, 2, 0)
    assert 0 < a < b
    # the double queue keeps two buffers, the mutex stack one
    assert lib.iwpp_workspace_bytes(100000, 1, 0) > lib.iwpp_workspace_bytes(100000, 0, 0)


def test_invalid_arguments_rejected_before_any_device_work():
    lib = iwpp.load()
    st = iwpp.Stats()
    # bad connectivity, bad dtype, pitch too small, negative size
    assert lib.iwpp_reconstruct(None, 16, 16, 64, 64, 64, 64, 0, 6, 2, None, None, ctypes.byref(st)) == 1
    assert lib.iwpp_reconstruct(None, 16, 16, 64, 64, 64, 64, 9, 8, 2, None, None, ctypes.byref(st)) == 1
    assert lib.iwpp_reconstruct(None, 16, 16, 32, 64, 64, 64, 0, 8, 2, None, None, ctypes.byref(st)) == 1
    assert lib.iwpp_reconstruct(None, 16, 16, 64, 64, -1, 64, 0, 8, 2, None, None, ctypes.byref(st)) == 1
    assert lib.iwpp_reconstruct(None, None, None, 64, 64, 64, 64, 0, 8, 2, None, None, ctypes.byref(st)) == 1
    assert lib.iwpp_last_status() == 1


def test_no_device_reported_without_gpu():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    lib = iwpp.load()
    h = ctypes.c_void_p()
    assert lib.iwpp_handle_create(ctypes.byref(h), 0) == 6
    # a valid empty image needs no device at all
    st = iwpp.Stats()
    assert lib.iwpp_reconstruct(None, None, None, 0, 0, 0, 0, 0, 8, 2, None, None, ctypes.byref(st)) == 0


def test_server_host_side_checks():
    lib = iwpp.load()
    srv = ctypes.c_void_p()
    bad = iwpp.ServerConfig(lanes=-1)
    assert lib.iwpp_server_create(ctypes.byref(srv), 0, ctypes.byref(bad)) == 1
    bad = iwpp.ServerConfig(tile_rows=48)
    assert lib.iwpp_server_create(ctypes.byref(srv), 0, ctypes.byref(bad)) == 1
    assert lib.iwpp_server_create(None, 0, None) == 1
    t = ctypes.c_ulonglong()
    assert lib.iwpp_server_submit(None, 16, 16, 16, 64, 64, 64, 64, 64, 0, 8, ctypes.byref(t)) == 1
    assert lib.iwpp_server_wait(None, 1, 0, None) == 1
    assert lib.iwpp_server_stats_get(None, None) == 1
    assert lib.iwpp_server_destroy(None) == 0
    try:
        import torch
        if torch.cuda.is_available():
            return
    except ImportError:
        pass
    assert lib.iwpp_server_create(ctypes.byref(srv), 0, None) == 6


def test_selftest_and_checker_host_side():
    lib = iwpp.load()
    r = iwpp.QueueTestResult()
    assert lib.iwpp_queue_selftest(0, -1, 0, 2, ctypes.byref(r)) == 1
    assert lib.iwpp_queue_selftest(0, -1, 128, 99, ctypes.byref(r)) == 1
    n = ctypes.c_ulonglong()
    assert lib.iwpp_fixed_point_violations(16, 16, 64, 64, 64, 64, 0, 8, None, None) == 1
    assert lib.iwpp_fixed_point_violations(16, 16, 32, 64, 64, 64, 0, 8, None, ctypes.byref(n)) == 1
    assert lib.iwpp_fixed_point_violations(None, None, 0, 0, 0, 0, 0, 8, None, ctypes.byref(n)) == 0
    try:
        import torch
        if torch.cuda.is_available():
            return
    except ImportError:
        pass
    assert lib.iwpp_queue_selftest(0, -1, 128, 2, ctypes.byref(r)) == 6
