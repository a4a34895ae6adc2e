"""The entry point that allocates nothing (iwpp_reconstruct_noalloc).

It exists for callers that cannot call cudaMalloc where they reconstruct --
a framework whose caching allocator owns the device memory, or a loop that
cannot afford cudaMalloc's device-wide synchronisation.  Its output must be
byte-identical to the allocating entry point's (reconstruction is exact),
on repeated calls that reuse the shared static scratch, and images beyond
the scratch must be refused with a clear status.  This file is collected last
so that a failure here never hides the other tests.
"""
import ctypes

import numpy as np
import pytest

import iwpp
from iwpp import synth

pytestmark = pytest.mark.gpu

CASES = [(0, 8, 1000, 700), (0, 4, 513, 257), (1, 8, 640, 480), (2, 8, 300, 200), (2, 4, 97, 61)]


def _dev(a):
    """A pitched device copy (rows padded to 128 bytes, as cudaMallocPitch
    would), returned as a 2-D view of the image columns."""
    import torch
    h, w = a.shape
    elems = -(-(w * a.itemsize) // 128) * 128 // a.itemsize
    host = a.view(np.int16) if a.dtype == np.uint16 else a
    buf = torch.zeros((h, elems), dtype=torch.from_numpy(host[:1, :1].copy()).dtype, device="cuda")
    buf[:, :w] = torch.from_numpy(np.ascontiguousarray(host)).cuda()
    return buf[:, :w]


def _host(t, dtype):
    a = t.cpu().numpy()
    return a.view(np.uint16) if dtype == np.uint16 else a


def _pitch(t):
    return t.stride(0) * t.element_size()


def test_noalloc_matches_allocating_entry_point_on_two_calls():
    import torch
    lib = iwpp.load()
    for call in range(2):
        for i, (dt, conn, w, h) in enumerate(CASES):
            mask = synth.noise_mask(w, h, dt, 900 + 10 * i + call, 3.0, 8)
            marker = synth.hdome_marker(mask, 35) if i % 2 == 0 else synth.sparse_marker(mask, 3 + i, 0.002)
            k = _dev(mask)
            ref = _dev(marker)
            st = iwpp.Stats()
            rc = lib.iwpp_reconstruct(None, ref.data_ptr(), k.data_ptr(), _pitch(ref), _pitch(k), w, h, dt, conn,
                                      iwpp.DEFAULT, None, None, ctypes.byref(st))
            assert rc == 0
            out = _dev(marker)
            torch.cuda.synchronize()
            rc = lib.iwpp_reconstruct_noalloc(out.data_ptr(), k.data_ptr(), _pitch(out), _pitch(k), w, h, dt, conn,
                                              None)
            assert rc == 0, iwpp.status_string(rc)
            assert np.array_equal(_host(out, marker.dtype), _host(ref, marker.dtype)), (call, dt, conn, w, h)


def test_noalloc_allocates_nothing_and_runs_on_a_side_stream():
    # A warm call (the device set-up is done) must leave the device's free
    # memory as it was: no cudaMalloc, no pool growth, no library workspace.
    # It runs on a non-default stream the caller owns.
    import torch
    lib = iwpp.load()
    dt, conn, w, h = CASES[0]
    mask = synth.noise_mask(w, h, dt, 977, 3.0, 8)
    marker = synth.hdome_marker(mask, 35)
    k = _dev(mask)
    ref = _dev(marker)
    assert lib.iwpp_reconstruct(None, ref.data_ptr(), k.data_ptr(), _pitch(ref), _pitch(k), w, h, dt, conn,
                                iwpp.DEFAULT, None, None, None) == 0
    outs = [_dev(marker) for _ in range(2)]
    side = torch.cuda.Stream()
    torch.cuda.synchronize()
    rc = lib.iwpp_reconstruct_noalloc(outs[0].data_ptr(), k.data_ptr(), _pitch(outs[0]), _pitch(k), w, h, dt, conn,
                                      ctypes.c_void_p(side.cuda_stream))
    assert rc == 0, iwpp.status_string(rc)
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    rc = lib.iwpp_reconstruct_noalloc(outs[1].data_ptr(), k.data_ptr(), _pitch(outs[1]), _pitch(k), w, h, dt, conn,
                                      ctypes.c_void_p(side.cuda_stream))
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert rc == 0, iwpp.status_string(rc)
    assert free_after >= free_before, free_before - free_after
    for o in outs:
        assert np.array_equal(_host(o, marker.dtype), _host(ref, marker.dtype))


# Scratch layout of one call (iwpp_noalloc.cu): counters and the image
# descriptor in the first 512 bytes, one state word per tile, then a ring of
# two entries per tile, each part 256-byte aligned -- at most 767 + 12 bytes
# per tile, at least 512 + 12.
_SCRATCH = 4 << 20
_TILES_FIT = (_SCRATCH - 767) // 12      # certainly fits
_TILES_OVER = (_SCRATCH - 512) // 12 + 1  # certainly does not


def test_noalloc_largest_image_that_fits_and_one_tile_row_more_than_that():
    # A 4-pixel-wide uint8 image has one 128 x 64 tile per 64 rows, so the
    # tile count sits right at the scratch bound with little memory (89 MB
    # per plane).  Content is generated on the device: random noise and an
    # h-dome marker (h = 40).
    import torch
    lib = iwpp.load()
    w = 4
    h = 64 * _TILES_FIT
    g = torch.Generator(device="cuda")
    g.manual_seed(1234)
    mask = torch.randint(0, 256, (h, w), dtype=torch.uint8, device="cuda", generator=g)
    marker = (mask.to(torch.int16) - 40).clamp_(min=0).to(torch.uint8)
    ref = marker.clone()
    out = marker.clone()
    assert lib.iwpp_reconstruct(None, ref.data_ptr(), mask.data_ptr(), w, w, w, h, 0, 8, iwpp.DEFAULT, None, None,
                                None) == 0
    torch.cuda.synchronize()
    rc = lib.iwpp_reconstruct_noalloc(out.data_ptr(), mask.data_ptr(), w, w, w, h, 0, 8, None)
    assert rc == 0, iwpp.status_string(rc)
    assert torch.equal(out, ref)
    assert not torch.equal(out, marker)
    # the same width with enough rows to pass the bound is refused before the
    # (never dereferenced) pointers are touched
    rc = lib.iwpp_reconstruct_noalloc(256, 256, w, w, w, 64 * _TILES_OVER, 0, 8, None)
    assert rc == 8, iwpp.status_string(rc)


def test_noalloc_refuses_rows_that_need_a_staging_copy():
    lib = iwpp.load()
    # a 513-byte pitch does not keep rows 4-byte aligned; the allocating entry
    # point would stage a copy, this one has no memory to do so
    rc = lib.iwpp_reconstruct_noalloc(256, 1024, 513, 513, 513, 10, 0, 8, None)
    assert rc == 1


def test_noalloc_refuses_images_beyond_the_scratch():
    lib = iwpp.load()
    # 131072 x 65536 uint8 needs about a million tiles: refused before any
    # device memory is touched (the pointers are never dereferenced)
    rc = lib.iwpp_reconstruct_noalloc(256, 256, 131072, 131072, 131072, 65536, 0, 8, None)
    assert rc == 8
    assert "too large" in iwpp.status_string(rc)
