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
