"""The 16384 x 16384 spiral-corridor images (the worst case for propagation:
a one-pixel corridor of 1 048 194 pixels at the dtype maximum, threaded
through smoothed noise, seeded at its start) in uint8, uint16 and int32,
8-connectivity, at full size: the GPU result must equal the CPU oracle bit
for bit under every schedule the library offers for them -- the untuned
default, the fixed whole-image passes, and the front stage (top-level
labelling, passes, the engine from a seed check).  The oracle runs on host
threads while the GPU works.

int32 masks span the full signed range, so negative values next to the
image border exercise the "outside pixels do not exist" rule of the
reference (IWPP MP/src/MorphologicalReconstruction.cu:252-256), where a
zero-padded border would be wrong."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import iwpp
import oracle
from iwpp import synth

pytestmark = pytest.mark.gpu

SCHEDULES = {
    "default": None,
    "fixed_passes": lambda: iwpp.Config.make(init_passes=32, solver=2),
    "front_passes": lambda: iwpp.Config.make(front_passes=1),
}


def _dev(a):
    import torch
    return torch.from_numpy(a.view(np.int16) if a.dtype == np.uint16 else a).cuda()


def _host(t, dtype):
    a = t.cpu().numpy()
    return a.view(np.uint16) if dtype == np.uint16 else a


@pytest.fixture(scope="module")
def spirals():
    """(dtype, marker, mask, corridor pixels, oracle future) per pixel type;
    the three oracle runs overlap the GPU tests."""
    ex = ThreadPoolExecutor(max_workers=3)
    out = {}
    for dt in (synth.U8, synth.U16, synth.I32):
        marker, mask, n = synth.config2(dt)
        out[dt] = (marker, mask, n, ex.submit(oracle.reconstruct, marker, mask, 8))
    yield out
    ex.shutdown(wait=True)


@pytest.mark.parametrize("schedule", list(SCHEDULES))
@pytest.mark.parametrize("dt", [synth.U8, synth.U16, synth.I32])
def test_spiral_16384_bitexact(spirals, dt, schedule):
    import torch
    marker, mask, n_corridor, ref_future = spirals[dt]
    m0, k = _dev(marker), _dev(mask)
    m = m0.clone()
    make = SCHEDULES[schedule]
    st = iwpp.reconstruct(m, k, connectivity=8, config=make() if make else None)
    assert st.status == 0
    res = _host(m, marker.dtype)
    ref = ref_future.result()
    if not np.array_equal(res, ref):
        bad = np.argwhere(res != ref)
        raise AssertionError(f"{len(bad)} pixels differ from the oracle, first at {bad[0].tolist()}")
    # size-independent properties on top: a fixed point, idempotent, and the
    # corridor filled end to end
    assert iwpp.fixed_point_violations(m, k, 8) == 0
    again = m.clone()
    assert iwpp.reconstruct(again, k, connectivity=8).status == 0
    assert torch.equal(again, m)
    top = {synth.U8: 255, synth.U16: 65535, synth.I32: 2**31 - 1}[dt]
    assert int((res == top).sum()) >= n_corridor
