"""GPU: the queue self-test (the reference's fill / read-back check on this
library's queues) and the fixed-point checker, which carries parity to the
full 16384^2 configuration-2 images through size-independent properties:
the result is a fixed point of the propagation rule, lies between the
(clipped) marker and the mask, and reconstructing it again changes nothing."""
import numpy as np
import pytest

import iwpp
import oracle
from iwpp import synth

pytestmark = pytest.mark.gpu

VARIANTS = ["mutex", "double", "unique", "async"]


def _dev(a):
    import torch
    return torch.from_numpy(a.view(np.int16) if a.dtype == np.uint16 else a).cuda()


def _host(t, dtype):
    a = t.cpu().numpy()
    return a.view(np.uint16) if dtype == np.uint16 else a


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("side,copies", [(128, 2), (300, 3), (1, 1)])
def test_queue_selftest(variant, side, copies):
    r = iwpp.queue_selftest(variant, side, copies)
    assert r["status"] == 0
    assert r["mismatched"] == 0 and r["first_bad"] == -1, r
    assert r["entries"] == r["expected"]
    assert r["expected"] == side * side * (1 if variant == "unique" else copies)


@pytest.mark.parametrize("dt", [0, 1, 2])
@pytest.mark.parametrize("conn", [4, 8])
def test_fixed_point_checker(dt, conn):
    mask = synth.noise_mask(333, 257, dt, 90 + dt, 3.0, 6)
    marker = synth.hdome_marker(mask, 20)
    ref = oracle.reconstruct(marker, mask, conn)
    k = _dev(mask)
    assert iwpp.fixed_point_violations(_dev(ref), k, conn) == 0
    assert iwpp.fixed_point_violations(_dev(marker), k, conn) > 0
    # plant one defect: a pixel lowered below what its neighbours force
    bad = ref.copy()
    ys, xs = np.nonzero(ref > marker)
    y, x = int(ys[len(ys) // 2]), int(xs[len(xs) // 2])
    bad[y, x] = marker[y, x]
    assert iwpp.fixed_point_violations(_dev(bad), k, conn) == 1
