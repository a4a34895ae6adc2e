"""The CPU oracle (test infrastructure): three schedules of the reference's
propagation rule must agree, and hand-computed known answers must hold."""
import numpy as np
import pytest

import oracle

DTYPES = [np.uint8, np.uint16, np.int32]


def _rand_case(rng, dt, h, w, respect_precondition):
    info = np.iinfo(dt)
    lo, hi = (0, 255) if dt == np.uint8 else (0, 4000) if dt == np.uint16 else (-4000, 4000)
    mask = rng.integers(lo, hi + 1, (h, w)).astype(dt)
    marker = rng.integers(lo, hi + 1, (h, w)).astype(dt)
    if respect_precondition:
        marker = np.minimum(marker, mask)
    if rng.random() < 0.3:
        marker = np.full((h, w), info.min, dt)
        marker[rng.integers(0, h), rng.integers(0, w)] = mask.max()
    return marker, mask


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("conn", [4, 8])
def test_schedules_agree(dt, conn):
    rng = np.random.default_rng(1234 + conn)
    for i in range(60):
        h, w = int(rng.integers(1, 30)), int(rng.integers(1, 30))
        marker, mask = _rand_case(rng, dt, h, w, respect_precondition=(i % 2 == 0))
        a = oracle.reconstruct(marker, mask, conn)
        b = oracle.reconstruct_sr(marker, mask, conn)
        c = oracle.reconstruct_jacobi(marker, mask, conn)
        assert np.array_equal(a, b) and np.array_equal(a, c), (i, h, w)


def test_diagonal_only_connection_4_vs_8():
    mask = np.array([[9, 0, 0], [0, 9, 0], [0, 0, 9]], np.uint8)
    marker = np.zeros_like(mask)
    marker[0, 0] = 9
    r4 = oracle.reconstruct(marker, mask, 4)
    r8 = oracle.reconstruct(marker, mask, 8)
    assert r4.tolist() == [[9, 0, 0], [0, 0, 0], [0, 0, 0]]
    assert r8.tolist() == [[9, 0, 0], [0, 9, 0], [0, 0, 9]]


def test_corridor_single_seed():
    # a one-pixel corridor of 200 with one seed propagates end to end, the
    # neighbours get min(200, mask) = mask, the rest keeps the marker
    mask = np.full((5, 12), 50, np.uint8)
    mask[2, :] = 200
    marker = np.zeros_like(mask)
    marker[2, 0] = 200
    r = oracle.reconstruct(marker, mask, 4)
    assert (r[2] == 200).all()
    assert (r[[1, 3]] == 50).all()
    assert (r[[0, 4]] == 50).all()


def test_plateau_capped_by_seed_value():
    mask = np.full((4, 4), 100, np.uint8)
    marker = np.zeros_like(mask)
    marker[0, 0] = 60
    r = oracle.reconstruct(marker, mask, 8)
    assert (r == 60).all()


def test_signed_negative_values_and_border():
    lo = np.iinfo(np.int32).min
    mask = np.array([[-5, -3, -9], [-7, -1, -2]], np.int32)
    marker = np.full_like(mask, lo)
    marker[1, 1] = -1
    r = oracle.reconstruct(marker, mask, 8)
    # every pixel is reached: result = min(-1, mask) = mask
    assert r.tolist() == mask.tolist()
    r4 = oracle.reconstruct(marker, mask, 4)
    # 4-conn: (0,0) is reached through (0,1) or (1,0), both adjacent to (1,1)
    assert r4.tolist() == mask.tolist()
    # zero padding would be wrong for int32: nothing outside raises anything
    marker2 = np.full_like(mask, lo)
    r2 = oracle.reconstruct(marker2, mask, 8)
    assert (r2 == lo).all()


def test_marker_above_mask_is_kept():
    # the reference rule never lowers a pixel (MR.cu:43-44); without the clip
    # a pixel above its mask stays and raises neighbours up to their mask
    mask = np.array([[10, 10, 10]], np.uint8)
    marker = np.array([[0, 50, 0]], np.uint8)
    r = oracle.reconstruct(marker, mask, 4)
    assert r.tolist() == [[10, 50, 10]]
    c = oracle.clip(marker, mask)
    assert c.tolist() == [[0, 10, 0]]


def test_empty_and_degenerate_shapes():
    for shape in [(1, 1), (1, 7), (7, 1)]:
        mask = np.arange(np.prod(shape), dtype=np.uint8).reshape(shape) + 10
        marker = np.zeros_like(mask)
        marker.flat[0] = 200
        r = oracle.reconstruct(marker, mask, 8)
        assert np.array_equal(r, oracle.reconstruct_jacobi(marker, mask, 8))
    e = np.zeros((0, 5), np.uint8)
    assert oracle.reconstruct(e, e, 4).shape == (0, 5)


def test_sweep_restatement_is_monotone_and_bounded():
    rng = np.random.default_rng(5)
    mask = rng.integers(0, 256, (40, 300)).astype(np.uint8)
    marker = np.minimum(rng.integers(0, 256, (40, 300)).astype(np.uint8), mask)
    full = oracle.reconstruct(marker, mask, 8)
    for d in range(4):
        s = oracle.sweep(marker, mask, d, 8)
        assert (s >= marker).all() and (s <= full).all()
