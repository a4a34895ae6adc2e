"""GPU parity of the front stage (iwpp_config.front_passes = 1): the pixels at
the mask's largest value raised by connected-component labelling, four
whole-image passes, then the seed check and the tile engine from the tiles
still violating a constraint.  Every
result must equal the CPU oracle bit for bit, for every pixel type,
connectivity and queue variant, on ragged and degenerate shapes, unclipped
markers, padded pitches, batches and graph plans."""
import os

import numpy as np
import pytest

import iwpp
import oracle
from iwpp import synth

pytestmark = pytest.mark.gpu

VARIANTS = ["mutex", "double", "unique", "async"]
NP = {0: np.uint8, 1: np.uint16, 2: np.int32}
FRONT = dict(front_passes=1)


def to_dev(a):
    import torch
    return torch.from_numpy(a.view(np.int16) if a.dtype == np.uint16 else a).cuda()


def from_dev(t, dtype):
    a = t.cpu().numpy()
    return a.view(np.uint16) if dtype == np.uint16 else a


def run(marker, mask, conn, variant="async", **cfg):
    m, k = to_dev(marker), to_dev(mask)
    st = iwpp.reconstruct(m, k, connectivity=conn, variant=variant, config=iwpp.Config.make(**{**FRONT, **cfg}))
    return from_dev(m, marker.dtype), st


@pytest.mark.parametrize("dt", [0, 1, 2])
@pytest.mark.parametrize("conn", [4, 8])
@pytest.mark.parametrize("variant", VARIANTS)
def test_front_random_shapes(dt, conn, variant):
    rng = np.random.default_rng(500 + 10 * dt + conn + len(variant))
    shapes = [(1, 1), (1, 131), (131, 1), (3, 5), (64, 128), (65, 129), (200, 333), (513, 257), (130, 1029)]
    decided_off = 0
    for i, (h, w) in enumerate(shapes):
        mask = synth.noise_mask(w, h, dt, 80 + i, 2.0, 3)
        marker = synth.sparse_marker(mask, 9 + i, 0.01) if i % 3 == 0 else \
            synth.hdome_marker(mask, int(rng.integers(5, 80)))
        ref = oracle.reconstruct(marker, mask, conn)
        out, st = run(marker, mask, conn, variant)
        assert st.status == 0
        assert np.array_equal(out, ref), (h, w, int((out != ref).sum()))
        # the top-level stage (6 kernels), two whole-image passes, the seed
        # check and the engine ran
        assert st.launches >= 6 + 8 + 3 and st.front_stage == 1
        # decided on the device: on images this small an initial front is
        # large against the tile count (or empty), so the stage is left out
        # and the engine starts from the first seed check's list
        out, st = run(marker, mask, conn, variant, front_passes=3)
        assert st.status == 0
        assert np.array_equal(out, ref), (h, w, "decided", int((out != ref).sum()))
        if st.front_stage == 0:
            assert st.top_pixels == 0
            decided_off += 1
        # the seed check alone: the engine starts from the tiles it lists
        out, st = run(marker, mask, conn, variant, front_passes=4)
        assert st.status == 0 and st.front_stage == 0 and st.top_pixels == 0
        assert np.array_equal(out, ref), (h, w, "seeded", int((out != ref).sum()))
    assert decided_off == len(shapes)


@pytest.mark.parametrize("variant", VARIANTS)
def test_front_spirals_and_config0(variant):
    for dt in (0, 1, 2):
        marker, mask, _ = synth.spiral_case(1024, 1024, dt, sigma=8.0, arm_pitch=32, nseeds=4)
        ref = oracle.reconstruct(marker, mask, 8)
        out, st = run(marker, mask, 8, variant)
        assert np.array_equal(out, ref), (dt, int((out != ref).sum()))
        # the corridor is carried by the stage: the engine only finishes
        # (alone it revisits the tiles along the corridor many times over)
        assert st.visits < 2 * st.tiles
    marker, mask = synth.config0()
    ref = oracle.reconstruct(marker, mask, 8)
    out, _ = run(marker, mask, 8, variant)
    assert np.array_equal(out, ref)


@pytest.mark.parametrize("dt", [0, 1, 2])
@pytest.mark.parametrize("conn", [4, 8])
def test_front_top_level_plateaus_and_corridors(dt, conn):
    # the top level as a dense plateau (labelling tiles with more top pixels
    # than their saved list holds are labelled again), as one-pixel
    # corridors crossing many tiles (tiles whose list is saved), and as
    # isolated pixels; a labelling tile with more components than node slots
    # (a checkerboard of single pixels) keeps the extra ones for the passes
    rng = np.random.default_rng(40 + dt * 2 + conn)
    info = np.iinfo(NP[dt])
    h, w = 700, 1500
    top = info.max
    mask = rng.integers(info.min // 2 if dt == 2 else 0, top // 2, (h, w), dtype=np.int64).astype(NP[dt])
    mask[100:260, 200:560] = top                                 # plateau
    mask[400, 10:1490] = top                                     # horizontal corridor
    mask[300:690, 1200] = top                                    # vertical corridor
    mask[400:690, 700] = top                                     # corridor meeting the first
    yy, xx = np.mgrid[0:64, 0:128]
    mask[512:576, 896:1024][((yy + xx) % 2 == 0)[:, :128]] = top  # checkerboard: > 64 components
    mask[5, 5] = top                                             # isolated
    marker = np.full((h, w), info.min if dt == 2 else 0, NP[dt])
    marker[150, 300] = top - 7
    marker[400, 1480] = top - 3
    marker[689, 700] = top - 1
    marker[520, 900] = top - 5
    marker[rng.integers(0, h, 50), rng.integers(0, w, 50)] = top // 3
    marker = np.minimum(marker, mask)
    ref = oracle.reconstruct(marker, mask, conn)
    for variant in ("unique", "async"):
        out, st = run(marker, mask, conn, variant)
        assert st.status == 0
        assert np.array_equal(out, ref), (variant, int((out != ref).sum()))
        assert st.top_pixels == int((mask == top).sum())


@pytest.mark.parametrize("variant", ["unique", "async"])
def test_front_decided_on_the_device_takes_the_stage_for_sparse_seeds(variant):
    # a 4096^2 spiral with four seeds: a handful of dirty tiles among 2048,
    # so the device takes the stage
    marker, mask, _ = synth.spiral_case(4096, 4096, 0, sigma=8.0, arm_pitch=64, nseeds=4)
    ref = oracle.reconstruct(marker, mask, 8)
    out, st = run(marker, mask, 8, variant, front_passes=3)
    assert st.status == 0 and st.front_stage == 1 and st.top_pixels > 0
    assert np.array_equal(out, ref), int((out != ref).sum())


def test_front_untuned_default_on_large_images():
    # 8192^2 (2^26 pixels): the untuned default decides on the device.  A
    # spiral with few seeds takes the stage, an h-dome image does not; both
    # results equal those of the stage forced on and forced off, and are
    # fixed points
    iwpp.tune_clear()
    nt = os.cpu_count() or 1
    spiral_m, spiral_k, _ = synth.spiral_case(8192, 8192, 0, sigma=16.0, arm_pitch=256, nseeds=16, nthreads=nt)
    hd_k = synth.noise_mask(8192, 8192, 0, 5, 8.0, 8000, nthreads=nt)
    hd_m = synth.hdome_marker(hd_k, 40)
    for (marker, mask), want in (((spiral_m, spiral_k), 1), ((hd_m, hd_k), 0)):
        m, k = to_dev(marker), to_dev(mask)
        st = iwpp.reconstruct(m, k, connectivity=8)
        assert st.status == 0 and st.front_stage == want
        assert iwpp.fixed_point_violations(m, k, 8) == 0
        got = m.cpu().numpy()
        for fp in (1, 2):
            out, st2 = run(marker, mask, 8, front_passes=fp)
            assert st2.front_stage == (1 if fp == 1 else 0)
            assert np.array_equal(out, got), (want, fp)


@pytest.mark.parametrize("tile_rows", [32, 64])
def test_front_unclipped_noise(tile_rows):
    # raw noise with the marker above the mask at half of the pixels (no
    # precondition), full value ranges (int32 negatives next to the border)
    rng = np.random.default_rng(7 + tile_rows)
    for dt in (0, 1, 2):
        info = np.iinfo(NP[dt])
        mask = rng.integers(info.min, info.max, (300, 700), dtype=np.int64).astype(NP[dt])
        marker = rng.integers(info.min, info.max, (300, 700), dtype=np.int64).astype(NP[dt])
        for conn in (4, 8):
            ref = oracle.reconstruct(marker, mask, conn)
            out, _ = run(marker, mask, conn, "async", tile_rows=tile_rows)
            assert np.array_equal(out, ref), (dt, conn)


def test_front_padded_pitch_and_unaligned_rows():
    import torch
    mask = synth.noise_mask(301, 197, 0, 3, 2.0, 4)
    marker = synth.hdome_marker(mask, 25)
    ref = oracle.reconstruct(marker, mask, 8)
    # a 512-byte pitch (rows on 16-byte boundaries: tiles staged by cp.async)
    # and a 308-byte pitch (4-byte aligned only: lane-word loads)
    for pitch in (512, 308):
        big_m = torch.full((197, pitch), 77, dtype=torch.uint8, device="cuda")
        big_k = torch.full((197, pitch), 99, dtype=torch.uint8, device="cuda")
        big_m[:, :301] = torch.from_numpy(marker).cuda()
        big_k[:, :301] = torch.from_numpy(mask).cuda()
        st = iwpp.reconstruct(big_m[:, :301], big_k[:, :301], connectivity=8, config=iwpp.Config.make(**FRONT))
        assert st.status == 0
        assert np.array_equal(big_m[:, :301].cpu().numpy(), ref), pitch
        assert bool((big_m[:, 301:] == 77).all())  # the padding is not touched


def test_front_batch_and_plan():
    specs = synth.config3_specs(6)
    pairs, refs, pristine = [], [], []
    for s in specs:
        small = synth.ImageSpec(s.index, s.width // 4, s.height // 4, s.dtype, s.conn, s.marker_kind, s.h8, s.seed)
        marker, mask = synth.spec_images(small)
        refs.append(oracle.reconstruct(marker, mask, s.conn))
        tm = to_dev(marker)
        pristine.append(tm.clone())
        pairs.append((tm, to_dev(mask), s.conn, marker.dtype))
    for variant in VARIANTS:
        for p, q in zip(pairs, pristine):
            p[0].copy_(q)
        st = iwpp.reconstruct_batch([(p[0], p[1], p[2]) for p in pairs], variant=variant,
                                    config=iwpp.Config.make(**FRONT))
        assert st.status == 0
        for p, ref in zip(pairs, refs):
            assert np.array_equal(from_dev(p[0], p[3]), ref), variant
    h = iwpp.Handle(0)
    plan = iwpp.Plan(h, [(p[0], p[1], p[2]) for p in pairs], config=iwpp.Config.make(**FRONT))
    for _ in range(2):
        for p, q in zip(pairs, pristine):
            p[0].copy_(q)
        plan.launch()
        assert plan.sync().status == 0
        for p, ref in zip(pairs, refs):
            assert np.array_equal(from_dev(p[0], p[3]), ref)
    plan.close()
    h.close()


def test_front_timeout_is_reported():
    # the phantom-work hook stalls the engine after the passes: the call must
    # come back with IWPP_ERR_TIMEOUT, the result a valid lower bound
    marker, mask = synth.config0()
    m, k = to_dev(marker), to_dev(mask)
    st = iwpp.reconstruct(m, k, connectivity=8, config=iwpp.Config.make(**FRONT, timeout_ms=200, phantom_work=1),
                          check=False)
    assert st.status == 3
    ref = oracle.reconstruct(marker, mask, 8)
    part = from_dev(m, marker.dtype)
    assert np.all(part <= ref) and np.all(part >= marker)
