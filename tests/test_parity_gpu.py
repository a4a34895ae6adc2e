"""GPU parity: every result of libiwpp.so (through the C ABI) must equal the
CPU oracle bit for bit, for all three queue variants, both connectivities,
all pixel types, ragged / unaligned / degenerate shapes and the restart path."""
import ctypes

import numpy as np
import pytest

import iwpp
import oracle
from iwpp import synth

pytestmark = pytest.mark.gpu

VARIANTS = ["mutex", "double", "unique", "async"]
NP = {0: np.uint8, 1: np.uint16, 2: np.int32}


def _torch():
    import torch
    return torch


def to_dev(a):
    torch = _torch()
    if a.dtype == np.uint16:
        return torch.from_numpy(a.view(np.int16)).cuda()
    return torch.from_numpy(a).cuda()


def from_dev(t, dtype):
    a = t.cpu().numpy()
    return a.view(np.uint16) if dtype == np.uint16 else a


def gpu_reconstruct(marker, mask, conn, variant="unique", config=None):
    m, k = to_dev(marker), to_dev(mask)
    stats = iwpp.reconstruct(m, k, connectivity=conn, variant=variant, config=config)
    return from_dev(m, marker.dtype), stats


@pytest.fixture(scope="module")
def cfg1():
    mask = synth.config1_mask()
    cases = {}
    for conn, h in synth.CONFIG1_CASES:
        marker = synth.hdome_marker(mask, h)
        cases[(conn, h)] = (marker, oracle.reconstruct(marker, mask, conn))
    return mask, cases


@pytest.mark.parametrize("variant", VARIANTS)
def test_config0(variant):
    marker, mask = synth.config0()
    ref = oracle.reconstruct(marker, mask, 8)
    out, stats = gpu_reconstruct(marker, mask, 8, variant)
    assert np.array_equal(out, ref)
    assert stats.status == 0 and stats.visits >= stats.tiles


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("case", synth.CONFIG1_CASES)
def test_config1(cfg1, variant, case):
    mask, cases = cfg1
    marker, ref = cases[case]
    out, stats = gpu_reconstruct(marker, mask, case[0], variant)
    assert np.array_equal(out, ref), int((out != ref).sum())


@pytest.mark.parametrize("dt", [0, 1, 2])
@pytest.mark.parametrize("conn", [4, 8])
@pytest.mark.parametrize("variant", VARIANTS)
def test_random_shapes(dt, conn, variant):
    rng = np.random.default_rng(100 * dt + conn + len(variant))
    npdt = NP[dt]
    shapes = [(1, 1), (1, 131), (131, 1), (3, 5), (37, 53), (64, 128), (65, 129), (200, 333), (513, 257)]
    for i, (h, w) in enumerate(shapes):
        mask = synth.noise_mask(w, h, dt, 50 + i, 2.0, 3)
        if i % 3 == 0:
            marker = synth.sparse_marker(mask, 7 + i, 0.01)
        else:
            marker = synth.hdome_marker(mask, int(rng.integers(5, 80)))
        ref = oracle.reconstruct(marker, mask, conn)
        out, _ = gpu_reconstruct(marker, mask, conn, variant)
        assert np.array_equal(out, ref), (h, w, int((out != ref).sum()))


@pytest.mark.parametrize("dt", [0, 1, 2])
@pytest.mark.parametrize("conn", [4, 8])
@pytest.mark.parametrize("variant", ["async", "unique"])
def test_pass_solver(dt, conn, variant):
    # solver 2: every visit by vertical / horizontal passes (packed-word
    # vertical chains, paired-row horizontal scans for uint8 / uint16), first
    # visits with every row dirty, revisits from the sides that rose; ragged
    # shapes (rows past the image inside a tile), both tile heights
    rng = np.random.default_rng(500 + 10 * dt + conn + len(variant))
    shapes = [(1, 1), (3, 5), (37, 53), (65, 129), (200, 333), (513, 257), (700, 1500)]
    for i, (h, w) in enumerate(shapes):
        mask = synth.noise_mask(w, h, dt, 90 + i, 2.0 + i, 3 + 2 * i)
        if i % 3 == 0:
            marker = synth.sparse_marker(mask, 27 + i, 0.002)
        else:
            marker = synth.hdome_marker(mask, int(rng.integers(5, 120)))
        ref = oracle.reconstruct(marker, mask, conn)
        for th in (32, 64):
            out, st = gpu_reconstruct(marker, mask, conn, variant, iwpp.Config.make(solver=2, tile_rows=th))
            assert st.status == 0
            assert np.array_equal(out, ref), (h, w, th, int((out != ref).sum()))


@pytest.mark.parametrize("dt", [0, 1, 2])
@pytest.mark.parametrize("conn", [4, 8])
@pytest.mark.parametrize("variant", VARIANTS)
def test_pixel_queue_solver(dt, conn, variant):
    # solver 3: revisits by the per-tile pixel queue (first visits by passes);
    # ragged shapes, both tile heights, h-dome and sparse markers, and the
    # configuration-1 images (many revisits, some past the queue's capacity,
    # which fall back to passes)
    rng = np.random.default_rng(300 + 10 * dt + conn + len(variant))
    shapes = [(1, 1), (3, 5), (37, 53), (65, 129), (200, 333), (513, 257), (700, 1500)]
    for i, (h, w) in enumerate(shapes):
        mask = synth.noise_mask(w, h, dt, 70 + i, 2.0 + i, 3 + 2 * i)
        if i % 3 == 0:
            marker = synth.sparse_marker(mask, 17 + i, 0.002)
        else:
            marker = synth.hdome_marker(mask, int(rng.integers(5, 120)))
        ref = oracle.reconstruct(marker, mask, conn)
        for th in (32, 64):
            out, st = gpu_reconstruct(marker, mask, conn, variant, iwpp.Config.make(solver=3, tile_rows=th))
            assert st.status == 0
            assert np.array_equal(out, ref), (h, w, th, int((out != ref).sum()))


@pytest.mark.parametrize("variant", VARIANTS)
def test_pixel_queue_solver_config1(cfg1, variant):
    mask, cases = cfg1
    for case in synth.CONFIG1_CASES:
        marker, ref = cases[case]
        out, st = gpu_reconstruct(marker, mask, case[0], variant, iwpp.Config.make(solver=3))
        assert st.status == 0
        assert np.array_equal(out, ref), (case, int((out != ref).sum()))


@pytest.mark.parametrize("plain", [0, 1])
@pytest.mark.parametrize("variant", VARIANTS)
def test_tma_and_plain_load_paths_agree(plain, variant):
    # 16-byte aligned images take the TMA box path unless plain loads are forced
    for dt in (0, 1, 2):
        mask = synth.noise_mask(1000, 333, dt, 60 + dt, 3.0, 10)
        marker = synth.hdome_marker(mask, 35)
        ref = oracle.reconstruct(marker, mask, 8)
        out, _ = gpu_reconstruct(marker, mask, 8, variant, iwpp.Config.make(plain_loads=plain))
        assert np.array_equal(out, ref), dt


@pytest.mark.parametrize("tile_rows", [32, 64])
def test_tile_rows_and_noise_without_precondition(tile_rows):
    # raw noise, marker above the mask at half of the pixels
    rng = np.random.default_rng(tile_rows)
    for dt in (0, 1, 2):
        npdt = NP[dt]
        info = np.iinfo(npdt)
        mask = rng.integers(info.min, info.max, (300, 700), dtype=np.int64).astype(npdt)
        marker = rng.integers(info.min, info.max, (300, 700), dtype=np.int64).astype(npdt)
        for conn in (4, 8):
            ref = oracle.reconstruct(marker, mask, conn)
            out, _ = gpu_reconstruct(marker, mask, conn, "unique", iwpp.Config.make(tile_rows=tile_rows))
            assert np.array_equal(out, ref), (dt, conn)


def test_spiral_small_all_types():
    for dt in (0, 1, 2):
        marker, mask, n = synth.spiral_case(1024, 1024, dt, sigma=8.0, arm_pitch=64, nseeds=8)
        ref = oracle.reconstruct(marker, mask, 8)
        for variant in VARIANTS:
            out, stats = gpu_reconstruct(marker, mask, 8, variant)
            assert np.array_equal(out, ref), (dt, variant)


def test_padded_pitch_and_views():
    torch = _torch()
    mask = synth.noise_mask(301, 97, 0, 3, 2.0, 4)
    marker = synth.hdome_marker(mask, 25)
    ref = oracle.reconstruct(marker, mask, 8)
    # pitched buffers (row stride 512 bytes), sentinel in the padding
    big_m = torch.full((97, 512), 77, dtype=torch.uint8, device="cuda")
    big_k = torch.full((97, 512), 78, dtype=torch.uint8, device="cuda")
    big_m[:, :301] = torch.from_numpy(marker).cuda()
    big_k[:, :301] = torch.from_numpy(mask).cuda()
    iwpp.reconstruct(big_m[:, :301], big_k[:, :301], connectivity=8)
    out = big_m.cpu().numpy()
    assert np.array_equal(out[:, :301], ref)
    assert (out[:, 301:] == 77).all(), "padding bytes must not be touched"
    # unaligned rows (offset 1 byte, odd pitch) go through aligned staging
    flat_m = torch.zeros(97 * 301 + 1, dtype=torch.uint8, device="cuda")
    flat_k = torch.zeros(97 * 301 + 1, dtype=torch.uint8, device="cuda")
    vm = flat_m[1:].view(97, 301)
    vk = flat_k[1:].view(97, 301)
    vm.copy_(torch.from_numpy(marker).cuda())
    vk.copy_(torch.from_numpy(mask).cuda())
    iwpp.reconstruct(vm, vk, connectivity=8)
    assert np.array_equal(vm.cpu().numpy(), ref)
    assert int(flat_m[0].item()) == 0


@pytest.mark.parametrize("variant,cap", [("double", 16), ("mutex", 1)])
def test_overflow_restarts_keep_result(variant, cap):
    # The mutex stack's capacity is at least the tile count (the first stack
    # holds every tile) and each CTA buffers the entries its warps insert,
    # so the global stack overflows only when buffers spill onto a stack
    # still holding most first entries: one CTA (two as a second try), whose
    # buffer fills with the duplicate inserts of the mutex form.
    marker, mask = synth.config0()
    ref = oracle.reconstruct(marker, mask, 8)
    restarts = 0
    for grid in ((0,) if variant == "double" else (1, 2)):
        cfg = iwpp.Config.make(queue_capacity=cap, max_restarts=100000, grid_ctas=grid)
        out, stats = gpu_reconstruct(marker, mask, 8, variant, cfg)
        assert np.array_equal(out, ref), grid
        restarts += stats.restarts
        if restarts:
            break
    assert restarts > 0


def test_overflow_restart_cap_reports_error():
    marker, mask = synth.config0()
    cfg = iwpp.Config.make(queue_capacity=1, max_restarts=1)
    m, k = to_dev(marker), to_dev(mask)
    st = iwpp.reconstruct(m, k, connectivity=8, variant="double", config=cfg, check=False)
    assert st.status == 5
    # the partial result is still a valid lower bound of the answer
    ref = oracle.reconstruct(marker, mask, 8)
    out = m.cpu().numpy()
    assert (out >= marker).all() and (out <= ref).all()


def test_reference_compatible_entry_point(monkeypatch):
    torch = _torch()
    size = 512
    mask = synth.noise_mask(size, size, 0, 11, 4.0, 20)
    marker = synth.hdome_marker(mask, 30)
    ref = oracle.reconstruct(marker, mask, 4)
    for env in ("mutex", "double", "unique", "async"):
        monkeypatch.setenv("IWPP_QUEUE_VARIANT", env)
        pitch = 1024  # like cudaMallocPitch
        bm = torch.zeros((size, pitch), dtype=torch.uint8, device="cuda")
        bk = torch.zeros((size, pitch), dtype=torch.uint8, device="cuda")
        bm[:, :size] = torch.from_numpy(marker).cuda()
        bk[:, :size] = torch.from_numpy(mask).cuda()
        iwpp.configureHeapSize()
        iwpp.clipImage(bm.data_ptr(), bk.data_ptr(), pitch, pitch, size)
        iwpp.MorphologicalReconstruction(bm.data_ptr(), bk.data_ptr(), pitch, pitch, size)
        assert np.array_equal(bm[:, :size].cpu().numpy(), ref), env


def test_clip_matches_oracle():
    torch = _torch()
    rng = np.random.default_rng(3)
    for dt in (0, 1, 2):
        info = np.iinfo(NP[dt])
        a = rng.integers(info.min, info.max, (77, 133), dtype=np.int64).astype(NP[dt])
        b = rng.integers(info.min, info.max, (77, 133), dtype=np.int64).astype(NP[dt])
        ta, tb = to_dev(a), to_dev(b)
        iwpp.clip(ta, tb)
        torch.cuda.synchronize()
        assert np.array_equal(from_dev(ta, NP[dt]), oracle.clip(a, b))


@pytest.mark.parametrize("dt", [0, 1, 2])
@pytest.mark.parametrize("conn", [4, 8])
def test_whole_image_sweeps_match_restatement(dt, conn):
    torch = _torch()
    mask = synth.noise_mask(333, 91, dt, 21, 3.0, 5)
    marker = synth.sparse_marker(mask, 5, 0.002)
    for d in range(4):
        tm, tk = to_dev(marker), to_dev(mask)
        iwpp.sweep(tm, tk, d, conn)
        torch.cuda.synchronize()
        assert np.array_equal(from_dev(tm, NP[dt]), oracle.sweep(marker, mask, d, conn)), d


@pytest.mark.parametrize("dt", [0, 1, 2])
@pytest.mark.parametrize("width", [333, 1000, 4099])
def test_horizontal_sweeps_of_16_byte_rows(dt, width):
    # rows starting on 16-byte boundaries take the 16-byte-lane horizontal
    # sweep; the row's last lane is partial.  The padding after each row holds
    # the type's largest value in both planes: a read past the row's end
    # would raise pixels the oracle leaves.
    torch = _torch()
    h = 37
    mask = synth.noise_mask(width, h, dt, 23, 3.0, 5)
    marker = synth.sparse_marker(mask, 7, 0.002)
    pw = (width + 15) // 16 * 16 + 16
    top = np.iinfo(NP[dt]).max
    for d in (0, 2):
        for conn in (4, 8):
            bm = np.full((h, pw), top, NP[dt])
            bk = np.full((h, pw), top, NP[dt])
            bm[:, :width] = marker
            bk[:, :width] = mask
            tm, tk = to_dev(bm), to_dev(bk)
            iwpp.sweep(tm[:, :width], tk[:, :width], d, conn)
            torch.cuda.synchronize()
            out = from_dev(tm, NP[dt])
            assert np.array_equal(out[:, :width], oracle.sweep(marker, mask, d, conn)), (d, conn)
            assert (out[:, width:] == top).all()


@pytest.mark.parametrize("dt", [0, 1, 2])
@pytest.mark.parametrize("shape", [(2500, 131), (4500, 64)])
def test_vertical_sweeps_of_tall_images(dt, shape):
    # more than two segments of rows: the segmented vertical sweep
    torch = _torch()
    h, w = shape
    mask = synth.noise_mask(w, h, dt, 22, 3.0, 5)
    marker = synth.sparse_marker(mask, 6, 0.001)
    for d in (1, 3):
        tm, tk = to_dev(marker), to_dev(mask)
        iwpp.sweep(tm, tk, d, 4)
        torch.cuda.synchronize()
        assert np.array_equal(from_dev(tm, NP[dt]), oracle.sweep(marker, mask, d, 4)), d


def test_sweep_timing_reports_four_passes():
    mask = synth.noise_mask(1024, 1024, 0, 1, 4.0, 50)
    marker = synth.hdome_marker(mask, 40)
    tm, tk = to_dev(marker), to_dev(mask)
    ms = iwpp.sweep_timing(tm, tk, 8)
    assert len(ms) == 4 and all(t > 0 for t in ms)


def test_batch_mixed_types_and_connectivity():
    specs = synth.config3_specs(8)
    pairs, refs = [], []
    for s in specs:
        w, h = s.width // 4, s.height // 4
        small = synth.ImageSpec(s.index, w, h, s.dtype, s.conn, s.marker_kind, s.h8, s.seed)
        marker, mask = synth.spec_images(small)
        refs.append(oracle.reconstruct(marker, mask, s.conn))
        pairs.append((to_dev(marker), to_dev(mask), s.conn, marker.dtype))
    for variant in VARIANTS:
        devs = [(to_dev(from_dev(p[0], p[3])), p[1], p[2]) for p in pairs]
        iwpp.reconstruct_batch(devs, variant=variant)
        for (m, _, _), p, ref in zip(devs, pairs, refs):
            assert np.array_equal(from_dev(m, p[3]), ref), variant


def test_graph_plan_relaunch():
    torch = _torch()
    h = iwpp.Handle(0)
    marker, mask = synth.config0()
    ref = oracle.reconstruct(marker, mask, 8)
    tm, tk = to_dev(marker), to_dev(mask)
    pristine = tm.clone()
    plan = iwpp.Plan(h, [(tm, tk, 8)], variant="unique")
    for _ in range(3):
        tm.copy_(pristine)
        plan.launch()
        st = plan.sync()
        assert st.status == 0
        assert np.array_equal(tm.cpu().numpy(), ref)
    plan.close()
    h.close()


@pytest.mark.parametrize("variant", VARIANTS)
def test_device_wait_timeout_is_reported_not_hung(variant):
    # The phantom-work hook makes the job count one unit of work that never
    # arrives (a queue entry nobody inserts; a CTA that never reaches the
    # round barrier), so every device-side wait must run out: the call comes
    # back with IWPP_ERR_TIMEOUT after the 200 ms bound instead of hanging,
    # and the kernel has returned.
    import time

    marker, mask = synth.config0()
    m, k = to_dev(marker), to_dev(mask)
    t0 = time.perf_counter()
    st = iwpp.reconstruct(m, k, connectivity=8, variant=variant,
                          config=iwpp.Config.make(timeout_ms=200, phantom_work=1), check=False)
    elapsed = time.perf_counter() - t0
    assert st.status == 3, st.status
    assert 0.19 < elapsed < 30.0
    # pixels are only ever raised, so whatever the run left is still a lower
    # bound of the reconstruction, never above it
    ref = oracle.reconstruct(marker, mask, 8)
    part = from_dev(m, marker.dtype)
    assert np.all(part <= ref) and np.all(part >= marker)
    # the library and the context stay usable afterwards
    out, st2 = gpu_reconstruct(marker, mask, 8, variant)
    assert st2.status == 0
    assert np.array_equal(out, ref)


def test_graph_plan_with_unaligned_images():
    # widths that leave rows unaligned: the plan stages them inside the graph
    h = iwpp.Handle(0)
    pairs, refs, pristine = [], [], []
    for i, (w, hh, dt, conn) in enumerate([(301, 97, 0, 8), (513, 200, 0, 4), (77, 61, 1, 8), (129, 33, 2, 4)]):
        mask = synth.noise_mask(w, hh, dt, 700 + i, 2.0, 3)
        marker = synth.hdome_marker(mask, 30)
        refs.append(oracle.reconstruct(marker, mask, conn))
        tm, tk = to_dev(marker), to_dev(mask)
        pristine.append(tm.clone())
        pairs.append((tm, tk, conn, marker.dtype))
    plan = iwpp.Plan(h, [(p[0], p[1], p[2]) for p in pairs])
    for _ in range(2):
        for p, q in zip(pairs, pristine):
            p[0].copy_(q)
        plan.launch()
        plan.sync()
        for p, ref in zip(pairs, refs):
            assert np.array_equal(from_dev(p[0], p[3]), ref)
    plan.close()
    h.close()
