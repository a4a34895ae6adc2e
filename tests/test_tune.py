"""The autotuner and its tuning table (iwpp_autotune, iwpp_tune_*).

CPU: the table's text form round-trips, a malformed file changes nothing,
lookups resolve the workload class.  GPU: autotuning returns a valid
configuration and leaves the markers reconstructed bit-exactly; a table
entry steers calls made with default configuration fields."""
import ctypes
import os

import numpy as np
import pytest

import iwpp
import oracle
from iwpp import synth


def _write(path, lines):
    with open(path, "w") as f:
        f.write("# test table\n")
        for line in lines:
            f.write(line + "\n")


def test_table_round_trip(tmp_path):
    iwpp.tune_clear()
    assert iwpp.tune_entries() == 0
    p = tmp_path / "t.txt"
    # variant dtype conn pxclass batch tile_rows solver init_passes queue_mult [front_passes]
    # (a v1 line without the last field, a v2 line with it)
    # (the last field: 0 no front stage, 1 always, 2 decided on the device,
    # 3 the seed check alone)
    _write(p, ["3 0 8 24 0 32 1 0 0", "0 1 4 20 1 64 2 1 16 1", "2 0 8 28 0 64 0 4 0 2"])
    iwpp.tune_load(str(p))
    assert iwpp.tune_entries() == 3
    assert iwpp.tune_lookup("unique", 0, 8, 16384 * 16384) == {"tile_rows": 64, "solver": 0, "init_passes": 4,
                                                                 "front_passes": 3, "queue_capacity": 0}
    # 4096 x 4096 = 2^24 pixels: class 24
    assert iwpp.tune_lookup("async", 0, 8, 4096 * 4096) == {"tile_rows": 32, "solver": 1, "init_passes": 0,
                                                          "front_passes": 2, "queue_capacity": 0}
    assert iwpp.tune_lookup("async", 0, 8, 4096 * 4096 - 1) is None  # class 23
    assert iwpp.tune_lookup("async", 0, 8, 4096 * 4096, batch=True) is None
    e = iwpp.tune_lookup("mutex", 1, 4, 1 << 20, batch=True)
    assert e == {"tile_rows": 64, "solver": 2, "init_passes": 1, "front_passes": 1, "queue_capacity": -16}
    q = tmp_path / "u.txt"
    iwpp.tune_save(str(q))
    lines = [ln.split() for ln in open(q) if not ln.startswith("#")]
    assert sorted(lines) == sorted([["0", "1", "4", "20", "1", "64", "2", "1", "16", "1"],
                                    ["3", "0", "8", "24", "0", "32", "1", "0", "0", "0"],
                                    ["2", "0", "8", "28", "0", "64", "0", "4", "0", "2"]])
    iwpp.tune_clear()
    assert iwpp.tune_entries() == 0


def test_malformed_table_changes_nothing(tmp_path):
    iwpp.tune_clear()
    good = tmp_path / "good.txt"
    _write(good, ["3 0 8 24 0 64 0 0 0"])
    iwpp.tune_load(str(good))
    for bad_line in ["3 0 8 24 0 48 0 0 0", "3 0 8 24 0 64 7 0 0", "3 0 8", "x y z", "3 0 8 24 0 64 0 0 0 4",
                     "3 0 8 24 0 64 0 0 0 1 9"]:
        bad = tmp_path / "bad.txt"
        _write(bad, ["3 1 8 20 0 32 1 0 0", bad_line])
        with pytest.raises(iwpp.IwppError):
            iwpp.tune_load(str(bad))
        assert iwpp.tune_entries() == 1
    with pytest.raises(iwpp.IwppError):
        iwpp.tune_load(str(tmp_path / "missing.txt"))
    iwpp.tune_clear()


def test_autotune_rejects_bad_arguments():
    lib = iwpp.load()
    res = iwpp.TuneResult()
    assert lib.iwpp_autotune(None, None, 0, -1, 0, None, ctypes.byref(res)) == 1
    img = (iwpp.Image * 1)()
    img[0] = iwpp.Image(16, 16, 64, 64, 64, 64, 0, 6)  # bad connectivity
    assert lib.iwpp_autotune(ctypes.c_void_p(1), img, 1, -1, 0, None, ctypes.byref(res)) == 1


def _dev(a):
    import torch
    return torch.from_numpy(a.view(np.int16) if a.dtype == np.uint16 else a).cuda()


def _host(t, dtype):
    a = t.cpu().numpy()
    return a.view(np.uint16) if dtype == np.uint16 else a


@pytest.mark.gpu
def test_default_tile_height_follows_the_tile_count():
    iwpp.tune_clear()
    # 88 tiles of 64 rows: fewer than the device keeps warps resident
    assert iwpp.tile_count(1000, 700, 0, 0) == iwpp.tile_count(1000, 700, 0, 32)
    # 65536 tiles of 64 rows: more than 2.5 per warp any device keeps resident
    assert iwpp.tile_count(32768, 16384, 0, 0) == iwpp.tile_count(32768, 16384, 0, 64)


@pytest.mark.gpu
def test_table_entry_steers_default_calls(tmp_path):
    iwpp.tune_clear()
    mask = synth.noise_mask(1000, 700, 0, 31, 3.0, 5)
    marker = synth.hdome_marker(mask, 25)
    ref = oracle.reconstruct(marker, mask, 8)
    t64 = iwpp.tile_count(1000, 700, 0, 64)
    t32 = iwpp.tile_count(1000, 700, 0, 32)
    m, k = _dev(marker), _dev(mask)
    st = iwpp.reconstruct(m, k, connectivity=8, variant="async")
    assert st.tiles == t32 and np.array_equal(_host(m, marker.dtype), ref)
    cls = (1000 * 700).bit_length() - 1
    p = tmp_path / "t.txt"
    _write(p, [f"3 0 8 {cls} 0 64 2 1 0"])
    iwpp.tune_load(str(p))
    m, k = _dev(marker), _dev(mask)
    st = iwpp.reconstruct(m, k, connectivity=8, variant="async")
    assert st.tiles == t64 and np.array_equal(_host(m, marker.dtype), ref)
    # explicit fields win over the table
    m, k = _dev(marker), _dev(mask)
    st = iwpp.reconstruct(m, k, connectivity=8, variant="async", config=iwpp.Config.make(tile_rows=32))
    assert st.tiles == t32 and np.array_equal(_host(m, marker.dtype), ref)
    iwpp.tune_clear()


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["async", "mutex"])
def test_autotune_single_image(variant):
    iwpp.tune_clear()
    mask = synth.noise_mask(1500, 1100, 1, 32, 4.0, 9)
    marker = synth.sparse_marker(mask, 33, 0.001)
    ref = oracle.reconstruct(marker, mask, 8)
    m, k = _dev(marker), _dev(mask)
    res = iwpp.autotune([(m, k, 8)], variant=variant, repeats=1)
    assert np.array_equal(_host(m, marker.dtype), ref)
    assert res["tile_rows"] in (32, 64) and res["solver"] in (0, 1, 2) and 0 <= res["init_passes"] <= 64
    assert res["candidates"] >= 6 and res["best_ms"] > 0 and res["default_ms"] >= res["best_ms"]
    assert iwpp.tune_entries() == 1
    got = iwpp.tune_lookup(variant, 1, 8, 1500 * 1100)
    assert got["tile_rows"] == res["tile_rows"] and got["solver"] == res["solver"]
    # a default call now runs with the tuned configuration, same bytes
    m2 = _dev(marker)
    iwpp.reconstruct(m2, k, connectivity=8, variant=variant)
    assert np.array_equal(_host(m2, marker.dtype), ref)
    iwpp.tune_clear()


@pytest.mark.gpu
def test_autotune_batch_records_a_batch_class():
    iwpp.tune_clear()
    pairs, refs = [], []
    for i, (w, h, dt, conn) in enumerate([(300, 200, 0, 8), (517, 333, 1, 4), (128, 900, 0, 4)]):
        mask = synth.noise_mask(w, h, dt, 60 + i, 2.0, 3)
        marker = synth.hdome_marker(mask, 15 + 10 * i)
        refs.append(oracle.reconstruct(marker, mask, conn))
        pairs.append((_dev(marker), _dev(mask), conn, marker.dtype))
    iwpp.autotune([(m, k, c) for m, k, c, _ in pairs], repeats=1)
    for (m, _, _, dt), ref in zip(pairs, refs):
        assert np.array_equal(_host(m, dt), ref)
    assert iwpp.tune_entries() == 1
    total = 300 * 200 + 517 * 333 + 128 * 900
    assert iwpp.tune_lookup("default", -1, -1, total, batch=True) is not None
    iwpp.tune_clear()
