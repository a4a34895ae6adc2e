"""iwpp_cli: the reference's command line (marker mask output usePGMLoader)
with PGM / TIFF / raw I/O.  CPU: image format round trips through
--convert (no GPU).  GPU: reconstructions from files equal the oracle."""
import os
import subprocess

import numpy as np
import pytest

import iwpp
import oracle
from iwpp import _build, synth


@pytest.fixture(scope="module")
def cli():
    _build.build_all()
    return _build.CLI


def write_pgm(path, a, ascii_=False):
    h, w = a.shape
    maxv = 255 if a.dtype == np.uint8 else 65535
    with open(path, "wb") as f:
        f.write(f"P{'2' if ascii_ else '5'}\n# made by the test\n{w} {h}\n{maxv}\n".encode())
        if ascii_:
            f.write(" ".join(str(int(v)) for v in a.ravel()).encode() + b"\n")
        elif a.dtype == np.uint8:
            f.write(a.tobytes())
        else:
            f.write(a.astype(">u2").tobytes())


def run(cli, *args):
    return subprocess.run([cli, *map(str, args)], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                          timeout=300)


def read_raw(path, shape, dtype):
    return np.fromfile(path, dtype=dtype).reshape(shape)


@pytest.mark.parametrize("dtype,ascii_", [(np.uint8, False), (np.uint16, False), (np.uint8, True)])
def test_pgm_tiff_raw_round_trip(cli, tmp_path, dtype, ascii_):
    rng = np.random.default_rng(5)
    a = rng.integers(0, 256 if dtype == np.uint8 else 65536, size=(37, 53)).astype(dtype)
    write_pgm(tmp_path / "a.pgm", a, ascii_)
    assert run(cli, "--convert", tmp_path / "a.pgm", tmp_path / "a.tif").returncode == 0
    assert run(cli, "--convert", tmp_path / "a.tif", tmp_path / "a.raw").returncode == 0
    assert np.array_equal(read_raw(tmp_path / "a.raw", a.shape, dtype), a)
    assert run(cli, "--convert", tmp_path / "a.tif", tmp_path / "b.pgm").returncode == 0
    assert run(cli, "--convert", tmp_path / "b.pgm", tmp_path / "b.raw").returncode == 0
    assert np.array_equal(read_raw(tmp_path / "b.raw", a.shape, dtype), a)


def test_int32_raw_tiff_round_trip(cli, tmp_path):
    a = np.arange(-600, 600, dtype=np.int32).reshape(30, 40) * 1000003
    a.tofile(tmp_path / "a.raw")
    assert run(cli, "--convert", tmp_path / "a.raw", tmp_path / "a.tiff", "--raw", "40x30:i32").returncode == 0
    assert run(cli, "--convert", tmp_path / "a.tiff", tmp_path / "b.raw").returncode == 0
    assert np.array_equal(read_raw(tmp_path / "b.raw", a.shape, np.int32), a)
    # int32 does not fit a PGM
    assert run(cli, "--convert", tmp_path / "a.tiff", tmp_path / "c.pgm").returncode != 0


def test_malformed_inputs_are_refused(cli, tmp_path):
    (tmp_path / "bad.pgm").write_bytes(b"P5\n10 10\n255\nshort")
    assert run(cli, "--convert", tmp_path / "bad.pgm", tmp_path / "o.raw").returncode == 2
    (tmp_path / "bad2.pgm").write_bytes(b"P5\nx y\n255\n")
    assert run(cli, "--convert", tmp_path / "bad2.pgm", tmp_path / "o.raw").returncode == 2
    (tmp_path / "x.raw").write_bytes(b"\0" * 10)
    assert run(cli, "--convert", tmp_path / "x.raw", tmp_path / "o.pgm").returncode == 2  # no --raw
    assert run(cli).returncode == 1
    assert run(cli, "a", "b").returncode == 1


@pytest.mark.gpu
@pytest.mark.parametrize("conn", [4, 8])
def test_reconstruction_from_pgm_files(cli, tmp_path, conn):
    mask = synth.noise_mask(512, 512, synth.U8, 71, 3.0, 20)
    marker = synth.hdome_marker(mask, 30)
    write_pgm(tmp_path / "marker.pgm", marker)
    write_pgm(tmp_path / "mask.pgm", mask)
    r = run(cli, tmp_path / "marker.pgm", tmp_path / "mask.pgm", tmp_path / "out.pgm", 1, "--conn", conn)
    assert r.returncode == 0, r.stderr
    assert r.stdout.startswith("Tempo de execu")
    assert run(cli, "--convert", tmp_path / "out.pgm", tmp_path / "out.raw").returncode == 0
    out = read_raw(tmp_path / "out.raw", mask.shape, np.uint8)
    assert np.array_equal(out, oracle.reconstruct(oracle.clip(marker, mask), mask, conn))


@pytest.mark.gpu
def test_reconstruction_uint16_tiff_and_unclipped_marker(cli, tmp_path):
    mask = synth.noise_mask(300, 211, synth.U16, 72, 2.0, 5)
    marker = synth.sparse_marker(mask, 73, 0.002)
    marker = np.maximum(marker, (mask // 3).astype(np.uint16))
    marker[5, 5] = 65535  # above the mask: the clip lowers it
    write_pgm(tmp_path / "marker.pgm", marker)
    write_pgm(tmp_path / "mask.pgm", mask)
    r = run(cli, tmp_path / "marker.pgm", tmp_path / "mask.pgm", tmp_path / "out.tif", 0, "--conn", 8,
            "--variant", "unique", "--repeat", 3, "--init-passes", 2, "--solver", 2, "--tile-rows", 32)
    assert r.returncode == 0, r.stderr
    assert run(cli, "--convert", tmp_path / "out.tif", tmp_path / "out.raw").returncode == 0
    out = read_raw(tmp_path / "out.raw", mask.shape, np.uint16)
    assert np.array_equal(out, oracle.reconstruct(oracle.clip(marker, mask), mask, 8))
