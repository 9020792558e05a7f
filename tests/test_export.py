"""Image export and snapshots, host side: the oracle's conversions against the reference's own
(golden vectors from texture_save.cu's kernels), the engine's plate palette, the PNG encoder
(decoded with zlib, every chunk CRC checked) and snapshot file validation."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import master_thesis_gb300 as T
import oracle as O
from conftest import decode_png


def test_oracle_palette_matches_reference(golden):
    g = golden("ref_export")
    np.testing.assert_array_equal(O.plate_palette(), g["rgb"].reshape(256, 3))


def test_oracle_gray16_matches_reference(golden):
    g = golden("ref_export")
    np.testing.assert_array_equal(O.gray16(g["h1"], float(g["lo1"]), float(g["hi1"])), g["g1"])
    np.testing.assert_array_equal(O.gray16(g["h2"], float(g["lo2"]), float(g["hi2"])), g["g2"])


def test_engine_palette_matches_reference(golden):
    g = golden("ref_export")
    np.testing.assert_array_equal(T.plate_palette(), g["rgb"].reshape(256, 3))
    assert tuple(T.plate_palette()[255]) == (230, 235, 240)


@pytest.mark.parametrize("shape", [(1, 1), (3, 7), (64, 33), (200, 300)])
def test_png_gray16_round_trip(shape):
    rng = np.random.default_rng(shape[0] * 1000 + shape[1])
    img = rng.integers(0, 65536, shape, dtype=np.uint16)
    px, chunks = decode_png(T.png_encode(img, T.PNG_GRAY16))
    assert chunks == ["IHDR", "IDAT", "IEND"]
    np.testing.assert_array_equal(px, img)


@pytest.mark.parametrize("shape", [(1, 1), (5, 9), (150, 200)])  # 150 x 200 x 3: several stored blocks
def test_png_rgb8_round_trip(shape):
    rng = np.random.default_rng(shape[0] + shape[1])
    img = rng.integers(0, 256, shape + (3,), dtype=np.uint8)
    px, _ = decode_png(T.png_encode(img, T.PNG_RGB8))
    np.testing.assert_array_equal(px, img)


def test_png_gray8_round_trip():
    img = (np.arange(70 * 1000) % 251).astype(np.uint8).reshape(70, 1000)  # 70 KB: two stored blocks
    px, _ = decode_png(T.png_encode(img, T.PNG_GRAY8))
    np.testing.assert_array_equal(px, img)


def test_png_rejects_bad_arguments():
    with pytest.raises(ValueError):
        T.png_encode(np.zeros((4, 4), np.uint8), T.PNG_RGB8)
    L = T.lib()
    n = C.c_size_t(0)
    buf = np.zeros(16, np.uint8)
    assert L.tecto_png_encode(buf.ctypes.data, 0, 4, T.PNG_GRAY8, None, 0, C.byref(n)) != 0
    assert L.tecto_png_encode(buf.ctypes.data, 4, 4, 7, None, 0, C.byref(n)) != 0
    assert L.tecto_png_encode(None, 4, 4, T.PNG_GRAY8, None, 0, C.byref(n)) != 0
    # too small an output buffer
    assert L.tecto_png_encode(buf.ctypes.data, 4, 4, T.PNG_GRAY8, None, 0, C.byref(n)) == 0
    small = np.zeros(int(n.value) - 1, np.uint8)
    assert L.tecto_png_encode(buf.ctypes.data, 4, 4, T.PNG_GRAY8, small.ctypes.data, small.size,
                              C.byref(n)) != 0


def test_snapshot_info_rejects_other_files(tmp_path):
    p = tmp_path / "not_a_snapshot.bin"
    p.write_bytes(b"TECTOSN0" + bytes(200))
    with pytest.raises(T.TectoError):
        T.snapshot_info(p)
    with pytest.raises(T.TectoError):
        T.snapshot_info(tmp_path / "missing.bin")
