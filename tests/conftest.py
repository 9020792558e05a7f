"""Shared pytest setup: the `gpu` marker, import paths and small helpers."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); runs the engine's kernels")


@pytest.fixture(scope="session")
def golden():
    def load(name: str):
        return np.load(GOLDEN / f"{name}.npz")
    return load


def fp_tol(a: np.ndarray) -> float:
    """The per-step FP32 tolerance: 1e-5 of the field's range (at least 1e-5 absolute)."""
    r = float(np.max(a) - np.min(a)) if a.size else 0.0
    return max(1e-5 * r, 1e-5)


def decode_png(data: bytes):
    """Minimal PNG reader for the engine's exports (non-interlaced grey or RGB, 8 or 16 bits, any
    filter type): checks the signature and every chunk CRC, returns (pixels, chunk type list)."""
    import struct
    import zlib

    assert data[:8] == b"\x89PNG\r\n\x1a\n", "PNG signature"
    pos, chunks, idat, ihdr = 8, [], b"", None
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert zlib.crc32(typ + body) == crc, f"CRC of {typ!r}"
        chunks.append(typ.decode())
        if typ == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    assert chunks[0] == "IHDR" and chunks[-1] == "IEND"
    W, H, depth, ctype, comp, filt, inter = ihdr
    assert comp == 0 and filt == 0 and inter == 0
    ch = {0: 1, 2: 3}[ctype]
    bpp = ch * depth // 8
    raw = zlib.decompress(idat)
    stride = W * bpp
    assert len(raw) == H * (stride + 1)
    out = np.zeros((H, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    for y in range(H):
        f = raw[y * (stride + 1)]
        line = np.frombuffer(raw, np.uint8, stride, y * (stride + 1) + 1).astype(np.int32)
        cur = line.copy() if f == 0 else np.zeros(stride, np.int32)
        for i in range(stride if f else 0):
            a = cur[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            if f == 0:
                p = 0
            elif f == 1:
                p = a
            elif f == 2:
                p = b
            elif f == 3:
                p = (a + b) // 2
            else:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                p = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
            cur[i] = (line[i] + p) & 0xFF
        out[y] = cur
        prev = cur
    if depth == 16:
        px = out.reshape(H, W * ch, 2).astype(np.uint16)
        px = (px[..., 0] << 8) | px[..., 1]
    else:
        px = out
    return px.reshape((H, W, ch) if ch > 1 else (H, W)), chunks
