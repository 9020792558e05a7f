"""The standalone radix sort and the CCL kernels against numpy / the oracle, including edge cases:
empty-ish and ragged sizes, all-equal keys, full 32-bit keys, wrap-around components, 1-wide grids.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import master_thesis_gb300 as T
import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    assert t.cuda.is_available(), "a CUDA GPU is required"
    return t


def gpu_sort(torch, keys: np.ndarray, vals: np.ndarray, key_bits: int):
    n = keys.size
    L = T.lib()
    kin = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    vin = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    kout = torch.empty_like(kin)
    vout = torch.empty_like(vin)
    nbytes = L.tecto_sort_scratch_bytes(n, key_bits)
    scratch = torch.empty(max(nbytes, 1), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    T.check(L.tecto_sort_pairs(kin.data_ptr(), vin.data_ptr(), kout.data_ptr(), vout.data_ptr(), n, key_bits,
                               scratch.data_ptr(), nbytes, stream), "tecto_sort_pairs")
    torch.cuda.synchronize()
    return kout.cpu().numpy().view(np.uint32), vout.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("n,bits,dist", [
    (1, 8, "uniform"), (255, 8, "uniform"), (4096, 12, "uniform"), (4097, 16, "uniform"),
    (100_000, 17, "uniform"), (1_000_003, 20, "uniform"), (70_000, 32, "uniform"),
    (50_000, 16, "equal"), (300_000, 22, "few"), (262_144, 18, "sorted"), (262_144, 18, "reversed"),
])
def test_sort_pairs_is_a_stable_sort(torch, n, bits, dist):
    rng = np.random.default_rng(n + bits)
    hi = (1 << bits) if bits < 32 else (1 << 32)
    if dist == "uniform":
        keys = rng.integers(0, hi, n, dtype=np.uint64).astype(np.uint32)
    elif dist == "equal":
        keys = np.full(n, 12345 % hi, np.uint32)
    elif dist == "few":
        keys = rng.choice(np.array([0, 7, hi - 1, 99991 % hi], np.uint64), n).astype(np.uint32)
    elif dist == "sorted":
        keys = np.sort(rng.integers(0, hi, n, dtype=np.uint64)).astype(np.uint32)
    else:
        keys = np.sort(rng.integers(0, hi, n, dtype=np.uint64))[::-1].astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    k, v = gpu_sort(torch, keys, vals, bits)
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(k, keys[order])
    np.testing.assert_array_equal(v, vals[order])


def ccl_gpu(ids: np.ndarray, mode: int) -> np.ndarray:
    H, W = ids.shape
    w = T.World(T.baseline_settings(), W, H)
    w.upload(T.FIELD_PLATE_ID, ids)
    w.ccl(mode)
    out = w.download(T.FIELD_LABELS)
    w.check()
    w.close()
    return out


def id_maps():
    rng = np.random.default_rng(17)
    yield "random3_70x45", rng.integers(0, 3, (45, 70)).astype(np.uint8)
    yield "random2_130x129", rng.integers(0, 2, (129, 130)).astype(np.uint8)
    yield "uniform_40x40", np.zeros((40, 40), np.uint8)
    yield "row_1x77", rng.integers(0, 2, (1, 77)).astype(np.uint8)
    yield "col_77x1", rng.integers(0, 2, (77, 1)).astype(np.uint8)
    yield "tiny_3x3", rng.integers(0, 2, (3, 3)).astype(np.uint8)
    spiral = np.zeros((64, 96), np.uint8)
    spiral[::2, :] = 1
    spiral[:, ::5] = 2
    yield "stripes_64x96", spiral
    diag = np.fromfunction(lambda y, x: ((x + y) % 7 == 0).astype(np.uint8), (50, 90)).astype(np.uint8)
    yield "diag_50x90", diag
    _, ids, _ = T.generate_world(300, 170, 12, 1.0, 9)
    yield "voronoi_300x170", ids
    # one tile spans the whole world: edges wrap back into the same tile
    yield "random2_32x16", rng.integers(0, 2, (16, 32)).astype(np.uint8)
    yield "random2_32x5", rng.integers(0, 2, (5, 32)).astype(np.uint8)
    yield "checker_48x20", np.fromfunction(lambda y, x: (x + y) % 2, (20, 48)).astype(np.uint8)
    yield "random4_33x17", rng.integers(0, 4, (17, 33)).astype(np.uint8)
    # long horizontal runs broken by sparse dots: run starts and skipped up edges
    runs = np.zeros((40, 100), np.uint8)
    runs[rng.integers(0, 40, 120), rng.integers(0, 100, 120)] = 1
    yield "sparse_dots_100x40", runs


@pytest.mark.parametrize("mode", [T.CCL_4, T.CCL_8, T.CCL_REF8])
@pytest.mark.parametrize("name,ids", list(id_maps()), ids=lambda v: v if isinstance(v, str) else "")
def test_ccl_matches_oracle(name, ids, mode):
    np.testing.assert_array_equal(ccl_gpu(ids, mode), O.ccl(ids, mode))


def test_ccl_ref8_matches_reference_golden(golden):
    g = golden("ref_ccl_cases")
    for case in ("random4", "random2", "diagonals", "stripes", "voronoi"):
        np.testing.assert_array_equal(ccl_gpu(g[f"{case}_id"], T.CCL_REF8), g[f"{case}_labels"], err_msg=case)


def test_ccl_large_voronoi_8192_row_band():
    """A wide world (8192 x 64) exercises long wrap-around components across many tiles."""
    _, ids, _ = T.generate_world(8192, 64, 64, 2.0, 3)
    for mode in (T.CCL_4, T.CCL_8):
        np.testing.assert_array_equal(ccl_gpu(ids, mode), O.ccl(ids, mode))
