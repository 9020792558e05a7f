"""tecto_sort_pairs_noalloc: the radix sort for callers that cannot allocate device memory.

A plugin host that owns a fixed device-memory budget, or a per-frame loop that must not hit
cudaFree's device-wide synchronisation, cannot give the sort a scratch buffer of its own.  This
entry point keeps its scratch in one static device array of the library instead.  The test drives
it through the C ABI and checks, on two calls in a row (the second reusing the array the first left
behind), that it returns exactly what the allocating entry point tecto_sort_pairs returns.  The
sort works on integers, so the tolerance is zero: results must be identical.  It also checks that
sizes above the array's capacity are refused before any GPU work.

This file is named so that pytest collects it last.
"""
from __future__ import annotations

import numpy as np
import pytest

import master_thesis_gb300 as T

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    assert t.cuda.is_available(), "a CUDA GPU is required"
    return t


def _dev(torch, a: np.ndarray):
    return torch.from_numpy(a.view(np.int32).copy()).cuda()


def _host(t) -> np.ndarray:
    return t.cpu().numpy().view(np.uint32)


def sort_allocating(torch, kin, vin, n, bits, stream):
    L = T.lib()
    kout, vout = torch.empty_like(kin), torch.empty_like(vin)
    nbytes = L.tecto_sort_scratch_bytes(n, bits)
    scratch = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    T.check(L.tecto_sort_pairs(kin.data_ptr(), vin.data_ptr(), kout.data_ptr(), vout.data_ptr(), n, bits,
                               scratch.data_ptr(), nbytes, stream), "tecto_sort_pairs")
    return _host(kout), _host(vout)


def sort_noalloc(torch, kin, vin, n, bits, stream):
    L = T.lib()
    kout, vout = torch.empty_like(kin), torch.empty_like(vin)
    T.check(L.tecto_sort_pairs_noalloc(kin.data_ptr(), vin.data_ptr(), kout.data_ptr(), vout.data_ptr(), n,
                                       bits, stream), "tecto_sort_pairs_noalloc")
    return _host(kout), _host(vout)


def test_noalloc_sort_matches_allocating_sort_on_two_calls_in_a_row(torch):
    stream = torch.cuda.current_stream().cuda_stream
    cap = 1 << 20  # TECTO_SORT_NOALLOC_MAX_PAIRS
    # first call: the full capacity with 32-bit keys (4 passes); second: a smaller, ragged size
    # with 22-bit keys (3 passes) that reuses what the first call left in the shared array;
    # third: one pass (8-bit keys) over a ragged size whose last tile holds a single key
    cases = [(cap, 32, 11), (300_007, 22, 12), (4097, 8, 13)]
    for n, bits, seed in cases:
        rng = np.random.default_rng(seed)
        keys = rng.integers(0, 1 << bits, n, dtype=np.uint64).astype(np.uint32)
        keys[: n // 8] = keys[0]  # a long run of equal keys exercises stability
        vals = rng.permutation(n).astype(np.uint32)
        kin, vin = _dev(torch, keys), _dev(torch, vals)
        k_ref, v_ref = sort_allocating(torch, kin, vin, n, bits, stream)
        k_new, v_new = sort_noalloc(torch, kin, vin, n, bits, stream)
        np.testing.assert_array_equal(k_new, k_ref)
        np.testing.assert_array_equal(v_new, v_ref)
        order = np.argsort(keys, kind="stable")
        np.testing.assert_array_equal(k_new, keys[order])
        np.testing.assert_array_equal(v_new, vals[order])


def test_noalloc_sort_allocates_no_device_memory(torch):
    """After a first call (which looks up the array's address), a call of full capacity leaves the
    device's free memory exactly as it was."""
    stream = torch.cuda.current_stream().cuda_stream
    n = 1 << 20
    rng = np.random.default_rng(21)
    keys = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    kin, vin = _dev(torch, keys), _dev(torch, vals)
    kout, vout = torch.empty_like(kin), torch.empty_like(vin)
    L = T.lib()
    T.check(L.tecto_sort_pairs_noalloc(kin.data_ptr(), vin.data_ptr(), kout.data_ptr(), vout.data_ptr(), n, 32,
                                       stream), "tecto_sort_pairs_noalloc")
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    T.check(L.tecto_sort_pairs_noalloc(kin.data_ptr(), vin.data_ptr(), kout.data_ptr(), vout.data_ptr(), n, 32,
                                       stream), "tecto_sort_pairs_noalloc")
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(_host(kout), keys[order])


def test_noalloc_sort_refuses_sizes_above_its_capacity(torch):
    L = T.lib()
    n = (1 << 20) + 1
    kin = torch.zeros(n, dtype=torch.int32, device="cuda")
    out = torch.empty_like(kin)
    out2 = torch.empty_like(kin)
    rc = L.tecto_sort_pairs_noalloc(kin.data_ptr(), kin.data_ptr(), out.data_ptr(), out2.data_ptr(), n, 20,
                                    torch.cuda.current_stream().cuda_stream)
    assert rc == -1
    assert b"TECTO_SORT_NOALLOC_MAX_PAIRS" in L.tecto_last_error_string()
    # aliasing outputs onto inputs is refused too
    rc = L.tecto_sort_pairs_noalloc(kin.data_ptr(), kin.data_ptr(), kin.data_ptr(), out2.data_ptr(), 1000, 20,
                                    torch.cuda.current_stream().cuda_stream)
    assert rc == -1
    # a good call right after the refused ones sorts correctly
    keys = np.random.default_rng(3).integers(0, 1 << 20, 5000, dtype=np.uint32)
    vals = np.arange(5000, dtype=np.uint32)
    k, v = sort_noalloc(torch, _dev(torch, keys), _dev(torch, vals), 5000, 20,
                        torch.cuda.current_stream().cuda_stream)
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(k, keys[order])
    np.testing.assert_array_equal(v, vals[order])
