"""Parity on the code paths that only sizes above 16.7 M cells take.

From 4096 tiles of 4096 keys (16 777 216 pairs) the onesweep passes run in their form for large
sorts (three blocks per SM).  The mixed batch of the headline benchmark (43.6 M cells) and the
8192^2 world (67 M cells) sort in that form, so it is checked here the way the smaller form is:
- the standalone sort at 20 M pairs, 26-bit keys with a long run of equal keys, at every digit
  width, against numpy's stable argsort;
- a batch of more than 16.7 M cells stepped twice, every world against the same world stepped
  alone (a world alone sorts in the small form, which the oracle pins), and two of them against
  the oracle;
- one 8192^2 world (64 plates, velocities in [-2, 2], 8-connected CCL every step) stepped once
  against the oracle: plate ids, arrival words and labels bit-exact, height, water and sediment
  within 1e-5 of the range; the sorted pairs checked for order, stability and permutation.

Reference behaviour replaced by the sort: registerPlateCollisions and processCollisions,
src/cuda_compute/plate_tectonics_kernel.cu:273-298, 677-745.
"""
from __future__ import annotations

import numpy as np
import pytest

import master_thesis_gb300 as T
import oracle as O
from conftest import fp_tol

pytestmark = pytest.mark.gpu

WIDE = 4096 * 4096


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    assert t.cuda.is_available(), "a CUDA GPU is required"
    return t


def sort_radix(torch, keys: np.ndarray, vals: np.ndarray, key_bits: int, rb: int):
    n = keys.size
    L = T.lib()
    kin = torch.from_numpy(keys.view(np.int32)).cuda()
    vin = torch.from_numpy(vals.view(np.int32)).cuda()
    kout = torch.empty_like(kin)
    vout = torch.empty_like(vin)
    nbytes = L.tecto_sort_scratch_bytes_radix(n, key_bits, rb)
    assert nbytes > 0
    scratch = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    T.check(L.tecto_sort_pairs_radix(kin.data_ptr(), vin.data_ptr(), kout.data_ptr(), vout.data_ptr(), n,
                                     key_bits, rb, scratch.data_ptr(), nbytes, stream), "tecto_sort_pairs_radix")
    torch.cuda.synchronize()
    out = kout.cpu().numpy().view(np.uint32), vout.cpu().numpy().view(np.uint32)
    del kin, vin, kout, vout, scratch
    return out


@pytest.fixture(scope="module")
def wide_case():
    n = 20_000_000
    rng = np.random.default_rng(2026)
    keys = rng.integers(0, 1 << 26, n, dtype=np.uint32)
    keys[5_000_000:8_000_000] = 12_345_678  # a run of 3 M equal keys across hundreds of tiles
    keys[-4096:] = (1 << 26) - 1            # the largest key fills the last tile
    vals = rng.permutation(n).astype(np.uint32)
    order = np.argsort(keys, kind="stable")
    return keys, vals, keys[order], vals[order]


@pytest.mark.parametrize("rb", [8, 9, 10, 11])
def test_wide_sort_is_numpys_stable_sort(torch, wide_case, rb):
    keys, vals, want_k, want_v = wide_case
    assert T.lib().tecto_sort_wide_pass(keys.size) == 1
    k, v = sort_radix(torch, keys, vals, 26, rb)
    np.testing.assert_array_equal(k, want_k)
    np.testing.assert_array_equal(v, want_v)


def test_sort_at_the_form_boundary(torch):
    """One pair below and at the first size of the large form, 24-bit keys, all digit widths."""
    rng = np.random.default_rng(5)
    for n in (WIDE - 4096, WIDE):
        keys = rng.integers(0, 1 << 24, n, dtype=np.uint32)
        vals = np.arange(n, dtype=np.uint32)
        order = np.argsort(keys, kind="stable")
        assert T.lib().tecto_sort_wide_pass(n) == (1 if n >= WIDE else 0)
        for rb in (8, 11):
            k, v = sort_radix(torch, keys, vals, 24, rb)
            np.testing.assert_array_equal(k, keys[order], err_msg=f"n={n} rb={rb}")
            np.testing.assert_array_equal(v, order.astype(np.uint32), err_msg=f"n={n} rb={rb}")


FIELDS = (T.FIELD_HEIGHT, T.FIELD_WATER, T.FIELD_SEDIMENT, T.FIELD_FLUX, T.FIELD_PLATE_ID, T.FIELD_LABELS,
          T.FIELD_COLLISION, T.FIELD_TYPE_BITMAP)


def batch_settings(rb, tile=4):
    s = T.baseline_settings()
    s.kernel.minCollisionSize = 3
    s.kernel.collisionTypeUpdateCooldown = 2
    s.sim.iterationsForCCL = 1
    s.step.sortRadixBits = rb
    s.step.hydraulicTile = tile
    s.step.thermalTile = 5 if tile == 9 else 4  # the marching kernels together, or the tiles
    return s


@pytest.mark.parametrize("rb,tile", [(8, 9), (11, 4)])
def test_batch_above_the_form_boundary_equals_worlds_alone(torch, rb, tile):
    """18 worlds, 18.6 M cells in all (25-bit batch keys, the large sort form), two steps; every
    world equals itself stepped alone (1 M cells or fewer: the small form), field by field.  The
    hydraulic sub-iterations run as the marching kernel (variant 9: strips of many worlds shared
    by persistent blocks) or as tiles (variant 4)."""
    stream = torch.cuda.Stream()
    rng = np.random.default_rng(99)
    shapes = [(1024, 1024)] * 12 + [(int(rng.integers(700, 1100)), int(rng.integers(500, 1000))) for _ in range(6)]
    cells = sum(W * H for W, H in shapes)
    assert cells >= WIDE and T.lib().tecto_sort_wide_pass(cells) == 1
    worlds = []
    b = T.Batch()
    for i, (W, H) in enumerate(shapes):
        w = T.World(batch_settings(rb, tile), W, H, seed=3000 + i)
        w.init_synthetic_device(4 + (7 * i) % 29, 1.0 + (i % 3) * 0.5, 500 + i)
        b.add(w, stream)
        worlds.append(w)
    b.step(2, stream)
    stream.synchronize()
    b.check(stream)
    got = [{f: w.download(f) for f in FIELDS} for w in worlds]
    b.close()
    for w in worlds:
        w.close()
    for i, (W, H) in enumerate(shapes):
        assert T.lib().tecto_sort_wide_pass(W * H) == 0
        a = T.World(batch_settings(rb, tile), W, H, seed=3000 + i)
        a.init_synthetic_device(4 + (7 * i) % 29, 1.0 + (i % 3) * 0.5, 500 + i)
        if i < 2:
            ow = O.OracleWorld(batch_settings(rb, tile), a.download(T.FIELD_HEIGHT), a.download(T.FIELD_PLATE_ID),
                               a.plates(), 3000 + i)
        a.step(2, stream)
        stream.synchronize()
        a.check(stream)
        for f in FIELDS:
            np.testing.assert_array_equal(got[i][f], a.download(f), err_msg=f"world {i} ({W}x{H}) field {f}")
        a.close()
        if i < 2:
            ow.step(2)
            np.testing.assert_array_equal(got[i][T.FIELD_PLATE_ID], ow.id, err_msg=f"world {i} ids vs oracle")
            np.testing.assert_array_equal(got[i][T.FIELD_LABELS], ow.labels, err_msg=f"world {i} labels vs oracle")
            np.testing.assert_array_equal(got[i][T.FIELD_COLLISION], ow.word, err_msg=f"world {i} words vs oracle")
            for f, want in ((T.FIELD_HEIGHT, ow.h), (T.FIELD_WATER, ow.w), (T.FIELD_SEDIMENT, ow.s)):
                assert float(np.max(np.abs(got[i][f] - want))) <= fp_tol(want), f"world {i} field {f} vs oracle"


def test_8192_world_one_step_matches_oracle(torch):
    """The stress configuration: 8192^2 (67 M cells, 26-bit keys), 64 plates, velocities in
    [-2, 2], 8-connected CCL on every step; one step against the oracle, with the marching
    hydraulic and thermal kernels (the autotuner's choices for this size)."""
    s = T.baseline_settings()
    s.step.hydraulicTile = 9
    s.step.thermalTile = 5
    s.sim.iterationsForCCL = 1
    s.step.cclConnectivity = T.CCL_8
    W = H = 8192
    assert T.lib().tecto_sort_wide_pass(W * H) == 1
    stream = torch.cuda.Stream()
    w = T.World(s, W, H, seed=1000)
    w.init_synthetic_device(64, 2.0, 1)
    ow = O.OracleWorld(s, w.download(T.FIELD_HEIGHT), w.download(T.FIELD_PLATE_ID), w.plates(), 1000)
    w.step(1, stream)
    stream.synchronize()
    w.check(stream)
    ow.step(1)
    np.testing.assert_array_equal(w.download(T.FIELD_PLATE_ID), ow.id)
    np.testing.assert_array_equal(w.download(T.FIELD_COLLISION), ow.word)
    np.testing.assert_array_equal(w.download(T.FIELD_LABELS), ow.labels)
    for f, want in ((T.FIELD_HEIGHT, ow.h), (T.FIELD_WATER, ow.w), (T.FIELD_SEDIMENT, ow.s)):
        got = w.download(f)
        assert float(np.max(np.abs(got - want))) <= fp_tol(want), f"field {f}"
    del ow
    keys = w.download(T.FIELD_SORT_KEYS).ravel()
    vals = w.download(T.FIELD_SORT_VALS).ravel()
    w.close()
    dk = np.diff(keys.astype(np.int64))
    assert np.all(dk >= 0)
    assert np.all(np.diff(vals.astype(np.int64))[dk == 0] > 0)  # stable: sources ascend in a run
    seen = np.zeros(W * H, np.bool_)
    seen[vals] = True
    assert seen.all()  # every source cell exactly once


def test_config1_2048_100_steps_match_oracle(torch):
    """The single large world: 2048^2, 32 plates, 100 steps (4-connected CCL every 10) against the
    oracle at the long-horizon bound, 1e-3 of the range for height, water and sediment; plate ids
    and labels bit-exact.  About 90 s of oracle stepping on 16 cores."""
    s = T.baseline_settings()
    stream = torch.cuda.Stream()
    w = T.World(s, 2048, 2048, seed=1000)
    w.init_synthetic(32, 1.0, 1)
    ow = O.OracleWorld(s, w.download(T.FIELD_HEIGHT), w.download(T.FIELD_PLATE_ID), w.plates(), 1000)
    w.step(100, stream)
    stream.synchronize()
    w.check(stream)
    ow.step(100)
    np.testing.assert_array_equal(w.download(T.FIELD_PLATE_ID), ow.id)
    np.testing.assert_array_equal(w.download(T.FIELD_LABELS), ow.labels)
    for f, want in ((T.FIELD_HEIGHT, ow.h), (T.FIELD_WATER, ow.w), (T.FIELD_SEDIMENT, ow.s)):
        got = w.download(f)
        r = float(want.max() - want.min())
        d = float(np.max(np.abs(got - want)))
        assert d <= max(1e-3 * r, 1e-5), f"field {f}: max |diff| {d}, range {r}"
    w.close()
