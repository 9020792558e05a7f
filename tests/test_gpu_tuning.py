"""Autotuned knobs on the GPU: every sort digit width (8..11 bits) and every hydraulic tile variant
leaves the results unchanged (the sort is stable, so the sorted pairs are the same permutation;
the tiles cover the same cells), the autotuner returns a valid choice without touching the
caller's worlds, and the batch phase entry points equal the per-world ones."""
from __future__ import annotations

import numpy as np
import pytest

import master_thesis_gb300 as T
import oracle as O

pytestmark = pytest.mark.gpu

FIELDS = (T.FIELD_HEIGHT, T.FIELD_WATER, T.FIELD_SEDIMENT, T.FIELD_FLUX, T.FIELD_PLATE_ID, T.FIELD_LABELS,
          T.FIELD_COLLISION, T.FIELD_SORT_KEYS, T.FIELD_SORT_VALS, T.FIELD_TYPE_BITMAP)


@pytest.fixture(scope="module")
def stream():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available(), "a CUDA GPU is required"
    return torch.cuda.Stream()


def settings(rb=0, tile=0):
    s = T.baseline_settings()
    s.kernel.minCollisionSize = 3
    s.kernel.collisionTypeUpdateCooldown = 2
    s.sim.iterationsForCCL = 2
    s.step.sortRadixBits = rb
    s.step.hydraulicTile = tile
    return s


def run(W, H, rb, tile, steps, stream, plates=12):
    w = T.World(settings(rb, tile), W, H, seed=1000)
    w.init_synthetic(plates, 1.5, 5)
    w.step(steps, stream)
    stream.synchronize()
    w.check(stream)
    return w


@pytest.mark.parametrize("W,H", [(33, 17), (256, 128), (1024, 768), (2048, 2048)])
def test_digit_widths_give_identical_steps(stream, W, H):
    """33x17 has 10-bit keys (one pass at 11 bits, two at 8); 2048^2 has 22-bit keys (two passes at
    11 bits, three at 8); 1024x768 has 20-bit keys (two passes at 10 and 11 bits)."""
    ref = run(W, H, 8, 0, 3, stream)
    want = {f: ref.download(f) for f in FIELDS}
    for rb in (9, 10, 11):
        w = run(W, H, rb, 0, 3, stream)
        for f in FIELDS:
            np.testing.assert_array_equal(w.download(f), want[f], err_msg=f"{W}x{H} rb={rb} field {f}")
        w.close()
    if W * H <= 256 * 128:
        s = settings(8, 0)
        o = T.World(s, W, H, seed=1000)
        o.init_synthetic(12, 1.5, 5)
        ow = O.OracleWorld(s, o.download(T.FIELD_HEIGHT), o.download(T.FIELD_PLATE_ID), o.plates(), 1000)
        ow.step(3)
        np.testing.assert_array_equal(want[T.FIELD_PLATE_ID], ow.id)
        np.testing.assert_array_equal(want[T.FIELD_HEIGHT], ow.h)


def test_digit_widths_in_a_batch(stream):
    """A batch's sort runs over all its cells (here 26-bit keys): 3 passes at 9..11 bits, 4 at 8."""
    rng = np.random.default_rng(11)
    shapes = [(int(rng.integers(100, 1400)), int(rng.integers(100, 1400))) for _ in range(80)]
    res = {}
    for rb in (8, 9, 11):
        b = T.Batch()
        ws = []
        for i, (W, H) in enumerate(shapes):
            w = T.World(settings(rb, 0), W, H, seed=2000 + i)
            w.init_synthetic_device(4 + i % 20, 1.0, 300 + i)
            b.add(w, stream)
            ws.append(w)
        assert sum(W * H for W, H in shapes) > 1 << 25
        b.step(2, stream)
        stream.synchronize()
        b.check(stream)
        res[rb] = [(w.download(T.FIELD_HEIGHT), w.download(T.FIELD_PLATE_ID), w.download(T.FIELD_LABELS))
                   for w in ws]
        b.close()
        for w in ws:
            w.close()
    for rb in (9, 11):
        for i, (a, c) in enumerate(zip(res[8], res[rb])):
            for x, y in zip(a, c):
                np.testing.assert_array_equal(x, y, err_msg=f"world {i} rb={rb}")


def test_world_autotune_keeps_results(stream):
    W, H = 640, 384
    plain = run(W, H, 8, 4, 4, stream)
    w = T.World(settings(0, 0), W, H, seed=1000)
    w.init_synthetic(12, 1.5, 5)
    h0 = w.download(T.FIELD_HEIGHT)
    t = w.autotune(stream)
    assert 1 <= t.hydraulicTile <= 9 and 8 <= t.sortRadixBits <= 11
    assert all(x > 0 for x in t.hydraulic_ms) and all(x > 0 for x in t.sort_ms)
    assert t.hydraulic_ms[t.hydraulicTile - 1] == min(t.hydraulic_ms)
    assert t.sort_ms[t.sortRadixBits - 8] == min(t.sort_ms)
    np.testing.assert_array_equal(w.download(T.FIELD_HEIGHT), h0)  # tuning ran on scratch worlds
    assert w.iteration == 0
    w.step(4, stream)
    stream.synchronize()
    w.check(stream)
    for f in FIELDS:
        np.testing.assert_array_equal(w.download(f), plain.download(f), err_msg=f"field {f}")
    assert T.autotune_lookup(0, W * H, 1) == (t.hydraulicTile, t.sortRadixBits, t.thermalTile)
    assert 1 <= t.thermalTile <= 5 and t.thermal_ms[t.thermalTile - 1] == min(t.thermal_ms)


def test_shape_autotune_and_batch_autotune(stream):
    T.autotune_clear()
    shapes = [(256, 256), (512, 256), (128, 128), (1024, 512)]
    t = T.autotune(settings(), shapes, stream)
    assert T.autotune_lookup(0, sum(a * b for a, b in shapes), len(shapes)) == (t.hydraulicTile, t.sortRadixBits,
                                                                                 t.thermalTile)
    b = T.Batch()
    ws = []
    for i, (W, H) in enumerate(shapes):
        w = T.World(settings(), W, H, seed=10 + i)
        w.init_synthetic_device(8, 1.0, 20 + i)
        b.add(w, stream)
        ws.append(w)
    tb = b.autotune(stream)
    assert 1 <= tb.hydraulicTile <= 8 and 8 <= tb.sortRadixBits <= 11
    b.step(2, stream)
    stream.synchronize()
    b.check(stream)
    b.close()


def test_batch_phases_equal_world_phases(stream):
    shapes = [(100, 60), (256, 128), (33, 17)]
    alone, mixed = [], []
    b = T.Batch()
    for i, (W, H) in enumerate(shapes):
        for lst in (alone, mixed):
            w = T.World(settings(), W, H, seed=40 + i)
            w.init_synthetic(6, 1.0, 50 + i)
            w.step(1, stream)
            lst.append(w)
    for w in mixed:
        b.add(w, stream)
    b.thermal(7, stream)
    b.hydraulic(5, 0.02, stream)
    for w in alone:
        w.thermal(7, stream)
        w.hydraulic(5, 0.02, stream)
    stream.synchronize()
    for a, m in zip(alone, mixed):
        for f in (T.FIELD_HEIGHT, T.FIELD_WATER, T.FIELD_SEDIMENT, T.FIELD_FLUX):
            np.testing.assert_array_equal(a.download(f), m.download(f))
    b.close()
