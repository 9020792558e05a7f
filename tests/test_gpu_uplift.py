"""The reference uplift (TECTO_UPLIFT_REFERENCE) on the GPU against the oracle: phase by phase
(resolve + uplift heights, ids, JFA seeds and distances), whole steps, and worlds in a batch
equal to the same worlds alone.  Integer fields bit-exact; heights within the per-step FP32
tolerance (in practice bit-exact: both sides use the engine's own exp/log10 and IEEE operations)."""
from __future__ import annotations

import numpy as np
import pytest

import master_thesis_gb300 as T
import oracle as O
from conftest import fp_tol

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def stream():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available(), "a CUDA GPU is required"
    return torch.cuda.Stream()


def settings(prop_threshold=12000.0):
    s = T.default_settings()
    s.kernel.minCollisionSize = 3
    s.kernel.collisionTypeUpdateCooldown = 2
    s.kernel.continentalPropThreshold = prop_threshold
    s.sim.iterationsForCCL = 3
    s.step.upliftMode = T.UPLIFT_REFERENCE
    return s


def make(W, H, plates, vel, gen, st, seed=1000):
    w = T.World(st, W, H, seed=seed)
    w.init_synthetic(plates, vel, gen)
    h = w.download(T.FIELD_HEIGHT)
    w.upload(T.FIELD_HEIGHT, (np.float32(10000) + np.float32(10000) * h).astype(np.float32))
    return w


@pytest.mark.parametrize("W,H,plates,gen", [(64, 48, 8, 21), (100, 60, 6, 3), (33, 17, 4, 5), (256, 128, 12, 9)])
def test_uplift_phase_matches_oracle(W, H, plates, gen):
    st = settings()
    w = make(W, H, plates, 1.5, gen, st)
    h = w.download(T.FIELD_HEIGHT)
    ids = w.download(T.FIELD_PLATE_ID)
    pl = w.plates()
    bm = np.zeros(T.NUM_PAIRS, np.uint8)
    div = np.zeros(T.NUM_DIV_WORDS, np.uint32)
    uplifted = 0
    for it in range(5):
        offx, offy, nxt = O.plate_offsets(pl)
        _, word, _, _ = O.collision_words(ids, offx, offy)
        bm = O.collision_types(word, h, offx, offy, st, bm)
        w.collide()
        np.testing.assert_array_equal(w.download(T.FIELD_COLLISION), word)
        hn, idn, acc, div, uh, ut = O.resolve_ex(ids, h, word, offx, offy, bm, div, st, 1000, it)
        hu, seed, dist = O.uplift_ref(word, uh, ut, h, pl, idn, hn, st)
        uplifted += int((hu != hn).sum())
        w.resolve()
        np.testing.assert_array_equal(w.download(T.FIELD_PLATE_ID), idn, err_msg=f"ids step {it}")
        np.testing.assert_array_equal(w.download(T.FIELD_JFA_SEED), seed, err_msg=f"JFA seeds step {it}")
        np.testing.assert_array_equal(w.download(T.FIELD_JFA_DIST), dist, err_msg=f"JFA distances step {it}")
        got = w.download(T.FIELD_HEIGHT)
        d = float(np.max(np.abs(got.astype(np.float64) - hu)))
        assert d <= fp_tol(hu), f"heights step {it}: max |diff| {d}"
        np.testing.assert_array_equal(got, hu, err_msg=f"heights step {it} (bit-exact)")
        # continue without erosion: the engine's state becomes the next step's input
        w.thermal(0)
        w.finish()
        h = w.download(T.FIELD_HEIGHT)
        ids = w.download(T.FIELD_PLATE_ID)
        pl = nxt
    w.check()
    assert uplifted > 0


@pytest.mark.parametrize("W,H", [(64, 64), (128, 96)])
def test_uplift_steps_match_oracle(stream, W, H):
    st = settings()
    w = make(W, H, 8, 1.5, 7, st)
    ow = O.OracleWorld(st, w.download(T.FIELD_HEIGHT), w.download(T.FIELD_PLATE_ID), w.plates(), 1000)
    for it in range(6):
        w.step(1, stream)
        stream.synchronize()
        ow.step()
        np.testing.assert_array_equal(w.download(T.FIELD_PLATE_ID), ow.id, err_msg=f"ids {it}")
        np.testing.assert_array_equal(w.download(T.FIELD_LABELS), ow.labels, err_msg=f"labels {it}")
        for name, f, want in (("h", T.FIELD_HEIGHT, ow.h), ("w", T.FIELD_WATER, ow.w), ("s", T.FIELD_SEDIMENT, ow.s)):
            got = w.download(f)
            d = float(np.max(np.abs(got.astype(np.float64) - want)))
            assert d <= fp_tol(want), f"{name} step {it}: max |diff| {d}"
    w.check(stream)


def test_uplift_batch_equals_alone(stream):
    st = settings()
    specs = [(64, 48, 8, 21), (100, 60, 6, 3), (33, 17, 4, 5), (200, 120, 10, 8)]
    alone = [make(W, H, P, 1.5, g, st, seed=500 + i) for i, (W, H, P, g) in enumerate(specs)]
    mixed = [make(W, H, P, 1.5, g, st, seed=500 + i) for i, (W, H, P, g) in enumerate(specs)]
    b = T.Batch()
    for w in mixed:
        b.add(w, stream)
    b.step(4, stream)
    for w in alone:
        w.step(4, stream)
    stream.synchronize()
    b.check(stream)
    for i, (a, m) in enumerate(zip(alone, mixed)):
        for f in (T.FIELD_HEIGHT, T.FIELD_PLATE_ID, T.FIELD_WATER, T.FIELD_LABELS):
            np.testing.assert_array_equal(a.download(f), m.download(f), err_msg=f"world {i} field {f}")
    b.close()
