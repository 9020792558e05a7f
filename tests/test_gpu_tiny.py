"""Worlds smaller than one tile, and thinner than a stencil's halo, on every phase (reference
uplift, plate dynamics, relabel and merges included): the engine equals the oracle bit for bit, as
the wrap-around rules of the reference apply however small the grid."""
from __future__ import annotations

import numpy as np
import pytest

import master_thesis_gb300 as T
import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def stream():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available(), "a CUDA GPU is required"
    return torch.cuda.Stream()


def settings(kind):
    s = T.baseline_settings() if kind == "baseline" else T.default_settings()
    if kind == "reference":
        s.step.upliftMode = T.UPLIFT_REFERENCE
        s.step.hydraulicIterations = 3
    s.step.plateDynamics = T.PLATE_DYNAMICS_REFERENCE
    s.step.platePolicy = T.PLATE_RELABEL | T.PLATE_MERGE
    s.sim.iterationsForCCL = 1
    s.kernel.minPlateSize = 1
    s.kernel.minCollisionSize = 1
    s.kernel.collisionTypeUpdateCooldown = 1
    return s


@pytest.mark.parametrize("tile", [0, 8, 9])
@pytest.mark.parametrize("kind", ["baseline", "reference"])
@pytest.mark.parametrize("W,H", [(1, 1), (1, 7), (5, 1), (2, 3), (3, 2), (7, 5), (65, 3), (3, 70)])
def test_tiny_worlds_match_oracle(stream, kind, W, H, tile):
    s = settings(kind)
    s.step.hydraulicTile = tile
    s.step.thermalTile = 5 if tile == 9 else 0  # the marching kernels together
    w = T.World(s, W, H, seed=500)
    w.init_synthetic(min(3, W * H), 1.7, 2, stream)
    if kind == "reference":
        h = w.download(T.FIELD_HEIGHT, stream)
        w.upload(T.FIELD_HEIGHT, (np.float32(10000) + np.float32(10000) * h).astype(np.float32), stream)
    o = O.OracleWorld(s, w.download(T.FIELD_HEIGHT, stream), w.download(T.FIELD_PLATE_ID, stream), w.plates(stream),
                      500)
    for step in range(4):
        w.step(1, stream)
        o.step(1)
        w.check(stream)
        for f, want in ((T.FIELD_PLATE_ID, o.id), (T.FIELD_HEIGHT, o.h), (T.FIELD_WATER, o.w),
                        (T.FIELD_SEDIMENT, o.s), (T.FIELD_LABELS, o.labels)):
            np.testing.assert_array_equal(w.download(f, stream), want, err_msg=f"{W}x{H} step {step} field {f}")
        np.testing.assert_array_equal(w.plates(stream), o.plates, err_msg=f"{W}x{H} step {step} plates")
        np.testing.assert_array_equal(w.plate_dynamics(stream), o.dyn, err_msg=f"{W}x{H} step {step} dynamics")


def test_tiny_reference_initialisation(stream):
    for W, H in ((1, 1), (2, 3), (9, 1)):
        s = T.default_settings()
        s.sim.numStartingPlates = 3
        s.sim.numVoronoiSeeds[0], s.sim.numVoronoiSeeds[1] = 5, 9
        w = T.World(s, W, H, seed=3)
        w.init_reference(stream)
        sx, sy, sid, pl, _ = O.reference_seeds(W, H, 3, 3, (5, 9))
        h, ids = O.init_reference(W, H, 3, sx, sy, sid)
        np.testing.assert_array_equal(w.download(T.FIELD_PLATE_ID, stream), ids)
        np.testing.assert_array_equal(w.download(T.FIELD_HEIGHT, stream), h)
