"""Plate relabel and merges on the GPU against the CPU oracle (whose merges the reference's kernels
pin, test_oracle_policy.py): every field, the plate records and the plate dynamics records agree
bit for bit step after step, with and without plate dynamics, for two CCL connectivities, alone
and in a batch whose worlds label on different steps."""
from __future__ import annotations

import numpy as np
import pytest

import master_thesis_gb300 as T
import oracle as O

pytestmark = pytest.mark.gpu

FIELDS = (T.FIELD_HEIGHT, T.FIELD_WATER, T.FIELD_SEDIMENT, T.FIELD_PLATE_ID, T.FIELD_LABELS,
          T.FIELD_TYPE_BITMAP, T.FIELD_DIV_BITMAP)


@pytest.fixture(scope="module")
def stream():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available(), "a CUDA GPU is required"
    return torch.cuda.Stream()


def settings(dynamics=True, conn=T.CCL_REF8, period=1):
    s = T.baseline_settings()
    s.step.plateDynamics = T.PLATE_DYNAMICS_REFERENCE if dynamics else T.PLATE_DYNAMICS_OFF
    s.step.platePolicy = T.PLATE_RELABEL | T.PLATE_MERGE
    s.step.cclConnectivity = conn
    s.sim.iterationsForCCL = period
    s.kernel.minCollisionSize = 3
    s.kernel.collisionTypeUpdateCooldown = 2
    s.kernel.minPlateSize = 3
    s.kernel.mergeMinVelocity = 0.35
    s.kernel.mergeDotDirectionThreshold = 0.95
    s.kernel.mergeVelocityDiffThreshold = 0.05
    s.kernel.targetMaximumPlateArea = 3000
    return s


def make(s, W, H, plates, gen, stream):
    w = T.World(s, W, H, seed=900 + gen)
    w.init_synthetic(plates, 1.8, gen, stream)
    o = O.OracleWorld(s, w.download(T.FIELD_HEIGHT, stream), w.download(T.FIELD_PLATE_ID, stream),
                      w.plates(stream), 900 + gen)
    return w, o


def oracle_field(o, f):
    return {T.FIELD_HEIGHT: o.h, T.FIELD_WATER: o.w, T.FIELD_SEDIMENT: o.s, T.FIELD_PLATE_ID: o.id,
            T.FIELD_LABELS: o.labels, T.FIELD_TYPE_BITMAP: o.bitmap, T.FIELD_DIV_BITMAP: o.div}[f]


@pytest.mark.parametrize("dynamics", [True, False])
@pytest.mark.parametrize("conn", [T.CCL_REF8, T.CCL_4])
@pytest.mark.parametrize("W,H,plates", [(64, 64, 12), (100, 60, 20), (37, 23, 6)])
def test_policy_matches_oracle(stream, dynamics, conn, W, H, plates):
    s = settings(dynamics, conn)
    w, o = make(s, W, H, plates, 3, stream)
    changed = False
    for step in range(8):
        before = o.id.copy()
        w.step(1, stream)
        o.step(1)
        for f in FIELDS:
            np.testing.assert_array_equal(w.download(f, stream), oracle_field(o, f),
                                          err_msg=f"step {step} field {f}")
        np.testing.assert_array_equal(w.plates(stream), o.plates, err_msg=f"step {step} plates")
        np.testing.assert_array_equal(w.plate_dynamics(stream), o.dyn, err_msg=f"step {step} plate dynamics")
        changed = changed or len(np.unique(o.id)) != len(np.unique(before))
    assert changed, "no relabel or merge changed the plate count"


def test_policy_in_a_batch_equals_alone(stream):
    s = settings(True, T.CCL_REF8, period=2)
    specs = [(64, 64, 10, 1), (48, 80, 8, 2), (90, 40, 14, 3)]
    alone = [make(s, W, H, p, g, stream)[0] for W, H, p, g in specs]
    mixed = [make(s, W, H, p, g, stream)[0] for W, H, p, g in specs]
    mixed[1].step(1, stream)  # label on different steps than the others
    alone[1].step(1, stream)
    for w in alone:
        w.step(5, stream)
    b = T.Batch()
    for w in mixed:
        b.add(w, stream)
    b.step(5, stream)
    stream.synchronize()
    for i, (a, m) in enumerate(zip(alone, mixed)):
        for f in FIELDS:
            np.testing.assert_array_equal(a.download(f, stream), m.download(f, stream), err_msg=f"world {i} field {f}")
        np.testing.assert_array_equal(a.plates(stream), m.plates(stream))
        np.testing.assert_array_equal(a.plate_dynamics(stream), m.plate_dynamics(stream))
    b.close()


def test_unknown_policy_bits_are_refused(stream):
    s = settings()
    s.step.platePolicy = 8
    w = T.World(s, 32, 32)
    w.init_synthetic(3, 1.0, 1, stream)
    with pytest.raises(T.TectoError):
        w.step(1, stream)


def test_reference_configuration_100_steps(stream):
    """Everything on for 100 steps: the reference's initialisation, default settings and uplift,
    plate dynamics with an asthenosphere texture, relabel after every CCL, merges.  The engine
    stays bit-identical to the oracle throughout."""
    s = T.default_settings()
    s.step.upliftMode = T.UPLIFT_REFERENCE
    s.step.hydraulicIterations = 4
    s.step.plateDynamics = T.PLATE_DYNAMICS_REFERENCE
    s.step.platePolicy = T.PLATE_RELABEL | T.PLATE_MERGE
    s.sim.iterationsForCCL = 5
    s.sim.numStartingPlates = 10
    s.sim.numVoronoiSeeds[0], s.sim.numVoronoiSeeds[1] = 60, 150
    s.kernel.minPlateSize = 20
    s.kernel.targetMaximumPlateArea = 6000
    W, H = 128, 96
    w = T.World(s, W, H, seed=2024)
    w.init_reference(stream)
    pr = np.random.default_rng(2).random((40, 50)).astype(np.float32)
    w.set_asthenosphere(pr, stream)
    o = O.OracleWorld(s, w.download(T.FIELD_HEIGHT, stream), w.download(T.FIELD_PLATE_ID, stream),
                      w.plates(stream), 2024)
    o.dyn = w.plate_dynamics(stream)
    o.pressure = pr
    counts = []
    for chunk in range(10):
        w.step(10, stream)
        o.step(10)
        w.check(stream)
        for f in FIELDS:
            np.testing.assert_array_equal(w.download(f, stream), oracle_field(o, f), err_msg=f"step {10 * chunk + 9} field {f}")
        np.testing.assert_array_equal(w.plates(stream), o.plates)
        np.testing.assert_array_equal(w.plate_dynamics(stream), o.dyn)
        counts.append(len(np.unique(o.id)))
    assert w.iteration == 100
    assert min(counts) >= 1
