"""Plate dynamics on the GPU (TECTO_PLATE_DYNAMICS_REFERENCE) against the CPU oracle, which the
reference's own kernels pin (test_oracle_dynamics.py): every field, the plate records and the plate
dynamics records agree bit for bit over several steps, alone, in a mixed batch and after a snapshot
resume; the per-plate sums are fixed point, so repeated runs give the same bits."""
from __future__ import annotations

import numpy as np
import pytest

import master_thesis_gb300 as T
import oracle as O

pytestmark = pytest.mark.gpu

FIELDS = (T.FIELD_HEIGHT, T.FIELD_WATER, T.FIELD_SEDIMENT, T.FIELD_FLUX, T.FIELD_PLATE_ID, T.FIELD_LABELS,
          T.FIELD_TYPE_BITMAP, T.FIELD_DIV_BITMAP)


@pytest.fixture(scope="module")
def stream():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available(), "a CUDA GPU is required"
    return torch.cuda.Stream()


def settings(kind="baseline"):
    s = T.baseline_settings() if kind == "baseline" else T.default_settings()
    if kind == "reference":
        s.step.upliftMode = T.UPLIFT_REFERENCE
        s.step.hydraulicIterations = 4
    s.step.plateDynamics = T.PLATE_DYNAMICS_REFERENCE
    s.kernel.minCollisionSize = 3
    s.kernel.collisionTypeUpdateCooldown = 2
    s.kernel.frictionCoefficientContinental = 0.3
    s.kernel.frictionCoefficientSubduction = 0.05
    s.kernel.frictionCoefficientAccretion = 0.15
    s.kernel.mergeWaitAfterSplit = 3
    s.sim.iterationsForCCL = 3
    return s


def pressure_for(W, H, seed):
    if seed is None:
        return None
    return np.random.default_rng(seed).random((max(H // 2, 3), max(W // 3, 3))).astype(np.float32)


def make(s, W, H, plates, gen, pseed, stream, kind="baseline"):
    w = T.World(s, W, H, seed=1000 + gen)
    w.init_synthetic(plates, 1.5, gen, stream)
    if kind == "reference":
        h = w.download(T.FIELD_HEIGHT, stream)
        w.upload(T.FIELD_HEIGHT, (np.float32(10000) + np.float32(10000) * h).astype(np.float32), stream)
    pr = pressure_for(W, H, pseed)
    if pr is not None:
        w.set_asthenosphere(pr, stream)
    o = O.OracleWorld(s, w.download(T.FIELD_HEIGHT, stream), w.download(T.FIELD_PLATE_ID, stream), w.plates(stream),
                      1000 + gen)
    o.pressure = pr
    return w, o


def oracle_field(o, f):
    return {T.FIELD_HEIGHT: o.h, T.FIELD_WATER: o.w, T.FIELD_SEDIMENT: o.s, T.FIELD_FLUX: o.flux,
            T.FIELD_PLATE_ID: o.id, T.FIELD_LABELS: o.labels, T.FIELD_TYPE_BITMAP: o.bitmap,
            T.FIELD_DIV_BITMAP: o.div}[f]


def assert_same(w, o, stream, msg):
    for f in FIELDS:
        np.testing.assert_array_equal(w.download(f, stream), oracle_field(o, f), err_msg=f"{msg}: field {f}")
    np.testing.assert_array_equal(w.plates(stream), o.plates, err_msg=f"{msg}: plates")
    np.testing.assert_array_equal(w.plate_dynamics(stream), o.dyn, err_msg=f"{msg}: plate dynamics")


@pytest.mark.parametrize("kind", ["baseline", "reference"])
@pytest.mark.parametrize("W,H,pseed", [(64, 64, 5), (100, 60, None), (33, 17, 6), (256, 128, 7)])
def test_dynamics_match_oracle(stream, kind, W, H, pseed):
    s = settings(kind)
    w, o = make(s, W, H, 8, 3, pseed, stream, kind)
    v0 = w.plates(stream)["velocity"].copy()
    for step in range(6):
        w.step(1, stream)
        o.step(1)
        assert_same(w, o, stream, f"{kind} {W}x{H} step {step}")
    d = w.plate_dynamics(stream)
    assert (d["frictionLoss"] > 0).any(), "no plate met friction"
    assert not np.array_equal(w.plates(stream)["velocity"], v0), "velocities never changed"


def test_dynamics_in_a_mixed_batch_equal_alone(stream):
    s = settings()
    specs = [(64, 64, 6, 1, 11), (100, 60, 5, 2, None), (33, 17, 3, 3, 12), (128, 96, 9, 4, 13)]
    alone = [make(s, W, H, p, g, ps, stream)[0] for W, H, p, g, ps in specs]
    mixed = [make(s, W, H, p, g, ps, stream)[0] for W, H, p, g, ps in specs]
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
        np.testing.assert_array_equal(a.plates(stream), m.plates(stream), err_msg=f"world {i} plates")
        np.testing.assert_array_equal(a.plate_dynamics(stream), m.plate_dynamics(stream), err_msg=f"world {i} dyn")
    b.close()


def test_phase_calls_equal_the_step(stream):
    s = settings()
    a, _ = make(s, 96, 64, 7, 4, 8, stream)
    b, _ = make(s, 96, 64, 7, 4, 8, stream)
    for _ in range(3):
        a.step(1, stream)
        b.collide(stream)
        b.resolve(stream)
        b.thermal(s.step.thermalIterations, stream)
        b.hydraulic(s.step.hydraulicIterations, s.step.hydraulicDt, stream)
        b.finish(stream)
    for f in FIELDS:
        np.testing.assert_array_equal(a.download(f, stream), b.download(f, stream), err_msg=f"field {f}")
    np.testing.assert_array_equal(a.plate_dynamics(stream), b.plate_dynamics(stream))


def test_snapshot_resume_with_dynamics(tmp_path, stream):
    s = settings()
    a, _ = make(s, 80, 56, 6, 5, 9, stream)
    a.step(4, stream)
    p = tmp_path / "dyn.snap"
    a.save_snapshot(p, stream)
    b = T.World.from_snapshot(p, stream)
    a.step(4, stream)
    b.step(4, stream)
    for f in FIELDS:
        np.testing.assert_array_equal(a.download(f, stream), b.download(f, stream), err_msg=f"field {f}")
    np.testing.assert_array_equal(a.plates(stream), b.plates(stream))
    np.testing.assert_array_equal(a.plate_dynamics(stream), b.plate_dynamics(stream))


def test_unknown_dynamics_mode_is_refused(stream):
    s = settings()
    s.step.plateDynamics = 7
    w = T.World(s, 32, 32)
    w.init_synthetic(3, 1.0, 1, stream)
    with pytest.raises(T.TectoError):
        w.step(1, stream)
