"""The reference's world initialisation on the GPU (tecto_world_init_reference) against the oracle,
which the reference's own kernels pin (test_oracle_init.py): plate ids, heights, plate records and
CCL labels bit for bit, and the first steps of the initialised world."""
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


def settings(plates, gens):
    s = T.default_settings()
    s.step.upliftMode = T.UPLIFT_GAUSSIAN
    s.kernel.minCollisionSize = 3
    s.kernel.collisionTypeUpdateCooldown = 2
    s.sim.iterationsForCCL = 3
    s.sim.numStartingPlates = plates
    s.sim.numVoronoiGenerations = len(gens)
    for i, v in enumerate(gens):
        s.sim.numVoronoiSeeds[i] = v
    return s


@pytest.mark.parametrize("W,H,seed,plates,gens", [(96, 64, 1234, 12, (60, 150)), (50, 80, 7, 5, ()),
                                                  (512, 384, 42, 16, (200, 500)), (300, 200, 5, 30, (3000,))])
def test_init_matches_oracle(stream, W, H, seed, plates, gens):
    s = settings(plates, gens)
    w = T.World(s, W, H, seed=seed)
    w.init_reference(stream)
    sx, sy, sid, pl, dy = O.reference_seeds(W, H, seed, plates, gens)
    h, ids = O.init_reference(W, H, seed, sx, sy, sid)
    np.testing.assert_array_equal(w.download(T.FIELD_PLATE_ID, stream), ids)
    np.testing.assert_array_equal(w.download(T.FIELD_HEIGHT, stream), h)
    np.testing.assert_array_equal(w.plates(stream), pl)
    got = w.plate_dynamics(stream)
    for f in ("velocitySmoothed", "directionSmoothed_x", "directionSmoothed_y"):
        np.testing.assert_array_equal(got[f], dy[f])
    labels = np.zeros((H, W), np.uint32)
    O.lib().or_ccl(W, H, O._P(ids), O._P(labels), s.step.cclConnectivity)
    np.testing.assert_array_equal(w.download(T.FIELD_LABELS, stream), labels)
    assert w.iteration == 0
    assert not w.download(T.FIELD_WATER, stream).any()


def test_initialised_world_steps_like_the_oracle(stream):
    W, H, seed = 128, 96, 77
    s = settings(10, (80,))
    w = T.World(s, W, H, seed=seed)
    w.init_reference(stream)
    o = O.OracleWorld(s, w.download(T.FIELD_HEIGHT, stream), w.download(T.FIELD_PLATE_ID, stream), w.plates(stream),
                      seed)
    for step in range(4):
        w.step(1, stream)
        o.step(1)
        np.testing.assert_array_equal(w.download(T.FIELD_PLATE_ID, stream), o.id, err_msg=f"ids step {step}")
        np.testing.assert_array_equal(w.download(T.FIELD_HEIGHT, stream), o.h, err_msg=f"heights step {step}")


@pytest.mark.parametrize("spacing", [0.0, 0.001])
def test_server_admits_reference_initialised_worlds(stream, spacing):
    """Served requests initialised with the reference's initialisation give the same worlds as
    initialising and stepping them directly.  Each request has its own plate count, a field the
    initialisation alone reads; with all arrivals at t = 0 the three worlds share the batch."""
    s = settings(1, (40,))
    reqs = [T.Request(width=W, height=H, plates=p, steps=st, velRange=1.0, genSeed=0, worldSeed=500 + i,
                      arrival_s=spacing * i)
            for i, (W, H, p, st) in enumerate([(64, 64, 6, 3), (96, 48, 4, 2), (80, 80, 9, 4)])]
    sv = T.Server(s, 3 * T.world_bytes(96, 80), max_worlds=3)
    sv.set_init(T.SERVER_INIT_REFERENCE)
    res, st = sv.run_trace(reqs, stream)
    assert st.completed == 3, [(r.status, r.admit_s, r.finish_s, T.lib().tecto_last_error_string()) for r in res]
    for i, q in enumerate(reqs):
        ws = settings(q.plates, (40,))
        w = T.World(ws, q.width, q.height, seed=q.worldSeed)
        w.init_reference(stream)
        w.step(q.steps, stream)
        assert np.float32(w.download(T.FIELD_HEIGHT, stream).astype(np.float64).sum()) == res[i].height_checksum
    sv.close()


def test_initialize_with_arguments(stream):
    """tecto_world_init(world, plates, generations): initialize(numStartingPlates, numVoronoiSeeds)."""
    import ctypes as C
    s = T.default_settings()
    a = T.World(s, 80, 60, seed=11)
    b = T.World(s, 80, 60, seed=11)
    gens = (C.c_int * 2)(30, 70)
    T.check(T.lib().tecto_world_init(a.ptr, 6, gens, 2, stream.cuda_stream), "tecto_world_init")
    s2 = s.copy()
    s2.sim.numStartingPlates, s2.sim.numVoronoiGenerations = 6, 2
    s2.sim.numVoronoiSeeds[0], s2.sim.numVoronoiSeeds[1] = 30, 70
    b.set_settings(s2)
    b.init_reference(stream)
    for f in (T.FIELD_HEIGHT, T.FIELD_PLATE_ID, T.FIELD_LABELS):
        np.testing.assert_array_equal(a.download(f, stream), b.download(f, stream))
    np.testing.assert_array_equal(a.plates(stream), b.plates(stream))
    with pytest.raises(T.TectoError):
        T.check(T.lib().tecto_world_init(a.ptr, 0, gens, 2, stream.cuda_stream), "tecto_world_init")


def test_batch_joins_worlds_initialised_differently(stream):
    """Worlds whose settings differ only in initialisation fields share a batch; a world whose step
    settings differ is refused."""
    a = T.World(settings(6, (40,)), 64, 48, seed=1)
    b = T.World(settings(9, (30, 70)), 64, 48, seed=2)
    a.init_reference(stream)
    b.init_reference(stream)
    bt = T.Batch()
    bt.add(a, stream)
    bt.add(b, stream)
    bt.step(2, stream)
    stream.synchronize()
    bt.check(stream)
    c_settings = settings(6, (40,))
    c_settings.kernel.gravity = 9.0
    c = T.World(c_settings, 64, 48, seed=3)
    c.init_reference(stream)
    with pytest.raises(T.TectoError):
        bt.add(c, stream)
    bt.close()
    for w in (a, b, c):
        w.close()
