"""Batches and the server on the GPU: each world's result is the same alone and in a mixed batch
(uneven sizes, worlds joining and leaving mid-flight, different ping-pong parity at join), the
device-side generator equals the host generator, and the server's continuous batching returns the
same worlds as serving the requests one at a time."""
from __future__ import annotations

import numpy as np
import pytest

import master_thesis_gb300 as T
import oracle as O

pytestmark = pytest.mark.gpu

FIELDS = (T.FIELD_HEIGHT, T.FIELD_WATER, T.FIELD_SEDIMENT, T.FIELD_FLUX, T.FIELD_PLATE_ID, T.FIELD_LABELS,
          T.FIELD_TYPE_BITMAP, T.FIELD_DIV_BITMAP, T.FIELD_ACCRETION)

SPECS = [(64, 64, 8, 1), (100, 60, 5, 2), (33, 17, 3, 3), (128, 32, 6, 4), (200, 150, 12, 5), (256, 128, 9, 6)]


@pytest.fixture(scope="module")
def stream():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available(), "a CUDA GPU is required"
    return torch.cuda.Stream()


def settings(tile=0):
    s = T.baseline_settings()
    s.kernel.minCollisionSize = 3
    s.kernel.collisionTypeUpdateCooldown = 2
    s.sim.iterationsForCCL = 3
    s.step.hydraulicTile = tile
    s.step.thermalTile = 5 if tile == 9 else 0  # the marching kernels together
    return s


def make(spec, s):
    W, H, plates, seed = spec
    w = T.World(s, W, H, seed=1000 + seed)
    w.init_synthetic(plates, 1.0, seed)
    return w


def assert_same(a: T.World, b: T.World, msg):
    for f in FIELDS:
        np.testing.assert_array_equal(a.download(f), b.download(f), err_msg=f"{msg}: field {f}")
    np.testing.assert_array_equal(a.plates(), b.plates(), err_msg=f"{msg}: plates")
    assert a.iteration == b.iteration


@pytest.mark.parametrize("tile", [4, 9])
def test_batch_equals_alone_with_joins_and_leaves(stream, tile):
    """Tiles (hydraulic variant 4) and the marching kernels (hydraulic 9, thermal 5), whose strip
    table and persistent block ranges are rebuilt at every membership change."""
    s = settings(tile)
    alone = [make(sp, s) for sp in SPECS]
    mixed = [make(sp, s) for sp in SPECS]
    # a world stepped alone first joins the batch with other ping-pong halves than the batch's
    mixed[3].step(1, stream)
    alone[3].step(1, stream)
    b = T.Batch()
    for w in mixed[:3]:
        b.add(w, stream)
    b.step(2, stream)
    for w in mixed[3:]:
        b.add(w, stream)
    b.step(3, stream)
    b.remove(mixed[1])
    b.step(4, stream)  # the first 8 worlds' counters now differ: CCL due per world
    stream.synchronize()
    b.check(stream)
    # steps each world took in the batch (world 3 also took one step alone before joining, which
    # its alone copy mirrored above)
    steps = [9, 5, 9, 7, 7, 7]
    for w, n in zip(alone, steps):
        w.step(n, stream)
    stream.synchronize()
    for i, (a, m) in enumerate(zip(alone, mixed)):
        assert_same(a, m, f"world {i} {SPECS[i]}")
    assert b.size() == (5, sum(sp[0] * sp[1] for k, sp in enumerate(SPECS) if k != 1))
    b.close()


def test_batch_matches_oracle(stream):
    s = settings()
    worlds = [make(sp, s) for sp in SPECS[:4]]
    oracles = [O.OracleWorld(s, w.download(T.FIELD_HEIGHT), w.download(T.FIELD_PLATE_ID), w.plates(),
                             1000 + sp[3]) for w, sp in zip(worlds, SPECS)]
    b = T.Batch()
    for w in worlds:
        b.add(w, stream)
    b.step(4, stream)
    stream.synchronize()
    for w, o in zip(worlds, oracles):
        o.step(4)
        np.testing.assert_array_equal(w.download(T.FIELD_PLATE_ID), o.id)
        np.testing.assert_array_equal(w.download(T.FIELD_LABELS), o.labels)
        np.testing.assert_array_equal(w.download(T.FIELD_HEIGHT), o.h)
        np.testing.assert_array_equal(w.download(T.FIELD_WATER), o.w)
        np.testing.assert_array_equal(w.download(T.FIELD_SEDIMENT), o.s)
    b.close()


@pytest.mark.parametrize("W,H,P", [(64, 64, 8), (300, 170, 12), (1024, 512, 48), (17, 33, 3)])
def test_device_generator_matches_host(W, H, P):
    w = T.World(T.baseline_settings(), W, H)
    w.init_synthetic_device(P, 1.0, 77)
    h, ids, pl = T.generate_world(W, H, P, 1.0, 77)
    np.testing.assert_array_equal(w.download(T.FIELD_HEIGHT), h)
    np.testing.assert_array_equal(w.download(T.FIELD_PLATE_ID), ids)
    np.testing.assert_array_equal(w.plates(), pl)


def test_server_continuous_batching_matches_one_at_a_time(stream):
    rng = np.random.default_rng(3)
    sizes = [(32, 32), (64, 64), (96, 64), (128, 128), (48, 96)]
    reqs = []
    for i in range(16):
        W, H = sizes[rng.integers(0, len(sizes))]
        reqs.append(T.Request(width=W, height=H, plates=int(rng.integers(3, 12)), steps=int(rng.integers(1, 9)),
                              velRange=1.0, genSeed=100 + i, worldSeed=2000 + i, arrival_s=0.002 * i))
    budget = 6 * T.world_bytes(128, 128)
    sv = T.Server(settings(), budget, max_worlds=8)
    res_c, st_c = sv.run_trace(reqs, stream)
    res_s, st_s = sv.run_trace_sequential(reqs, stream)
    assert st_c.completed == st_s.completed == 16
    assert st_c.peak_bytes <= budget
    for i, (a, b) in enumerate(zip(res_c, res_s)):
        assert a.status == b.status == 0
        assert a.height_checksum == b.height_checksum, f"request {i}"
    # one request served directly through the plain API
    q = reqs[5]
    w = T.World(settings(), q.width, q.height, seed=q.worldSeed)
    w.init_synthetic_device(q.plates, q.velRange, q.genSeed)
    w.step(q.steps, stream)
    stream.synchronize()
    assert np.float32(w.download(T.FIELD_HEIGHT).astype(np.float64).sum()) == res_c[5].height_checksum
    sv.close()


def test_size_aware_admission_on_the_gpu(stream):
    """Two heavy requests (2^20 cells) and light ones arriving together: the heavy ones run one
    after the other in arrival order while the light ones ride along, and every request's world
    equals the one-at-a-time path's."""
    reqs = [T.Request(width=1024, height=1024, plates=8, steps=3, velRange=1.0, genSeed=700, worldSeed=7000,
                      arrival_s=0.0),
            T.Request(width=2048, height=512, plates=6, steps=2, velRange=1.0, genSeed=701, worldSeed=7001,
                      arrival_s=0.0)]
    reqs += [T.Request(width=96, height=64, plates=5, steps=2 + i % 3, velRange=1.0, genSeed=710 + i,
                       worldSeed=7100 + i, arrival_s=0.0) for i in range(6)]
    sv = T.Server(settings(), 3 * T.world_bytes(2048, 512))
    res_c, st_c = sv.run_trace(reqs, stream)
    res_s, _ = sv.run_trace_sequential(reqs, stream)
    assert st_c.completed == 8
    assert res_c[1].admit_s >= res_c[0].finish_s                 # heavy requests one at a time
    assert all(r.admit_s < res_c[0].finish_s for r in res_c[2:])  # the light ones ride along
    for i, (a, b) in enumerate(zip(res_c, res_s)):
        assert a.status == b.status == 0 and a.height_checksum == b.height_checksum, f"request {i}"
    sv.close()


def test_live_serving_matches_the_trace_replay(stream):
    """Requests submitted one by one while earlier ones are mid-flight, ticks driven by the caller:
    every ticket's final world equals the trace replay's and the one-at-a-time path's."""
    rng = np.random.default_rng(4)
    sizes = [(32, 32), (64, 64), (96, 64), (128, 128), (48, 96)]
    reqs = []
    for i in range(12):
        W, H = sizes[rng.integers(0, len(sizes))]
        reqs.append(T.Request(width=W, height=H, plates=int(rng.integers(3, 12)), steps=int(rng.integers(0, 8)),
                              velRange=1.0, genSeed=300 + i, worldSeed=4000 + i, arrival_s=0.0))
    budget = 4 * T.world_bytes(128, 128)
    sv = T.Server(settings(), budget, max_worlds=5)
    res_s, _ = sv.run_trace_sequential(reqs, stream)
    tickets = []
    for i, q in enumerate(reqs):  # three submissions per tick
        tickets.append(sv.submit(q))
        if i % 3 == 2:
            sv.tick(stream)
    sv.drain(stream)
    st = sv.live_stats()
    assert st.completed == len(reqs) and st.peak_bytes <= budget and st.max_active <= 5
    for i, t in enumerate(tickets):
        state, r = sv.poll(t)
        assert state == T.REQUEST_DONE and r.status == 0
        assert r.height_checksum == res_s[i].height_checksum, f"request {i}"
    res_c, _ = sv.run_trace(reqs, stream)  # the same server replays a trace once nothing is pending
    assert [r.height_checksum for r in res_c] == [r.height_checksum for r in res_s]
    sv.close()


def test_async_field_copies_round_trip(stream):
    """tecto_world_upload_async / download_async are stream-ordered: upload, step, download and
    one wait give the same fields as the synchronous calls."""
    torch = pytest.importorskip("torch")
    s = settings()
    a, b = make(SPECS[4], s), make(SPECS[4], s)
    W, H = SPECS[4][0], SPECS[4][1]
    rng = np.random.default_rng(2)
    water = torch.from_numpy(np.abs(rng.normal(0, 0.1, (H, W))).astype(np.float32)).pin_memory()
    out = torch.empty((H, W), dtype=torch.float32).pin_memory()
    L = T.lib()
    sp = stream.cuda_stream
    T.check(L.tecto_world_upload_async(a.ptr, T.FIELD_WATER, water.data_ptr(), W * H * 4, sp), "upload_async")
    a.step(2, stream)
    T.check(L.tecto_world_download_async(a.ptr, T.FIELD_WATER, out.data_ptr(), W * H * 4, sp), "download_async")
    stream.synchronize()
    b.upload(T.FIELD_WATER, water.numpy())
    b.step(2, stream)
    stream.synchronize()
    np.testing.assert_array_equal(out.numpy(), b.download(T.FIELD_WATER))
    with pytest.raises(T.TectoError):
        T.check(L.tecto_world_upload_async(a.ptr, T.FIELD_WATER, water.data_ptr(), 12, sp), "upload_async")


def test_packed_transfers_equal_per_world_copies(stream):
    """tecto_batch_upload_async / download_async: one packed host buffer per field for all worlds
    gives the same state as copies world by world."""
    torch = pytest.importorskip("torch")
    s = settings()
    a = [make(sp, s) for sp in SPECS]
    b = [make(sp, s) for sp in SPECS]
    ba, bb = T.Batch(), T.Batch()
    for w in a:
        ba.add(w, stream)
    for w in b:
        bb.add(w, stream)
    ba.step(2, stream)
    bb.step(2, stream)
    stream.synchronize()
    rng = np.random.default_rng(9)
    offs = bb.offsets()
    assert offs[-1] == sum(w.W * w.H for w in b)
    fields = {T.FIELD_HEIGHT: np.float32, T.FIELD_WATER: np.float32, T.FIELD_SEDIMENT: np.float32,
              T.FIELD_FLUX: np.float32, T.FIELD_PLATE_ID: np.uint8}
    for f, dt in fields.items():
        per = [(rng.random(w.download(f).shape) * 3).astype(dt) for w in a]
        for w, v in zip(a, per):
            w.upload(f, v, stream)
        packed = torch.from_numpy(np.concatenate([v.ravel() for v in per])).pin_memory()
        bb.upload_packed_async(f, packed.data_ptr(), packed.numel() * packed.element_size(), stream)
    stream.synchronize()
    ba.step(3, stream)
    bb.step(3, stream)
    for f in (T.FIELD_HEIGHT, T.FIELD_WATER, T.FIELD_FLUX, T.FIELD_PLATE_ID, T.FIELD_LABELS):
        out = torch.empty(int(offs[-1]) * (16 if f == T.FIELD_FLUX else 1 if f == T.FIELD_PLATE_ID else 4),
                          dtype=torch.uint8).pin_memory()
        bb.download_packed_async(f, out.data_ptr(), out.numel(), stream)
        stream.synchronize()
        got = out.numpy()
        for i, w in enumerate(a):
            ref = w.download(f).ravel().view(np.uint8)
            esz = ref.size // (w.W * w.H)
            np.testing.assert_array_equal(got[offs[i] * esz: offs[i + 1] * esz], ref, err_msg=f"world {i} field {f}")
    with pytest.raises(T.TectoError):
        bb.upload_packed_async(T.FIELD_HEIGHT, packed.data_ptr(), 12, stream)
    ba.close()
    bb.close()


def test_pipelined_transfers_equal_plain_ones(stream):
    """Staged uploads and gathered downloads on a second stream (tecto_batch_stage_upload_async /
    commit_upload / gather_download / fetch_download_async) give the same worlds and results as
    the single-stream packed calls, step after step with new inputs each step."""
    torch = pytest.importorskip("torch")
    s = settings()
    a = [make(sp, s) for sp in SPECS]
    b = [make(sp, s) for sp in SPECS]
    ba, bb = T.Batch(), T.Batch()
    for w in a:
        ba.add(w, stream)
    for w in b:
        bb.add(w, stream)
    L = T.lib()
    copy = torch.cuda.Stream()
    cs, ss = copy.cuda_stream, stream.cuda_stream
    total = int(bb.offsets()[-1])
    rng = np.random.default_rng(4)
    inputs = [torch.from_numpy((rng.random(total) * 2).astype(np.float32)).pin_memory() for _ in range(3)]
    outs_a = [torch.empty(total, dtype=torch.float32).pin_memory() for _ in range(3)]
    outs_b = [torch.empty(total, dtype=torch.float32).pin_memory() for _ in range(3)]
    nb = total * 4
    T.check(L.tecto_batch_stage_upload_async(bb.ptr, T.FIELD_WATER, inputs[0].data_ptr(), nb, cs), "stage")
    for k in range(3):
        # plain packed path
        ba.upload_packed_async(T.FIELD_WATER, inputs[k].data_ptr(), nb, stream)
        ba.step(1, stream)
        ba.download_packed_async(T.FIELD_HEIGHT, outs_a[k].data_ptr(), nb, stream)
        # pipelined path: the next step's input is staged while this step runs
        T.check(L.tecto_batch_commit_upload(bb.ptr, T.FIELD_WATER, ss), "commit")
        if k + 1 < 3:
            T.check(L.tecto_batch_stage_upload_async(bb.ptr, T.FIELD_WATER, inputs[k + 1].data_ptr(), nb, cs),
                    "stage")
        bb.step(1, stream)
        T.check(L.tecto_batch_gather_download(bb.ptr, T.FIELD_HEIGHT, ss), "gather")
        T.check(L.tecto_batch_fetch_download_async(bb.ptr, T.FIELD_HEIGHT, outs_b[k].data_ptr(), nb, cs), "fetch")
    stream.synchronize()
    copy.synchronize()
    for k in range(3):
        np.testing.assert_array_equal(outs_a[k].numpy(), outs_b[k].numpy(), err_msg=f"step {k}")
    for wa, wb in zip(a, b):
        np.testing.assert_array_equal(wa.download(T.FIELD_WATER), wb.download(T.FIELD_WATER))
    ba.close()
    bb.close()


def test_pipelined_transfers_two_steps_ahead(stream):
    """Each field's two staging buffers per direction let uploads run two steps ahead of their
    commits, on their own copy stream, with downloads on another: five steps of new inputs give the
    same results as the single-stream packed calls.  A third stage without a commit, a commit with
    nothing staged and a fetch with nothing gathered are refused."""
    torch = pytest.importorskip("torch")
    s = settings()
    a = [make(sp, s) for sp in SPECS]
    b = [make(sp, s) for sp in SPECS]
    ba, bb = T.Batch(), T.Batch()
    for w in a:
        ba.add(w, stream)
    for w in b:
        bb.add(w, stream)
    L = T.lib()
    up, down = torch.cuda.Stream(), torch.cuda.Stream()
    us, ds, ss = up.cuda_stream, down.cuda_stream, stream.cuda_stream
    total = int(bb.offsets()[-1])
    rng = np.random.default_rng(5)
    n = 5
    inputs = [torch.from_numpy((rng.random(total) * 2).astype(np.float32)).pin_memory() for _ in range(n)]
    ids_in = [torch.from_numpy(rng.integers(0, 6, total).astype(np.uint8)).pin_memory() for _ in range(n)]
    outs_a = [torch.empty(total, dtype=torch.float32).pin_memory() for _ in range(n)]
    outs_b = [torch.empty(total, dtype=torch.float32).pin_memory() for _ in range(n)]
    nb = total * 4

    def stage(k):
        T.check(L.tecto_batch_stage_upload_async(bb.ptr, T.FIELD_WATER, inputs[k].data_ptr(), nb, us), "stage")
        T.check(L.tecto_batch_stage_upload_async(bb.ptr, T.FIELD_PLATE_ID, ids_in[k].data_ptr(), total, us), "stage")

    stage(0)
    stage(1)
    assert L.tecto_batch_stage_upload_async(bb.ptr, T.FIELD_WATER, inputs[2].data_ptr(), nb, us) == -1  # TECTO_ERR_INVALID
    for k in range(n):
        ba.upload_packed_async(T.FIELD_WATER, inputs[k].data_ptr(), nb, stream)
        ba.upload_packed_async(T.FIELD_PLATE_ID, ids_in[k].data_ptr(), total, stream)
        ba.step(1, stream)
        ba.download_packed_async(T.FIELD_HEIGHT, outs_a[k].data_ptr(), nb, stream)
        T.check(L.tecto_batch_commit_upload(bb.ptr, T.FIELD_WATER, ss), "commit")
        T.check(L.tecto_batch_commit_upload(bb.ptr, T.FIELD_PLATE_ID, ss), "commit")
        if k + 2 < n:
            stage(k + 2)
        bb.step(1, stream)
        T.check(L.tecto_batch_gather_download(bb.ptr, T.FIELD_HEIGHT, ss), "gather")
        T.check(L.tecto_batch_fetch_download_async(bb.ptr, T.FIELD_HEIGHT, outs_b[k].data_ptr(), nb, ds), "fetch")
    assert L.tecto_batch_commit_upload(bb.ptr, T.FIELD_WATER, ss) == -1  # TECTO_ERR_INVALID
    assert L.tecto_batch_fetch_download_async(bb.ptr, T.FIELD_HEIGHT, outs_b[0].data_ptr(), nb, ds) == -1  # TECTO_ERR_INVALID
    stream.synchronize()
    up.synchronize()
    down.synchronize()
    for k in range(n):
        np.testing.assert_array_equal(outs_a[k].numpy(), outs_b[k].numpy(), err_msg=f"step {k}")
    for wa, wb in zip(a, b):
        for f in (T.FIELD_WATER, T.FIELD_PLATE_ID, T.FIELD_HEIGHT):
            np.testing.assert_array_equal(wa.download(f), wb.download(f))
    ba.close()
    bb.close()
