"""Image export and snapshots on the GPU: the exported PNGs decode to the reference's conversions
(the oracle's, which the golden vectors pin, and the reference's own kernels run on this GPU where
their cubin was built), and a world resumed from a snapshot steps bit-identically to the world
that saved it."""
from __future__ import annotations

import numpy as np
import pytest

import master_thesis_gb300 as T
import oracle as O
from conftest import decode_png

pytestmark = pytest.mark.gpu

FIELDS = (T.FIELD_HEIGHT, T.FIELD_WATER, T.FIELD_SEDIMENT, T.FIELD_FLUX, T.FIELD_PLATE_ID, T.FIELD_LABELS,
          T.FIELD_TYPE_BITMAP, T.FIELD_DIV_BITMAP, T.FIELD_COLLISION)


@pytest.fixture(scope="module")
def stream():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available(), "a CUDA GPU is required"
    return torch.cuda.Stream()


def world(W, H, mode=T.UPLIFT_GAUSSIAN, steps=3, stream=None):
    s = T.baseline_settings()
    s.step.upliftMode = mode
    s.sim.iterationsForCCL = 2
    s.kernel.minCollisionSize = 3
    s.kernel.collisionTypeUpdateCooldown = 2
    w = T.World(s, W, H, seed=77)
    w.init_synthetic(9, 1.5, 5, stream)
    if steps:
        w.step(steps, stream)
    return w, s


@pytest.mark.parametrize("shape", [(96, 64), (100, 37), (2048, 512)])
def test_height_export_gray16(tmp_path, stream, shape):
    W, H = shape
    w, s = world(W, H, stream=stream)
    h = w.download(T.FIELD_HEIGHT, stream)
    lo, hi = float(np.min(h)) + 0.1 * float(np.ptp(h)), float(np.max(h)) - 0.1 * float(np.ptp(h))
    p = tmp_path / "h.png"
    w.export_png(T.EXPORT_HEIGHT_GRAY16, p, lo, hi, stream)
    px, chunks = decode_png(p.read_bytes())
    assert chunks == ["IHDR", "sRGB", "IDAT", "IEND"]
    np.testing.assert_array_equal(px, O.gray16(h, lo, hi))
    assert px.min() == 0 and px.max() == 65535  # the range clips both ends


@pytest.mark.parametrize("shape", [(96, 64), (100, 37)])
def test_plate_export_rgb(tmp_path, stream, golden, shape):
    W, H = shape
    w, _ = world(W, H, stream=stream)
    ids = w.download(T.FIELD_PLATE_ID, stream)
    p = tmp_path / "ids.png"
    w.export_png(T.EXPORT_PLATES_RGB, p, stream=stream)
    px, chunks = decode_png(p.read_bytes())
    assert chunks == ["IHDR", "IDAT", "IEND"]
    np.testing.assert_array_equal(px, golden("ref_export")["rgb"].reshape(256, 3)[ids])


def test_exports_equal_reference_kernels_on_gpu(tmp_path, stream):
    """The reference's own convertFloatToGray16Kernel and convertGrayscaleToRgbKernel, compiled for
    sm_103a from its sources, on the same world."""
    if not O.REF_EXPORT_CUBIN.exists():
        pytest.skip("the reference's export kernels were not built here")
    w, s = world(256, 128, stream=stream)
    h = w.download(T.FIELD_HEIGHT, stream)
    ids = w.download(T.FIELD_PLATE_ID, stream)
    lo, hi = float(np.percentile(h, 5)), float(np.percentile(h, 95))
    w.export_png(T.EXPORT_HEIGHT_GRAY16, tmp_path / "h.png", lo, hi, stream)
    w.export_png(T.EXPORT_PLATES_RGB, tmp_path / "ids.png", stream=stream)
    np.testing.assert_array_equal(decode_png((tmp_path / "h.png").read_bytes())[0], O.ref_gpu_gray16(h, lo, hi))
    np.testing.assert_array_equal(decode_png((tmp_path / "ids.png").read_bytes())[0], O.ref_gpu_ids_rgb(ids))
    all_ids = np.arange(256, dtype=np.uint8).reshape(16, 16)
    np.testing.assert_array_equal(O.ref_gpu_ids_rgb(all_ids).reshape(256, 3), T.plate_palette())


def test_export_rejects_bad_arguments(tmp_path, stream):
    w, _ = world(32, 32, steps=0, stream=stream)
    with pytest.raises(T.TectoError):
        w.export_png(T.EXPORT_HEIGHT_GRAY16, tmp_path / "x.png", 1.0, 1.0, stream)  # empty range
    with pytest.raises(T.TectoError):
        w.export_png(5, tmp_path / "x.png", 0.0, 1.0, stream)
    with pytest.raises(T.TectoError):
        w.export_png(T.EXPORT_PLATES_RGB, tmp_path / "no_such_dir" / "x.png", stream=stream)


@pytest.mark.parametrize("mode", [T.UPLIFT_GAUSSIAN, T.UPLIFT_REFERENCE])
def test_snapshot_resume_is_bit_identical(tmp_path, stream, mode):
    a, s = world(120, 72, mode=mode, steps=3, stream=stream)
    p = tmp_path / "world.snap"
    a.save_snapshot(p, stream)
    W, H, s2 = T.snapshot_info(p)
    assert (W, H) == (120, 72) and s2.step.upliftMode == mode
    b = T.World.from_snapshot(p, stream)
    assert b.iteration == a.iteration == 3
    np.testing.assert_array_equal(a.plates(stream), b.plates(stream))
    a.step(5, stream)
    b.step(5, stream)
    for f in FIELDS:
        np.testing.assert_array_equal(a.download(f, stream), b.download(f, stream), err_msg=f"field {f}")
    np.testing.assert_array_equal(a.plates(stream), b.plates(stream))
    assert a.iteration == b.iteration == 8


def test_snapshot_size_mismatch(tmp_path, stream):
    a, s = world(64, 48, steps=1, stream=stream)
    p = tmp_path / "w.snap"
    a.save_snapshot(p, stream)
    other = T.World(s, 48, 64)
    with pytest.raises(T.TectoError):
        other.load_snapshot(p, stream)
    p.write_bytes(p.read_bytes()[:-1])  # truncated
    with pytest.raises(T.TectoError):
        T.World(s, 64, 48).load_snapshot(p, stream)


def test_server_writes_finished_requests(tmp_path, stream):
    """Served results written headless: every finished request leaves its two PNGs and a snapshot;
    continuous batching and one-at-a-time serving write identical files, and the snapshot resumes
    the request's final world."""
    s = T.baseline_settings()
    s.sim.iterationsForCCL = 3
    reqs = [T.Request(width=W, height=H, plates=p, steps=st, velRange=1.0, genSeed=300 + i, worldSeed=900 + i,
                      arrival_s=0.001 * i)
            for i, (W, H, p, st) in enumerate([(64, 64, 6, 3), (96, 48, 4, 5), (33, 17, 3, 2), (128, 64, 9, 4)])]
    what = T.SERVER_OUT_HEIGHT_PNG | T.SERVER_OUT_PLATES_PNG | T.SERVER_OUT_SNAPSHOT
    dirs = {}
    for name in ("continuous", "sequential"):
        d = tmp_path / name
        d.mkdir()
        sv = T.Server(s, 4 * T.world_bytes(128, 64), max_worlds=4)
        sv.set_output(d, what, -500.0, 500.0)
        res, st = (sv.run_trace if name == "continuous" else sv.run_trace_sequential)(reqs, stream)
        assert st.completed == len(reqs) and all(r.status == 0 for r in res)
        sv.close()
        dirs[name] = d
    for i, q in enumerate(reqs):
        for suffix in ("_height.png", "_plates.png", ".snap"):
            a = (dirs["continuous"] / f"request_{i}{suffix}").read_bytes()
            assert a == (dirs["sequential"] / f"request_{i}{suffix}").read_bytes(), f"request {i}{suffix}"
        w = T.World.from_snapshot(dirs["continuous"] / f"request_{i}.snap", stream)
        assert w.iteration == q.steps
        h = w.download(T.FIELD_HEIGHT, stream)
        assert np.float32(h.astype(np.float64).sum()) == res[i].height_checksum
        px, _ = decode_png((dirs["continuous"] / f"request_{i}_height.png").read_bytes())
        np.testing.assert_array_equal(px, O.gray16(h, -500.0, 500.0))
        px, _ = decode_png((dirs["continuous"] / f"request_{i}_plates.png").read_bytes())
        np.testing.assert_array_equal(px, T.plate_palette()[w.download(T.FIELD_PLATE_ID, stream)])


def test_live_server_writes_finished_tickets(tmp_path, stream):
    """Live serving writes each finished ticket's files, named by ticket, byte-identical to the
    files a trace replay writes for the same requests."""
    s = T.baseline_settings()
    reqs = [T.Request(width=W, height=H, plates=p, steps=st, velRange=1.0, genSeed=500 + i, worldSeed=700 + i,
                      arrival_s=0.0)
            for i, (W, H, p, st) in enumerate([(64, 32, 5, 2), (40, 40, 4, 3), (96, 64, 7, 0)])]
    what = T.SERVER_OUT_HEIGHT_PNG | T.SERVER_OUT_SNAPSHOT
    live, trace = tmp_path / "live", tmp_path / "trace"
    live.mkdir()
    trace.mkdir()
    sv = T.Server(s, 2 * T.world_bytes(96, 64), max_worlds=2)
    sv.set_output(live, what, -500.0, 500.0)
    tickets = [sv.submit(q) for q in reqs]
    sv.drain(stream)
    assert all(sv.poll(t)[0] == T.REQUEST_DONE and sv.poll(t)[1].status == 0 for t in tickets)
    sv.set_output(trace, what, -500.0, 500.0)
    res, st = sv.run_trace(reqs, stream)
    assert st.completed == len(reqs)
    sv.close()
    for t in tickets:
        for suffix in ("_height.png", ".snap"):
            assert (live / f"request_{t}{suffix}").read_bytes() == (trace / f"request_{t}{suffix}").read_bytes()


def test_server_output_to_a_missing_directory_fails_the_request(tmp_path, stream):
    sv = T.Server(T.baseline_settings(), T.world_bytes(64, 64) * 2, max_worlds=2)
    sv.set_output(tmp_path / "missing", T.SERVER_OUT_SNAPSHOT)
    res, st = sv.run_trace([T.Request(width=32, height=32, plates=3, steps=1, velRange=1.0, genSeed=1,
                                      worldSeed=1, arrival_s=0.0)], stream)
    assert res[0].status == T.TectoError(-1, "").code
    sv.close()
