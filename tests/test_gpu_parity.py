"""Engine (CUDA, through the C ABI) against the CPU oracle, phase by phase and step by step.

Integer results (advection, sorted pairs, arrival words, plate ids, pair bitmaps, accretion marks,
CCL labels) must be bit-exact.  FP32 fields must stay within 1e-5 of the field's range per step
and within 1e-3 of the range after 100 steps; the engine and the oracle evaluate the same IEEE
operations in the same order, so in practice they agree bit for bit, which the tests report.
"""
from __future__ import annotations

import numpy as np
import pytest

import master_thesis_gb300 as T
import oracle as O
from conftest import fp_tol

pytestmark = pytest.mark.gpu

SIZES = [(64, 64), (100, 60), (33, 17), (256, 128)]


@pytest.fixture(scope="module")
def torch_stream():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available(), "a CUDA GPU is required"
    return torch.cuda.Stream()


def make_settings(kind: str) -> T.Settings:
    if kind == "baseline":
        s = T.baseline_settings()
    else:
        s = T.default_settings()
        s.step.upliftMode = T.UPLIFT_GAUSSIAN
    s.kernel.minCollisionSize = 3          # small grids: let pairs get typed quickly
    s.kernel.collisionTypeUpdateCooldown = 2
    s.sim.iterationsForCCL = 3
    return s


def make_world(kind, W, H, plates=8, vel=1.0, gen=7):
    s = make_settings(kind)
    w = T.World(s, W, H, seed=1000)
    w.init_synthetic(plates, vel, gen)
    if kind == "reference":  # reference height scale (metres)
        h = w.download(T.FIELD_HEIGHT)
        w.upload(T.FIELD_HEIGHT, (np.float32(10000) + np.float32(10000) * h).astype(np.float32))
    return s, w


def assert_fp(name, got, want, step, report):
    tol = fp_tol(want)
    d = float(np.max(np.abs(got.astype(np.float64) - want.astype(np.float64)))) if got.size else 0.0
    report.setdefault(name, []).append(d)
    assert d <= tol, f"{name} step {step}: max |diff| {d} > {tol}"


@pytest.mark.parametrize("kind", ["baseline", "reference"])
@pytest.mark.parametrize("W,H", SIZES)
def test_phases_match_oracle(kind, W, H):
    st, w = make_world(kind, W, H)
    h = w.download(T.FIELD_HEIGHT)
    ids = w.download(T.FIELD_PLATE_ID)
    pl = w.plates()
    water = np.zeros((H, W), np.float32)
    sed = np.zeros((H, W), np.float32)
    flux = np.zeros((H, W, 4), np.float32)
    bm = np.zeros(T.NUM_PAIRS, np.uint8)
    div = np.zeros(T.NUM_DIV_WORDS, np.uint32)
    report = {}
    for it in range(5):
        # collide: offsets, advection + sort, words, types
        offx, offy, nxt = O.plate_offsets(pl)
        dest, word, sk, sv = O.collision_words(ids, offx, offy)
        bm = O.collision_types(word, h, offx, offy, st, bm)
        w.collide()
        np.testing.assert_array_equal(w.download(T.FIELD_SORT_KEYS).ravel(), sk, err_msg=f"sorted keys {it}")
        np.testing.assert_array_equal(w.download(T.FIELD_SORT_VALS).ravel(), sv, err_msg=f"sorted values {it}")
        np.testing.assert_array_equal(w.download(T.FIELD_COLLISION), word, err_msg=f"words {it}")
        np.testing.assert_array_equal(w.download(T.FIELD_TYPE_BITMAP), bm, err_msg=f"bitmap {it}")
        np.testing.assert_array_equal(w.plates(), nxt, err_msg=f"plate centres {it}")
        # resolve (+ Gaussian uplift)
        hn, idn, acc, div = O.resolve(ids, h, word, offx, offy, bm, div, st, 1000, it)
        w.resolve()
        np.testing.assert_array_equal(w.download(T.FIELD_PLATE_ID), idn, err_msg=f"resolved ids {it}")
        np.testing.assert_array_equal(w.download(T.FIELD_DIV_BITMAP), div, err_msg=f"div bitmap {it}")
        assert_fp("resolve.h", w.download(T.FIELD_HEIGHT), hn, it, report)
        hn = w.download(T.FIELD_HEIGHT)  # continue from the engine's state (same within tol)
        # thermal
        ht = O.thermal(hn, st.step.thermalIterations, st)
        w.thermal(st.step.thermalIterations)
        assert_fp("thermal.h", w.download(T.FIELD_HEIGHT), ht, it, report)
        ht = w.download(T.FIELD_HEIGHT)
        # hydraulic
        hh, water, sed, flux = O.hydraulic(ht, water, sed, flux, st.step.hydraulicIterations,
                                           st.step.hydraulicDt, 1000 + it, st)
        w.hydraulic(st.step.hydraulicIterations, st.step.hydraulicDt)
        for name, f, want in (("hyd.h", T.FIELD_HEIGHT, hh), ("hyd.w", T.FIELD_WATER, water),
                              ("hyd.s", T.FIELD_SEDIMENT, sed), ("hyd.flux", T.FIELD_FLUX, flux)):
            assert_fp(name, w.download(f), want, it, report)
        hh, water = w.download(T.FIELD_HEIGHT), w.download(T.FIELD_WATER)
        sed, flux = w.download(T.FIELD_SEDIMENT), w.download(T.FIELD_FLUX)
        # finish: accretion, CCL every iterationsForCCL steps
        idf = O.accretion(hh, acc, idn, st)
        w.finish()
        np.testing.assert_array_equal(w.download(T.FIELD_ACCRETION), acc, err_msg=f"accretion marks {it}")
        np.testing.assert_array_equal(w.download(T.FIELD_PLATE_ID), idf, err_msg=f"final ids {it}")
        if it % st.sim.iterationsForCCL == 0:
            np.testing.assert_array_equal(w.download(T.FIELD_LABELS), O.ccl(idf, st.step.cclConnectivity),
                                          err_msg=f"labels {it}")
        h, ids, pl = hh, idf, nxt
    w.check()
    print(kind, W, H, {k: max(v) for k, v in report.items()})


@pytest.mark.parametrize("tile", [1, 2, 3, 4, 5, 6, 7, 8, 9])
@pytest.mark.parametrize("W,H,dt", [(100, 60, 0.02), (33, 17, 0.02), (300, 200, 0.02), (128, 96, 1.0),
                                    (57, 130, 0.02), (112, 9, 0.02), (170, 257, 0.029)])
def test_hydraulic_tile_variants_match_oracle(tile, W, H, dt):
    """Every hydraulic tile shape (interior tiles without wrap, edge tiles with it) gives the
    oracle's result; dt 1.0 takes the split transport path.  Variant 8 marches column strips of 56
    interior columns: 57 and 112 columns end on a strip of one column and on a whole strip, odd
    widths take the unpaired loads, and dt 0.029 lets transport reach nearly 1.5 cells.  Variant 9
    marches strips of 120 columns in chunks of 8 rows: 9 and 17 rows end inside the first or
    third chunk, 300 columns end on a strip of 60, and 170 x 257 ends on both."""
    st, w = make_world("baseline", W, H)
    st.step.hydraulicTile = tile
    w.set_settings(st)
    rng = np.random.default_rng(W * H + tile)
    water = np.abs(rng.normal(0, 0.2, (H, W))).astype(np.float32)
    sed = np.abs(rng.normal(0, 0.05, (H, W))).astype(np.float32)
    flux = np.abs(rng.normal(0, 0.02, (H, W, 4))).astype(np.float32)
    w.upload(T.FIELD_WATER, water)
    w.upload(T.FIELD_SEDIMENT, sed)
    w.upload(T.FIELD_FLUX, flux)
    h = w.download(T.FIELD_HEIGHT)
    w.hydraulic(7, dt)
    hh, ww, ss, ff = O.hydraulic(h, water, sed, flux, 7, dt, 1000, st)
    report = {}
    for name, f, want in (("h", T.FIELD_HEIGHT, hh), ("w", T.FIELD_WATER, ww), ("s", T.FIELD_SEDIMENT, ss),
                          ("flux", T.FIELD_FLUX, ff)):
        assert_fp(name, w.download(f), want, 0, report)
    w.check()


@pytest.mark.parametrize("tile", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("W,H,iters", [(100, 60, 7), (33, 17, 5), (300, 200, 10), (128, 96, 3)])
def test_thermal_tile_variants_match_oracle(tile, W, H, iters):
    """Every thermal tile shape and per-launch iteration split gives the oracle's result."""
    st, w = make_world("baseline", W, H)
    st.step.thermalTile = tile
    w.set_settings(st)
    rng = np.random.default_rng(W + H + tile)
    h = (w.download(T.FIELD_HEIGHT) + rng.normal(0, 0.05, (H, W))).astype(np.float32)
    w.upload(T.FIELD_HEIGHT, h)
    w.thermal(iters)
    want = O.thermal(h, iters, st)
    # bit for bit, zero signs included
    np.testing.assert_array_equal(w.download(T.FIELD_HEIGHT).view(np.uint32), want.view(np.uint32))
    w.check()


@pytest.mark.parametrize("tile", [4, 5])
@pytest.mark.parametrize("angle,amplitude", [(0.0, None), (-0.5, None), (0.5, -0.5)])
def test_thermal_general_parameters_match_oracle(tile, angle, amplitude):
    """A threshold below 2^-64 and flows that may be negative (negative threshold or amplitude)
    take the general forms of the tile and marching kernels: bit for bit the oracle's result."""
    st, w = make_world("baseline", 100, 60)
    st.step.thermalTile = tile
    st.kernel.thermalThresholdAngle = angle
    if amplitude is not None:
        st.kernel.thermalErosionAmplitude = amplitude
    w.set_settings(st)
    rng = np.random.default_rng(7 + tile)
    h = (w.download(T.FIELD_HEIGHT) + rng.normal(0, 0.05, (60, 100))).astype(np.float32)
    w.upload(T.FIELD_HEIGHT, h)
    w.thermal(3)
    want = O.thermal(h, 3, st)
    got = w.download(T.FIELD_HEIGHT)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    w.check()


@pytest.mark.parametrize("W,H,steps", [(64, 64, 12), (100, 60, 12), (256, 256, 6)])
def test_graph_steps_match_oracle(torch_stream, W, H, steps):
    st, w = make_world("baseline", W, H)
    ow = O.OracleWorld(st, w.download(T.FIELD_HEIGHT), w.download(T.FIELD_PLATE_ID), w.plates(), 1000)
    report = {}
    for it in range(steps):
        w.step(1, torch_stream)
        torch_stream.synchronize()
        ow.step()
        np.testing.assert_array_equal(w.download(T.FIELD_PLATE_ID), ow.id, err_msg=f"ids {it}")
        np.testing.assert_array_equal(w.download(T.FIELD_COLLISION), ow.word, err_msg=f"words {it}")
        np.testing.assert_array_equal(w.download(T.FIELD_LABELS), ow.labels, err_msg=f"labels {it}")
        for name, f, want in (("h", T.FIELD_HEIGHT, ow.h), ("w", T.FIELD_WATER, ow.w),
                              ("s", T.FIELD_SEDIMENT, ow.s), ("flux", T.FIELD_FLUX, ow.flux)):
            assert_fp(name, w.download(f), want, it, report)
    assert w.iteration == steps
    w.check(torch_stream)
    print(W, H, {k: max(v) for k, v in report.items()})


def test_config0_100_steps(torch_stream):
    """The CPU-runnable configuration: 256x256, 8 plates, 100 steps, 4-connected CCL every 10."""
    s = T.baseline_settings()
    w = T.World(s, 256, 256, seed=1000)
    w.init_synthetic(8, 1.0, 0)
    ow = O.OracleWorld(s, w.download(T.FIELD_HEIGHT), w.download(T.FIELD_PLATE_ID), w.plates(), 1000)
    w.step(100, torch_stream)
    torch_stream.synchronize()
    ow.step(100)
    w.check(torch_stream)
    np.testing.assert_array_equal(w.download(T.FIELD_PLATE_ID), ow.id)
    np.testing.assert_array_equal(w.download(T.FIELD_LABELS), ow.labels)
    for f, want in ((T.FIELD_HEIGHT, ow.h), (T.FIELD_WATER, ow.w), (T.FIELD_SEDIMENT, ow.s)):
        got = w.download(f)
        r = float(want.max() - want.min())
        assert float(np.max(np.abs(got - want))) <= max(1e-3 * r, 1e-5)


def test_size_independent_properties_2048(torch_stream):
    """At the benchmark size: the sort is a stable permutation grouping every arrival, the words
    are exactly the first four arrivals of each destination, ids stay in range."""
    s = T.baseline_settings()
    W = H = 2048
    w = T.World(s, W, H, seed=1000)
    w.init_synthetic(32, 1.0, 1)
    ids0 = w.download(T.FIELD_PLATE_ID)
    w.collide()
    keys = w.download(T.FIELD_SORT_KEYS).ravel().astype(np.int64)
    vals = w.download(T.FIELD_SORT_VALS).ravel().astype(np.int64)
    assert np.all(np.diff(keys) >= 0)
    same = np.diff(keys) == 0
    assert np.all(np.diff(vals)[same] > 0)  # stable: sources ascend within a destination
    assert np.array_equal(np.sort(vals), np.arange(W * H))
    word = w.download(T.FIELD_COLLISION).ravel()
    cnt = np.bincount(keys, minlength=W * H)
    assert np.array_equal(word == 0, cnt == 0)
    assert np.array_equal(word > 255, cnt >= 2)
    w.step(1)
    ids = w.download(T.FIELD_PLATE_ID)
    assert ids.max() < 32 and set(np.unique(ids)) <= set(np.unique(ids0))
    w.check()


def test_full_size_step_matches_oracle_2048(torch_stream):
    """One full step at the benchmark configuration (2048x2048, 32 plates) against the oracle."""
    s = T.baseline_settings()
    w = T.World(s, 2048, 2048, seed=1000)
    w.init_synthetic(32, 1.0, 1)
    ow = O.OracleWorld(s, w.download(T.FIELD_HEIGHT), w.download(T.FIELD_PLATE_ID), w.plates(), 1000)
    w.step(2, torch_stream)
    torch_stream.synchronize()
    ow.step(2)
    np.testing.assert_array_equal(w.download(T.FIELD_PLATE_ID), ow.id)
    np.testing.assert_array_equal(w.download(T.FIELD_LABELS), ow.labels)
    for f, want in ((T.FIELD_HEIGHT, ow.h), (T.FIELD_WATER, ow.w), (T.FIELD_SEDIMENT, ow.s)):
        assert float(np.max(np.abs(w.download(f) - want))) <= fp_tol(want)
