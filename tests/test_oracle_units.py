"""Unit properties of the oracle's building blocks (CPU)."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import pytest

import master_thesis_gb300 as T
import oracle as O


def test_engine_sine_within_two_ulp_of_libm():
    L = O.lib()
    xs = np.concatenate([np.linspace(0.0, 10.0, 20001), np.linspace(10.0, 6.0e4, 20001),
                         -np.linspace(0.0, 100.0, 2001)]).astype(np.float32)
    worst = 0.0
    for x in xs:
        ref = np.float32(math.sin(float(x)))
        got = np.float32(L.or_sinf(float(x)))
        ulp = float(np.spacing(np.float32(max(abs(ref), 1e-30))))
        worst = max(worst, abs(float(got) - float(ref)) / ulp)
    assert worst <= 2.0, worst


def test_lerp_endpoints_and_monotone():
    L = O.lib()
    assert L.or_lerp(2.0, 5.0, 0.0) == 2.0
    assert L.or_lerp(2.0, 5.0, 1.0) == 5.0
    vals = [L.or_lerp(-3.0, 7.0, t) for t in np.linspace(0, 1, 101)]
    assert all(b >= a for a, b in zip(vals, vals[1:]))


def test_gaussian_weights_normalised_symmetric():
    w = np.zeros(7, np.float32)
    O.lib().or_gaussian_weights(1.5, 3, w.ctypes.data)
    assert abs(float(w.sum()) - 1.0) < 1e-6
    np.testing.assert_array_equal(w, w[::-1])
    assert np.all(np.diff(w[:4]) > 0)


def test_rain_noise_range_and_determinism():
    L = O.lib()
    v = [L.or_rain_noise(x, y, 1234) for x in range(50) for y in range(50)]
    assert min(v) >= -1.0 and max(v) <= 1.0
    assert v == [L.or_rain_noise(x, y, 1234) for x in range(50) for y in range(50)]


def test_thermal_conserves_mass_roughly():
    h, _, _ = T.generate_world(48, 40, 6, 1.0, 4)
    out = O.thermal(h, 10, T.baseline_settings())
    assert abs(float(out.astype(np.float64).sum() - h.astype(np.float64).sum())) < 1e-3


@pytest.mark.parametrize("sigma,radius", [(1.5, 3), (0.8, 1), (3.0, 8)])
def test_gaussian_uplift_against_numpy_convolution(sigma, radius):
    """The new Gaussian uplift (upliftAmount on convergent cells, separable blur with wrap) against an
    independent float64 restatement with numpy: the oracle's resolve with and without the uplift
    differs by the blurred field, to float32 rounding."""
    import master_thesis_gb300 as T
    W, H = 48, 40
    h, ids, pl = T.generate_world(W, H, 7, 1.8, 12)
    offx, offy, _ = O.plate_offsets(pl)
    _, word, _, _ = O.collision_words(ids, offx, offy)
    s = T.baseline_settings()
    s.step.upliftSigma, s.step.upliftRadius, s.step.upliftAmount = sigma, radius, 0.25
    bm = np.zeros(32385, np.uint8)
    div = np.zeros(1013, np.uint32)
    s.step.upliftMode = T.UPLIFT_GAUSSIAN
    hg, *_ = O.resolve(ids, h, word, offx, offy, bm, div, s, 1000, 0)
    s.step.upliftMode = T.UPLIFT_NONE
    hn, *_ = O.resolve(ids, h, word, offx, offy, bm, div, s, 1000, 0)
    conv = (word > 0xFF).astype(np.float64) * 0.25
    k = np.exp(-0.5 * (np.arange(-radius, radius + 1) / sigma) ** 2)
    k /= k.sum()
    blur = np.zeros_like(conv)
    for d, wgt in zip(range(-radius, radius + 1), k):
        blur += wgt * np.roll(conv, -d, axis=1)
    out = np.zeros_like(conv)
    for d, wgt in zip(range(-radius, radius + 1), k):
        out += wgt * np.roll(blur, -d, axis=0)
    assert (word > 0xFF).sum() > 10
    np.testing.assert_allclose(hg.astype(np.float64) - hn.astype(np.float64), out, atol=2e-6, rtol=0)


def test_oracle_settings_and_layouts_equal_the_engines():
    """The CPU legs of bench.py use the oracle's copies of the settings, the struct layouts and the
    synthetic generator, so that they never load the engine; they must be the engine's exactly."""
    for name in ("KernelSettings", "SimulationSettings", "StepSettings", "Settings"):
        a, b = getattr(O, name), getattr(T, name)
        assert C.sizeof(a) == C.sizeof(b), name
        assert [(f, getattr(a, f).offset) for f, _ in a._fields_] == [(f, getattr(b, f).offset) for f, _ in b._fields_]
    assert O.PLATE_DTYPE == T.PLATE_DTYPE and O.PLATE_DYNAMICS_DTYPE == T.PLATE_DYNAMICS_DTYPE
    assert O.MAX_PLATES == T.MAX_PLATES
    assert bytes(O.default_settings()) == bytes(T.default_settings())
    assert bytes(O.baseline_settings()) == bytes(T.baseline_settings())


@pytest.mark.parametrize("W,H,P,vel,seed", [(1, 1, 1, 1.0, 0), (96, 64, 8, 1.0, 6), (257, 130, 32, 2.0, 12345),
                                            (64, 3, 255, 0.5, 2**63 + 7)])
def test_oracle_generator_equals_the_engines(W, H, P, vel, seed):
    ho, io, po = O.generate_world(W, H, P, vel, seed)
    he, ie, pe = T.generate_world(W, H, P, vel, seed)
    np.testing.assert_array_equal(ho, he)
    np.testing.assert_array_equal(io, ie)
    np.testing.assert_array_equal(po.view(np.uint8), pe.view(np.uint8))
