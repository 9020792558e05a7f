"""The oracle's reference uplift pinned to the reference's own kernels (golden vectors from
tests/golden/gen_golden.py: moveContinentalCollisions, combinePropagatedCollisions, the JFA
kernels and applyUplift run in ascending thread order): the processConvergence records and the
nearest-seed / distance fields bit for bit; heights within the per-step FP32 tolerance (the
reference's libm exp/log10 and the engine's own differ in the last bits)."""
from __future__ import annotations

import numpy as np
import pytest

import master_thesis_gb300 as T
import oracle as O
from conftest import fp_tol


def settings(prop_threshold):
    s = T.default_settings()
    s.kernel.minCollisionSize = 3
    s.kernel.collisionTypeUpdateCooldown = 2
    s.kernel.continentalPropThreshold = float(prop_threshold)
    s.step.upliftMode = T.UPLIFT_REFERENCE
    return s


@pytest.fixture(scope="module")
def fx(golden):
    return golden("ref_uplift_64x48")


def test_uplift_fixture_exercises_every_path(fx):
    steps = int(fx["steps"])
    assert sum(int(((fx[f"up_t_{i}"] & 1) == 1).sum()) for i in range(steps)) > 0  # continental
    assert sum(int((fx[f"h_up_{i}"] != fx[f"h_res_{i}"]).sum()) for i in range(steps)) > 100
    assert all(int((fx[f"seed_{i}"] >= 0).sum()) > 0 for i in range(steps))


def test_convergence_records_match(fx):
    st = settings(fx["prop_threshold"])
    steps = int(fx["steps"])
    div = np.zeros(T.NUM_DIV_WORDS, np.uint32)
    for i in range(steps):
        offx, offy, _ = O.plate_offsets(fx[f"plates_{i}"])
        hn, idn, acc, div_out, uh, ut = O.resolve_ex(fx[f"id_old_{i}"], fx[f"h_old_{i}"], fx[f"word_{i}"], offx,
                                                     offy, fx[f"bitmap_{i}"], div, st, int(fx["seed"]), i)
        conv = (fx[f"word_{i}"] >> 8) != 0
        np.testing.assert_array_equal(idn, fx[f"id_new_{i}"], err_msg=f"ids step {i}")
        np.testing.assert_array_equal(hn, fx[f"h_res_{i}"], err_msg=f"heights step {i}")
        np.testing.assert_array_equal(ut[conv], fx[f"up_t_{i}"][conv], err_msg=f"type bytes step {i}")
        np.testing.assert_array_equal(uh[conv], fx[f"up_h_{i}"][conv], err_msg=f"height sums step {i}")
        div = fx[f"div_{i}"]


def test_uplift_matches_reference(fx):
    st = settings(fx["prop_threshold"])
    worst = 0.0
    for i in range(int(fx["steps"])):
        out, seed, dist = O.uplift_ref(fx[f"word_{i}"], fx[f"up_h_{i}"], fx[f"up_t_{i}"], fx[f"h_old_{i}"],
                                       fx[f"plates_{i}"], fx[f"id_new_{i}"], fx[f"h_res_{i}"], st)
        np.testing.assert_array_equal(seed, fx[f"seed_{i}"], err_msg=f"JFA seeds step {i}")
        np.testing.assert_array_equal(dist, fx[f"dist_{i}"], err_msg=f"JFA distances step {i}")
        want = fx[f"h_up_{i}"]
        d = float(np.max(np.abs(out.astype(np.float64) - want)))
        worst = max(worst, d)
        assert d <= fp_tol(want), f"step {i}: max |diff| {d}"
    print("uplift max |diff| vs reference (libm exp/log10):", worst)


@pytest.mark.parametrize("x", [0.0, 1.0, -1.0, 0.5, 5.2, -20.0, -87.0, -100.0, 30.0, 88.0])
def test_expf_close_to_libm(x):
    got, want = O.expf(x), float(np.exp(np.float64(x)))
    assert abs(got - want) <= 2 * np.spacing(np.float32(want)) + 1e-45


@pytest.mark.parametrize("x", [1.0, 9.0, 17.0, 0.1, 1e-30, 1e30, 1.3333, 123456.0, 1e-40])
def test_log10f_close_to_libm(x):
    got, want = O.log10f(x), float(np.log10(np.float64(x)))
    assert abs(got - want) <= 4 * np.spacing(np.float32(abs(want)) if want else np.float32(1e-38))


def test_log10f_edges():
    assert O.log10f(0.0) == -np.inf
    assert np.isnan(O.log10f(-7.0))
    assert O.log10f(1.0) == 0.0
