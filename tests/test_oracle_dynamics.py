"""Plate dynamics in the oracle, pinned to the reference's own kernels (golden vectors from
processCollisions, accumulatePlateAngularCoords / calculatePlateCenters, computeCurl and
applyPlateMovementChanges compiled for the CPU): the collision friction per plate, the geometric
centres, the asthenosphere curl and the movement update."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import master_thesis_gb300 as T
import oracle as O


def settings(g):
    st = T.baseline_settings()
    st.kernel.minCollisionSize = 3
    st.kernel.collisionTypeUpdateCooldown = 2
    st.kernel.frictionCoefficientContinental, st.kernel.frictionCoefficientSubduction, \
        st.kernel.frictionCoefficientAccretion = (float(x) for x in g["fc"])
    st.step.plateDynamics = T.PLATE_DYNAMICS_REFERENCE
    return st


@pytest.fixture(scope="module")
def g(golden):
    return dict(golden("ref_dynamics"))


def test_collision_friction_matches_reference(g):
    """The reference sums the friction terms in thread order with float adds; the oracle sums the
    same float terms exactly in fixed point: equal to float rounding of the sum."""
    st = settings(g)
    W, H = int(g["W"]), int(g["H"])
    offx, offy, _ = O.plate_offsets(g["plates"])
    dyn = np.zeros(255, T.PLATE_DYNAMICS_DTYPE)
    dyn["mass"] = g["mass"]
    fric = np.zeros(255, np.int64)
    div = g["div"].copy()
    h_new = np.zeros((H, W), np.float32)
    id_new = np.zeros((H, W), np.uint8)
    acc = np.zeros((H, W), np.uint8)
    P = O._P
    ids, h, word, bitmap, plates = g["ids"], g["h"], g["word"], g["bitmap"], g["plates"]  # keep them alive
    O.lib().or_resolve_dyn(W, H, P(ids), P(h), P(word), P(offx), P(offy), P(bitmap), P(div), C.addressof(st), 1000,
                           3, P(h_new), P(id_new), P(acc), None, None, P(plates), P(dyn), P(fric))
    got = (fric.astype(np.float64) * 2.0 ** -40).astype(np.float32)
    ref = g["friction"]
    assert (ref != 0).sum() >= 5
    np.testing.assert_array_equal(got != 0, ref != 0)
    np.testing.assert_allclose(got, ref, rtol=2e-6, atol=1e-9)


def test_geometric_centres_match_reference(g):
    """Angular means: the reference sums libm sin / cos with float adds and takes libm atan2f; the
    oracle sums the engine's sin / cos exactly and takes its atan2: within 1e-3 cells."""
    for ids, key, skip in ((g["ids"], "centres", ()), (g["ids2"], "centres2", (3,))):
        H, W = ids.shape
        dyn = O.plate_stats(np.zeros(ids.shape, np.float32), ids, 1)
        present = np.bincount(ids[::10, ::10].ravel(), minlength=256)[:255] > 0
        sampled = present.copy()
        for k in skip:  # a plate around a whole axis has no defined angular mean
            present[k] = False
        assert present.sum() >= 2
        got = np.stack([dyn["geometricCenter_x"], dyn["geometricCenter_y"]], 1)
        ref = g[key]
        d = np.abs(got - ref)[present]
        d = np.minimum(d, np.array([W, H]) - d)  # a centre on a seam may land on either side
        assert d.max() < 1e-3, d.max()
        assert not got[~sampled].any()


def test_first_iteration_keeps_the_stored_centre(g):
    dyn_in = np.zeros(255, T.PLATE_DYNAMICS_DTYPE)
    dyn_in["geometricCenter_x"] = 7.0
    dyn = O.plate_stats(g["h"], g["ids"], 0, dyn_in)
    assert (dyn["geometricCenter_x"] == 7.0).all()
    assert dyn["size"].sum() == g["ids"].size
    np.testing.assert_allclose(dyn["mass"], np.bincount(g["ids"].ravel(), g["h"].ravel().astype(np.float64),
                                                         minlength=255)[:255], rtol=1e-6, atol=1e-3)


def test_curl_matches_reference(g):
    W, H = int(g["W"]), int(g["H"])
    pr = g["pressure"]
    got = np.array([[O.curl_at(pr, W, H, x, y) for x in range(W)] for y in range(H)], np.float32)
    np.testing.assert_array_equal(got, g["curl"])


def test_plate_motion_matches_reference(g):
    st = settings(g)
    W, H = int(g["W"]), int(g["H"])
    fric = np.rint(g["fric_in"].astype(np.float64) * 2.0 ** 40).astype(np.int64)
    plates, dyn = O.plate_motion(W, H, g["plates_in"], g["dyn_in"], fric, g["pressure"], st)
    ref_p, ref_d = g["plates_out"], g["dyn_out"]
    for f in ("velocity", "direction_x", "direction_y"):
        np.testing.assert_allclose(plates[f], ref_p[f], rtol=1e-6, atol=1e-7, err_msg=f)
    np.testing.assert_array_equal(plates["pixelCenter_x"], g["plates_in"]["pixelCenter_x"])  # moved elsewhere
    for f in ("velocitySmoothed", "directionSmoothed_x", "directionSmoothed_y"):
        np.testing.assert_allclose(dyn[f], ref_d[f], rtol=1e-6, atol=1e-7, err_msg=f)
    np.testing.assert_array_equal(dyn["mergeWaitTime"], ref_d["mergeWaitTime"])


def test_dynamics_change_the_plates_over_steps():
    st = T.baseline_settings()
    st.step.plateDynamics = T.PLATE_DYNAMICS_REFERENCE
    h, ids, pl = T.generate_world(48, 40, 5, 1.0, 8)
    a = O.OracleWorld(st, h, ids, pl, 1000)
    a.pressure = np.random.default_rng(1).random((20, 24)).astype(np.float32)
    a.step(3)
    st0 = T.baseline_settings()
    b = O.OracleWorld(st0, h, ids, pl, 1000)
    b.step(3)
    assert not np.array_equal(a.plates["velocity"], b.plates["velocity"])
    np.testing.assert_array_equal(b.plates["velocity"], pl["velocity"])
    assert (a.dyn["size"][:5] > 0).all()
