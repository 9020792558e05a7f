"""The CPU oracle against golden vectors produced by the reference's own kernels.

tests/golden/*.npz were generated by tests/golden/gen_golden.py, which runs the reference's
hot-path kernels (compiled for the CPU from their own sources, sequential thread emulation).  The
oracle, switched to libm's sinf as those kernels use on the CPU, must reproduce every phase bit
for bit.
"""
from __future__ import annotations

import numpy as np
import pytest

import master_thesis_gb300 as T
import oracle as O

STEP_CASES = ["ref_steps_baseline_64x64", "ref_steps_baseline_128x48", "ref_steps_reference_64x64"]


@pytest.fixture(autouse=True)
def _libm_sin():
    O.use_libm_sin(True)
    yield
    O.use_libm_sin(False)


def _settings(kind: str) -> T.Settings:
    s = T.baseline_settings() if kind == "baseline" else T.default_settings()
    s.kernel.minCollisionSize = 3
    s.kernel.collisionTypeUpdateCooldown = 2
    s.step.upliftMode = T.UPLIFT_NONE
    s.step.thermalIterations = 0
    s.step.cclConnectivity = T.CCL_REF8
    s.sim.iterationsForCCL = 1
    return s


@pytest.mark.parametrize("case", STEP_CASES)
def test_phases_match_reference_kernels(golden, case):
    g = golden(case)
    W, H, steps = int(g["W"]), int(g["H"]), int(g["steps"])
    st = _settings(str(g["kind"]))
    st.step.hydraulicIterations = int(g["hyd_iters"])
    st.step.hydraulicDt = float(g["dt"])
    h, ids, pl = g["h0"].copy(), g["id0"].copy(), g["plates0"].copy()
    w = np.zeros((H, W), np.float32)
    s = np.zeros((H, W), np.float32)
    f = np.zeros((H, W, 4), np.float32)
    bm = np.zeros(T.NUM_PAIRS, np.uint8)
    div = np.zeros(T.NUM_DIV_WORDS, np.uint32)
    seed = int(g["seed"])
    for it in range(steps):
        offx, offy, nxt = O.plate_offsets(pl)
        dest, word, sk, sv = O.collision_words(ids, offx, offy)
        np.testing.assert_array_equal(dest, g[f"dest_{it}"], err_msg=f"advection, step {it}")
        np.testing.assert_array_equal(word, g[f"word_{it}"], err_msg=f"arrival words, step {it}")
        # the stable sort's output regroups exactly the arrivals the words encode
        assert np.all(np.diff(sk.astype(np.int64)) >= 0)
        bm = O.collision_types(word, h, offx, offy, st, bm)
        np.testing.assert_array_equal(bm, g[f"bitmap_{it}"], err_msg=f"type bitmap, step {it}")
        hn, idn, acc, div = O.resolve(ids, h, word, offx, offy, bm, div, st, seed, it)
        np.testing.assert_array_equal(div, g[f"div_{it}"], err_msg=f"divergence bitmap, step {it}")
        np.testing.assert_array_equal(acc, g[f"acc_{it}"], err_msg=f"accretion marks, step {it}")
        hn, w, s, f = O.hydraulic(hn, w, s, f, st.step.hydraulicIterations, st.step.hydraulicDt, seed + it, st)
        idn = O.accretion(hn, acc, idn, st)
        np.testing.assert_array_equal(hn, g[f"h_{it}"], err_msg=f"height, step {it}")
        np.testing.assert_array_equal(w, g[f"w_{it}"], err_msg=f"water, step {it}")
        np.testing.assert_array_equal(s, g[f"s_{it}"], err_msg=f"sediment, step {it}")
        np.testing.assert_array_equal(f, g[f"flux_{it}"], err_msg=f"flux, step {it}")
        np.testing.assert_array_equal(idn, g[f"id_{it}"], err_msg=f"plate ids, step {it}")
        lab = O.ccl(idn, T.CCL_REF8)
        np.testing.assert_array_equal(lab, g[f"labels_{it}"], err_msg=f"CCL labels, step {it}")
        np.testing.assert_array_equal(nxt, g[f"plates_{it}"], err_msg=f"plate centres, step {it}")
        h, ids, pl = hn, idn, nxt


@pytest.mark.parametrize("case", STEP_CASES)
def test_full_step_matches_reference_composition(golden, case):
    g = golden(case)
    st = _settings(str(g["kind"]))
    st.step.hydraulicIterations = int(g["hyd_iters"])
    st.step.hydraulicDt = float(g["dt"])
    ow = O.OracleWorld(st, g["h0"], g["id0"], g["plates0"], int(g["seed"]))
    for it in range(int(g["steps"])):
        ow.step()
        for k in ("h", "id", "w", "s", "flux", "labels"):
            np.testing.assert_array_equal(getattr(ow, k), g[f"{k}_{it}"], err_msg=f"{k}, step {it}")


def test_thermal_matches_reference_where_race_free(golden):
    g = golden("ref_thermal_isolated_64x64")
    out = O.thermal(g["h_in"], 1, T.default_settings())
    np.testing.assert_array_equal(out, g["h_out"])


@pytest.mark.parametrize("case", ["random4", "random2", "diagonals", "stripes", "voronoi"])
def test_ccl_ref8_matches_reference(golden, case):
    g = golden("ref_ccl_cases")
    np.testing.assert_array_equal(O.ccl(g[f"{case}_id"], T.CCL_REF8), g[f"{case}_labels"])


def test_ccl_modes_are_nested():
    """4-connected components refine ref8 components, which refine 8-connected ones."""
    rng = np.random.default_rng(3)
    ids = rng.integers(0, 3, (40, 56)).astype(np.uint8)
    l4, lr, l8 = (O.ccl(ids, m) for m in (T.CCL_4, T.CCL_REF8, T.CCL_8))
    for fine, coarse in ((l4, lr), (lr, l8)):
        for lab in np.unique(fine):
            assert len(np.unique(coarse[fine == lab])) == 1
    for lab in (l4, lr, l8):
        idx = np.arange(ids.size).reshape(ids.shape)
        # each label is the smallest index carrying it, and equal labels share a plate id
        for v in np.unique(lab):
            m = lab == v
            assert idx[m].min() == v
            assert len(np.unique(ids[m])) == 1
