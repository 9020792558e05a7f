"""Plate relabel and merges in the oracle.  Merges are pinned to the reference's own kernels
(getNeighboringPlates, getPlateMerges run in thread order, clearCollisionTypes, the remap of
mergeAndCountSizeMass; golden vectors).  The relabel's ranking and id assignment run in the
reference inside one block with a barrier and atomics, which the CPU build cannot execute: they
are pinned to the reference's own kernels run on a GPU (tests/golden/gen_golden_relabel.py, on id
maps whose outcome does not depend on scheduling), and checked case by case against
createLabelIdLookup's rules."""
from __future__ import annotations

import numpy as np
import pytest

import master_thesis_gb300 as T
import oracle as O


def merge_settings(g):
    st = T.baseline_settings()
    (st.kernel.mergeMinVelocity, st.kernel.mergeDotDirectionThreshold,
     st.kernel.mergeVelocityDiffThreshold, area) = (float(v) for v in g["ks"])
    st.kernel.targetMaximumPlateArea = int(area)
    return st


def test_merges_match_reference(golden):
    g = golden("ref_policy")
    ids, bm, n = O.merge(g["ids"], g["plates"], g["dyn"], g["bitmap"], merge_settings(g))
    assert n == int((g["merge_ids"] == -1).sum()) >= 2
    np.testing.assert_array_equal(ids, g["out_ids"])
    np.testing.assert_array_equal(bm, g["out_bitmap"])


def labels_of(ids, conn=T.CCL_4):
    H, W = ids.shape
    lab = np.zeros((H, W), np.uint32)
    O.lib().or_ccl(W, H, O._P(np.ascontiguousarray(ids)), O._P(lab), conn)
    return lab


def records(sizes):
    pl = np.zeros(255, T.PLATE_DTYPE)
    dy = np.zeros(255, T.PLATE_DYNAMICS_DTYPE)
    for k, sz in sizes.items():
        pl[k]["velocity"] = 0.1 * (k + 1)
        pl[k]["direction_x"] = 1.0
        dy[k]["size"] = sz
        dy[k]["mass"] = 10.0 * (k + 1)
    return pl, dy


def test_relabel_rules():
    ids = np.zeros((12, 16), np.uint8)       # plate 0: the background
    ids[0:4, 0:6] = 1                         # plate 1 (largest part, 24 cells)
    ids[6:8, 8:11] = 1                        # plate 1 fragment, 6 cells >= minPlateSize
    ids[10, 2] = 1                            # plate 1 fragment, 1 cell < minPlateSize
    ids[2:4, 10:13] = 2                       # plate 2: two parts of 6 cells each
    ids[9:11, 11:14] = 2
    pl, dy = records({0: 120, 1: 31, 2: 12})  # plate 3 and above have no cells: free ids
    lab = labels_of(ids)
    out, pl2, dy2, left = O.relabel(ids, lab, pl, dy, 4)
    assert left == 0
    # the largest part of each plate keeps its id; equal largest parts both keep it
    assert (out[0:4, 0:6] == 1).all() and (out[2:4, 10:13] == 2).all() and (out[9:11, 11:14] == 2).all()
    # the 6-cell fragment takes the lowest free id, with a copy of plate 1's records
    assert (out[6:8, 8:11] == 3).all()
    assert pl2[3] == pl[1] and dy2[3] == dy[1]
    # the 1-cell fragment loses its id and takes its neighbours' (all plate 0); nothing else changes
    expect = ids.copy()
    expect[6:8, 8:11] = 3
    expect[10, 2] = 0
    np.testing.assert_array_equal(out, expect)


def test_relabel_without_free_ids_fills_from_neighbours():
    ids = np.zeros((8, 8), np.uint8)
    ids[0:3, 0:3] = 1
    ids[5:7, 5:7] = 1                         # a 4-cell fragment of plate 1
    pl, dy = records({0: 40, 1: 13, 2: 5})
    dy["size"][3:] = 1                        # every id in use: no free id for the fragment
    lab = labels_of(ids)
    out, _, _, left = O.relabel(ids, lab, pl, dy, 2)
    assert left == 0
    assert (out[5:7, 5:7] == 0).all()         # surrounded by plate 0


def test_free_ids_only_below_the_component_count():
    """createLabelIdLookup lists free ids only among its first min(255, components) threads."""
    ids = np.zeros((8, 8), np.uint8)
    ids[0:3, 0:3] = 5
    ids[5:7, 5:7] = 5
    pl, dy = records({0: 47, 5: 13})          # 3 components: free ids among 0..2 only, and 0 is used
    lab = labels_of(ids)
    out, _, _, _ = O.relabel(ids, lab, pl, dy, 2)
    assert (out[5:7, 5:7] == 1).all()


def test_policy_steps():
    st = T.baseline_settings()
    st.step.plateDynamics = T.PLATE_DYNAMICS_REFERENCE
    st.step.platePolicy = T.PLATE_RELABEL | T.PLATE_MERGE
    st.sim.iterationsForCCL = 1
    st.kernel.minPlateSize = 3
    st.kernel.mergeMinVelocity = 0.3
    st.kernel.targetMaximumPlateArea = 100000
    h, ids, pl = T.generate_world(64, 48, 9, 1.5, 4)
    w = O.OracleWorld(st, h, ids, pl, 1000)
    n0 = len(np.unique(w.id))
    w.step(6)
    assert (w.id != 255).all()
    assert len(np.unique(w.id)) <= n0 + 20


@pytest.mark.parametrize("case", ["free_id", "no_free_id"])
def test_relabel_matches_reference_kernels(golden, case):
    """The oracle's relabel equals the reference's own applyCCL relabel (its CCL, thrust ranking,
    getMaxSizeLabels, createLabelIdLookup, postCClIdReassign and assignUnassignedIdsToNeighbor, run
    on a GPU): labels, final ids, and which plate record each id slot holds afterwards."""
    g = golden("ref_relabel")
    ids = g[f"{case}_ids_in"]
    np.testing.assert_array_equal(labels_of(ids, T.CCL_REF8), g[f"{case}_labels"])
    pl = np.zeros(255, T.PLATE_DTYPE)
    dy = np.zeros(255, T.PLATE_DYNAMICS_DTYPE)
    pl["velocity"] = np.arange(255)          # a record's marker: the plate it belonged to
    dy["size"] = g[f"{case}_sizes"]
    out, pl2, _, left = O.relabel(ids, g[f"{case}_labels"], pl, dy, int(g[f"{case}_min_plate_size"]))
    assert left == 0
    np.testing.assert_array_equal(out, g[f"{case}_ids_out"])
    np.testing.assert_array_equal(pl2["velocity"], g[f"{case}_markers"])
    # the cells postCClIdReassign left without an id: changed cells not moved to a new id's slot
    moved = [k for k in range(255) if int(pl2["velocity"][k]) != k]
    lost = int(((out != ids) & ~np.isin(out, moved)).sum())
    assert lost == int(g[f"{case}_unassigned"]) > 0
