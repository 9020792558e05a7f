"""Generate the golden vectors that pin the oracle's CCL relabel to the reference's own kernels.

The relabel of PlateTectonicSim::applyCCL (MarWo22/master_thesis src/cuda_compute/
plate_tectonic_sim.cu:374-467) ranks components with thrust and decides ids in one block with a
barrier and atomics (createLabelIdLookup, plate_tectonics_kernel.cu:3130-3185), then fills cells
left without an id in place (assignUnassignedIdsToNeighbor, :2052-2101).  The CPU build of the
reference cannot run those, so this script runs them on a GPU: oracle/refgpu/ref_relabel.cu
launches the reference's device code (oracle/_ref/ref_kernels.cubin, built from the reference's
sources where they lie) with the same thrust calls between the kernels.

The id maps are built so that the outcome does not depend on thread scheduling:
  - at most one free id (a plate record with size 0 among the first `components` slots), and at
    most one fragment that could take it (the reference hands free ids out in atomic order);
  - every cell left without an id is an isolated single cell whose eight neighbours all keep
    their ids (the in-place fill would otherwise race), with a unique most frequent neighbour or
    an exact tie (settled by the neighbour order);
  - fewer components than 1 % of the cells (the reference's label buffer).

Run on a machine with a GPU (the cubin is built where the reference sources exist):

    python tests/golden/gen_golden_relabel.py [out.npz]     # default tests/golden/ref_relabel.npz
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import master_thesis_gb300 as T  # noqa: E402
import oracle as O  # noqa: E402


def case_free_id():
    """64 x 64: plate 1 has a large part and a fragment of 80 cells (>= minPlateSize 20) that takes
    the one free id, 3; plate 4's and plate 5's single cells are lost and filled (a unique
    neighbour, a 5-3 split across a plate border, and a 4-4 tie)."""
    W = H = 64
    ids = np.zeros((H, W), np.uint8)           # plate 0: the background, one component
    ids[2:18, 2:22] = 1                        # plate 1, 320 cells (its largest part)
    ids[30:38, 40:50] = 1                      # plate 1 fragment, 80 cells: takes free id 3
    ids[44:54, 4:14] = 2                       # plate 2, 100 cells
    ids[20:30, 50:60] = 4                      # plate 4, 100 cells ...
    ids[20:24, 52:56] = 4
    for y, x in ((5, 40), (40, 20), (58, 58)):  # ... and single cells inside plate 0
        ids[y, x] = 4
    ids[40:60, 24:34] = 6                      # plate 6, 200 cells
    ids[50, 28] = 5                            # plate 5: one cell inside plate 6 ...
    ids[2:8, 56:62] = 5                        # ... and its largest part, 36 cells
    # a lost cell beside plate 2's block: five neighbours of plate 0, three of plate 2
    ids[45, 14] = 4
    # a lost cell with four neighbours of plate 7 and four of plate 8 (a tie: the first of the
    # reference's neighbour order, +x, wins)
    ids[60:63, 14:17] = 7                      # plate 7, 10 cells
    ids[62, 17] = 7
    ids[60:63, 18:21] = 8                      # plate 8, 10 cells
    ids[60, 17] = 8
    ids[61, 17] = 4
    sizes = np.full(255, 100, np.int32)
    sizes[3] = 0                               # the one free id
    return ids, sizes, 20


def case_no_free_id():
    """32 x 32, minPlateSize 1: single-cell fragments would take a free id but none is left, so they
    are lost and filled; plate 2's two equal largest parts both keep their id."""
    W = H = 32
    ids = np.zeros((H, W), np.uint8)
    ids[2:10, 2:10] = 1                        # plate 1, 64 cells
    ids[20, 20] = 1                            # plate 1 single cell inside plate 0: no free id
    ids[4:8, 20:24] = 2                        # plate 2: two parts of 16 cells
    ids[24:28, 4:8] = 2
    ids[14:18, 14:19] = 3                      # plate 3, 20 cells
    ids[15, 16] = 2                            # plate 2 single cell inside plate 3
    sizes = np.full(255, 50, np.int32)         # every record has cells: no free id
    return ids, sizes, 1


def main(out: Path):
    cases = {"free_id": case_free_id(), "no_free_id": case_no_free_id()}
    arrays = {}
    for name, (ids, sizes, mps) in cases.items():
        s = T.baseline_settings()
        s.kernel.minPlateSize = mps
        got, labels, markers, rounds, left = O.ref_gpu_relabel(ids, sizes, s, max_rounds=16)
        assert rounds < 16, f"{name}: the fill did not settle"
        arrays.update({f"{name}_ids_in": ids, f"{name}_sizes": sizes, f"{name}_min_plate_size": np.int32(mps),
                       f"{name}_ids_out": got, f"{name}_labels": labels, f"{name}_markers": markers,
                       f"{name}_rounds": np.int32(rounds), f"{name}_unassigned": np.int32(left)})
        print(name, "unassigned", left, "fill rounds", rounds, "records moved",
              [(k, int(m)) for k, m in enumerate(markers) if int(m) != k])
    np.savez_compressed(out, **arrays)
    print("wrote", out)


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent / "ref_relabel.npz")
