"""The reference's world initialisation (initializeTectonics): the oracle's restatement of the host
draws equals the engine's, which call the C++ standard library as the reference does; the oracle's
per-cell plate ids and height map equal the reference's own initPlateIDs / initHeightmap (golden
vectors)."""
from __future__ import annotations

import numpy as np
import pytest

import master_thesis_gb300 as T
import oracle as O


@pytest.mark.parametrize("W,H,seed,plates,gens", [
    (96, 64, 1234, 12, (60, 150)), (50, 80, 7, 5, ()), (512, 256, 0, 16, (200, 500)),
    (33, 17, 2147483647, 255, (300,)), (64, 64, 4294967295, 3, (0,)), (128, 32, 99, 40, (10, 0, 20))])
def test_host_draws_match_the_standard_library(W, H, seed, plates, gens):
    e = T.reference_seeds(W, H, seed, plates, gens)
    o = O.reference_seeds(W, H, seed, plates, gens)
    for a, b, what in zip(e, o, ("seed x", "seed y", "seed id", "plates", "plate dynamics")):
        np.testing.assert_array_equal(a, b, err_msg=what)
    sx, sy, sid, pl, dy = e
    expect = gens[-1] if gens and gens[-1] >= plates else plates
    assert len(sx) == expect
    assert (sx >= 0).all() and (sx < H).all() and (sy >= 0).all() and (sy < W).all()  # {height, width} draws
    assert (pl["velocity"][:plates] >= 0).all() and (pl["velocity"][:plates] <= 1).all()
    np.testing.assert_allclose(np.hypot(pl["direction_x"][:plates], pl["direction_y"][:plates]), 1.0, atol=1e-6)
    assert not pl["velocity"][plates:].any()


@pytest.mark.parametrize("tag", ["a", "b"])
def test_cells_match_reference_kernels(golden, tag):
    g = golden("ref_init")
    W, H, seed = int(g[f"{tag}_W"]), int(g[f"{tag}_H"]), int(g[f"{tag}_seed"])
    sx, sy, sid = g[f"{tag}_sx"], g[f"{tag}_sy"], g[f"{tag}_sid"]
    e = T.reference_seeds(W, H, seed, int(g[f"{tag}_plates"]), g[f"{tag}_gens"])
    np.testing.assert_array_equal(e[0], sx)
    np.testing.assert_array_equal(e[2], sid)
    h, ids = O.init_reference(W, H, seed, sx, sy, sid)
    np.testing.assert_array_equal(ids, g[f"{tag}_ids"])
    np.testing.assert_array_equal(h, g[f"{tag}_h"])


@pytest.mark.parametrize("args", [(64, 64, 1, 0, ()), (64, 64, 1, 256, ()), (64, 64, 1, 4, (-1,)),
                                  (64, 64, 1, 4, (1,) * 9), (0, 64, 1, 4, ())])
def test_invalid_settings_are_refused(args):
    with pytest.raises(T.TectoError):
        T.reference_seeds(*args)
