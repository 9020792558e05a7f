"""The reference's own CUDA kernels, built from its sources into a cubin where the sources exist
(oracle/Makefile `refgpu`), load and run on this GPU through the timing harness of the reference
arm.  Skipped when the cubin was not built."""
from __future__ import annotations

import pytest

import master_thesis_gb300 as T
import oracle as O

pytestmark = pytest.mark.gpu


def test_reference_kernels_time_a_small_world():
    if not O.REF_CUBIN.exists():
        pytest.skip("the reference's device code was not built here (no reference sources)")
    h, ids, pl = T.generate_world(256, 256, 8, 1.0, 1)
    st = T.baseline_settings()
    ms = O.ref_gpu_time(256, 256, h, ids, pl, st, steps=2, warmup=1)
    assert 0.0 < ms < 1e4
