"""The C ABI without a GPU: the library loads, exports every declared entry point, and its
host-only parts (settings, config.json, synthetic generator, argument checks) behave."""
from __future__ import annotations

import ctypes as C
import re
import subprocess

import numpy as np
import pytest

import master_thesis_gb300 as T
from conftest import ROOT

HEADERS = sorted((ROOT / "include").glob("*.h"))
DECL = re.compile(r"^\s*(?:int|size_t|const char \*)\s*(tecto_\w+)\s*\(", re.M)


def declared():
    names = []
    for h in HEADERS:
        names += DECL.findall(h.read_text())
    return sorted(set(names))


def test_library_loads_and_exports_every_declared_symbol():
    L = T.lib()
    names = declared()
    assert len(names) >= 29
    out = subprocess.run(["nm", "-D", "--defined-only", str(T.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (tecto_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        getattr(L, n)


def test_version_string():
    assert b"sm_103a" in T.lib().tecto_version()


def test_default_settings_are_the_reference_defaults():
    s = T.default_settings()
    k = s.kernel
    assert C.sizeof(T.KernelSettings) == 50 * 4
    assert k.continentalCrustThreshold == 10000.0
    assert k.collisionTypeUpdateCooldown == 4 and k.minCollisionSize == 50
    assert np.float32(k.hydrationRainfall) == np.float32(0.101)
    assert np.float32(k.hydrationEvaporation) == np.float32(0.303)
    assert np.float32(k.gravity) == np.float32(9.81)
    assert k.thermalCellSize == 1000.0 and k.thermalThresholdAngle == 0.5
    assert s.sim.numStartingPlates == 16 and s.sim.seed == 1000 and s.sim.iterationsForCCL == 10
    assert list(s.sim.numVoronoiSeeds[:2]) == [200, 500] and s.sim.numVoronoiGenerations == 2
    assert s.step.hydraulicIterations == 10 and s.step.hydraulicDt == 1.0 and s.step.thermalIterations == 1


def test_baseline_settings_mapping():
    s = T.baseline_settings()
    k = s.kernel
    assert np.float32(k.hydrationRainfall) == np.float32(0.01)
    assert np.float32(k.hydrationEvaporation) == np.float32(0.05)
    assert np.float32(k.sedimentCapacity) == np.float32(0.1)
    assert np.float32(k.sedimentErosionRate) == np.float32(0.3)
    assert np.float32(k.sedimentDepositionRate) == np.float32(0.1)
    assert np.float32(k.thermalThresholdAngle * k.thermalCellSize) == np.float32(0.01)
    assert k.thermalErosionAmplitude * k.thermalErosionStrength == 0.5
    assert k.continentalCrustThreshold == 0.0
    assert s.step.hydraulicIterations == 20 and np.float32(s.step.hydraulicDt) == np.float32(0.02)
    assert s.step.thermalIterations == 10
    assert s.step.upliftMode == T.UPLIFT_GAUSSIAN and s.step.upliftRadius == 3
    assert np.float32(s.step.upliftSigma) == np.float32(1.5)
    assert s.step.cclConnectivity == T.CCL_4 and s.sim.iterationsForCCL == 10


def test_config_json_reference_keys_and_overrides():
    text = (ROOT / "tests" / "golden" / "config_example.json").read_text()
    s, w, h = T.settings_from_json(text)
    assert (w, h) == (1024, 1024)
    assert s.kernel.minCollisionSize == 7
    assert np.float32(s.kernel.hydrationRainfall) == np.float32(0.02)
    assert s.sim.iterationsForCCL == 5 and list(s.sim.numVoronoiSeeds[:3]) == [10, 20, 30]
    assert s.sim.numVoronoiGenerations == 3 and s.sim.seed == 42
    assert s.step.cclConnectivity == 8 and s.step.hydraulicIterations == 20
    # keys the engine does not know are skipped, the defaults stay
    assert s.kernel.continentalCrustThreshold == 10000.0


def test_config_json_rejects_malformed():
    with pytest.raises(T.TectoError):
        T.settings_from_json('{"heightmap_dimensions": {"x": }')


def test_generator_is_deterministic_and_follows_the_spec():
    h1, i1, p1 = T.generate_world(96, 64, 8, 1.0, 5)
    h2, i2, p2 = T.generate_world(96, 64, 8, 1.0, 5)
    np.testing.assert_array_equal(h1, h2)
    np.testing.assert_array_equal(i1, i2)
    np.testing.assert_array_equal(p1, p2)
    assert set(np.unique(i1)) <= set(range(8))
    cont = (i1 % 2) == 0
    assert abs(float(h1[cont].mean()) - 0.5) < 0.01 and abs(float(h1[~cont].mean()) + 0.5) < 0.01
    assert 0.03 < float(h1[cont].std()) < 0.07 and 0.01 < float(h1[~cont].std()) < 0.03
    v = p1[:8]
    vx = v["direction_x"] * v["velocity"]
    assert np.all(np.abs(vx) <= 1.0 + 1e-6) and np.all(v["velocity"] >= 0)
    assert np.all((v["pixelCenter_x"] >= 0) & (v["pixelCenter_x"] < 1))
    h3, _, _ = T.generate_world(96, 64, 8, 1.0, 6)
    assert not np.array_equal(h1, h3)


def test_invalid_arguments_are_rejected_without_touching_a_gpu():
    L = T.lib()
    s = T.default_settings()
    p = C.c_void_p()
    assert L.tecto_world_create(C.byref(s), 0, 10, 1, C.byref(p)) == -1
    assert L.tecto_world_create(None, 10, 10, 1, C.byref(p)) == -1
    assert L.tecto_world_create(C.byref(s), 1 << 16, 1 << 16, 1, C.byref(p)) == -1
    assert L.tecto_generate_world_host(8, 8, 0, 1.0, 1, None, None, None) == -1
    assert L.tecto_generate_world_host(8, 8, 256, 1.0, 1, None, None, None) == -1
    assert L.tecto_world_step(None, 1, None) == -1
    assert L.tecto_sort_pairs(None, None, None, None, 10, 8, None, 0, None) == -1
    assert L.tecto_sort_scratch_bytes(100, 0) == 0 and L.tecto_sort_scratch_bytes(100, 33) == 0
    assert L.tecto_sort_scratch_bytes(1 << 20, 20) > 4 * (1 << 22)
    assert L.tecto_sort_pairs_radix(None, None, None, None, 10, 8, 11, None, 0, None) == -1
    assert L.tecto_sort_scratch_bytes_radix(100, 20, 7) == 0 and L.tecto_sort_scratch_bytes_radix(100, 20, 12) == 0
    assert L.tecto_sort_scratch_bytes_radix(1 << 20, 20, 0) == L.tecto_sort_scratch_bytes(1 << 20, 20)
    assert L.tecto_sort_scratch_bytes_radix(1 << 20, 20, 11) > L.tecto_sort_scratch_bytes(1 << 20, 20)
    # the pass form for large sorts starts at 4096 tiles of 4096 keys
    assert L.tecto_sort_wide_pass(4096 * 4096) == 1 and L.tecto_sort_wide_pass(4096 * 4096 - 4096) == 0
    assert L.tecto_sort_wide_pass(4095 * 4096 + 1) == 1
    # the erosion kernels' arithmetic self-tests check their arguments before any device work
    assert L.tecto_selftest_div(None, None, None, 0, None) == 0
    assert L.tecto_selftest_div(None, None, None, 16, None) == -1
    assert L.tecto_selftest_div_var(None, None, None, 0, None) == 0
    assert L.tecto_selftest_div_var(None, None, None, 16, None) == -1
    assert L.tecto_selftest_rcp_sqrt(None, None) == -1
    assert L.tecto_world_destroy(None) == 0
