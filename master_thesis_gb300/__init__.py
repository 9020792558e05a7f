"""master_thesis_gb300 - GB300 (sm_103a) engine for the plate-tectonics simulation step.

Python binding of the C ABI in include/tecto.h (libtecto.so, built in-tree by _build.py).  The
engine itself is CUDA; this module only loads the library, mirrors its structs with ctypes and
offers a thin `World` wrapper.  There is no CPU fallback: if libtecto.so is missing or cannot be
loaded, `lib()` raises.
"""
from __future__ import annotations

import ctypes as C
import json
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libtecto.so"

TECTO_OK = 0
ERRORS = {
    -1: "TECTO_ERR_INVALID",
    -2: "TECTO_ERR_CUDA",
    -3: "TECTO_ERR_OOM",
    -4: "TECTO_ERR_DEVICE_TIMEOUT",
    -5: "TECTO_ERR_UNSUPPORTED",
    -6: "TECTO_ERR_BUDGET",
    -7: "TECTO_ERR_NOT_FOUND",
}
MAX_PLATES = 255
NUM_PAIRS = 32385
NUM_DIV_WORDS = 1013

UPLIFT_GAUSSIAN, UPLIFT_NONE, UPLIFT_REFERENCE = 0, 1, 2
CCL_4, CCL_8, CCL_REF8 = 4, 8, 9
PLATE_DYNAMICS_OFF, PLATE_DYNAMICS_REFERENCE = 0, 1
PLATE_RELABEL, PLATE_MERGE = 1, 2
PNG_GRAY16, PNG_RGB8, PNG_GRAY8 = 0, 1, 2
EXPORT_HEIGHT_GRAY16, EXPORT_PLATES_RGB = 0, 1
SERVER_OUT_HEIGHT_PNG, SERVER_OUT_PLATES_PNG, SERVER_OUT_SNAPSHOT = 1, 2, 4
SERVER_INIT_SYNTHETIC, SERVER_INIT_REFERENCE = 0, 1
REQUEST_WAITING, REQUEST_RUNNING, REQUEST_DONE = 0, 1, 2

(FIELD_HEIGHT, FIELD_WATER, FIELD_SEDIMENT, FIELD_FLUX, FIELD_PLATE_ID, FIELD_LABELS,
 FIELD_COLLISION, FIELD_TYPE_BITMAP, FIELD_DIV_BITMAP, FIELD_SORT_KEYS, FIELD_SORT_VALS,
 FIELD_ACCRETION, FIELD_JFA_SEED, FIELD_JFA_DIST) = range(14)

KERNEL_FIELDS = [
    ("inelasticCollisionMultiplierContinental", C.c_float),
    ("inelasticCollisionMultiplierSubduction", C.c_float),
    ("inelasticCollisionMultiplierAccretion", C.c_float),
    ("frictionCoefficientContinental", C.c_float),
    ("frictionCoefficientSubduction", C.c_float),
    ("frictionCoefficientAccretion", C.c_float),
    ("environmentalDragCoefficient", C.c_float),
    ("velocitySmoothingFactor", C.c_float),
    ("directionSmoothingFactor", C.c_float),
    ("breakScoreSmoothingFactor", C.c_float),
    ("mergeDotDirectionThreshold", C.c_float),
    ("mergeVelocityDiffThreshold", C.c_float),
    ("mergeMinVelocity", C.c_float),
    ("mergeWaitAfterSplit", C.c_int),
    ("minPlateSize", C.c_int),
    ("continentalCrustThreshold", C.c_float),
    ("divergence_height_target_min", C.c_float),
    ("divergence_height_target_max", C.c_float),
    ("divergence_interpolation_factor", C.c_float),
    ("collisionTypeUpdateCooldown", C.c_int),
    ("minCollisionSize", C.c_int),
    ("subductionOverUpliftMultiplier", C.c_float),
    ("subductionUnderUpliftMultiplier", C.c_float),
    ("continentalUpliftMultiplier", C.c_float),
    ("minUpliftClamp", C.c_float),
    ("maxUpliftClamp", C.c_float),
    ("upliftRange", C.c_int),
    ("subductionOverRange", C.c_int),
    ("continentalPropMaxIters", C.c_int),
    ("continentalPropThreshold", C.c_float),
    ("hydrationPipeCrossSection", C.c_float),
    ("hydrationPipeLength", C.c_float),
    ("hydrationRainfall", C.c_float),
    ("hydrationEvaporation", C.c_float),
    ("gravity", C.c_float),
    ("sedimentCapacity", C.c_float),
    ("sedimentErosionRate", C.c_float),
    ("sedimentDepositionRate", C.c_float),
    ("pressureAccumulation", C.c_float),
    ("pressureDecayRate", C.c_float),
    ("pressureBlurRange", C.c_int),
    ("pressureMultiplier", C.c_float),
    ("curlNoiseMultiplier", C.c_float),
    ("stressSplitThreshold", C.c_float),
    ("targetMinimumPlateArea", C.c_int),
    ("targetMaximumPlateArea", C.c_int),
    ("thermalErosionStrength", C.c_float),
    ("thermalErosionAmplitude", C.c_float),
    ("thermalCellSize", C.c_float),
    ("thermalThresholdAngle", C.c_float),
]


class KernelSettings(C.Structure):
    """tecto_kernel_settings: field-for-field mirror of the reference's KernelSettings."""
    _fields_ = KERNEL_FIELDS


class SimulationSettings(C.Structure):
    _fields_ = [
        ("numStartingPlates", C.c_int),
        ("seed", C.c_uint32),
        ("numVoronoiSeeds", C.c_int * 8),
        ("numVoronoiGenerations", C.c_int),
        ("iterationsForCCL", C.c_int),
    ]


class StepSettings(C.Structure):
    _fields_ = [
        ("hydraulicIterations", C.c_int),
        ("hydraulicDt", C.c_float),
        ("thermalIterations", C.c_int),
        ("upliftMode", C.c_int),
        ("upliftAmount", C.c_float),
        ("upliftSigma", C.c_float),
        ("upliftRadius", C.c_int),
        ("cclConnectivity", C.c_int),
        ("sortRadixBits", C.c_int),
        ("hydraulicTile", C.c_int),
        ("thermalTile", C.c_int),
        ("plateDynamics", C.c_int),
        ("platePolicy", C.c_int),
        ("reserved", C.c_int * 3),
    ]


class Settings(C.Structure):
    _fields_ = [("kernel", KernelSettings), ("sim", SimulationSettings), ("step", StepSettings)]

    def copy(self) -> "Settings":
        s = Settings()
        C.memmove(C.byref(s), C.byref(self), C.sizeof(Settings))
        return s


class Plate(C.Structure):
    _fields_ = [
        ("velocity", C.c_float),
        ("direction_x", C.c_float),
        ("direction_y", C.c_float),
        ("pixelCenter_x", C.c_float),
        ("pixelCenter_y", C.c_float),
    ]


class Request(C.Structure):
    """tecto_request: one world-generation job for the server."""
    _fields_ = [
        ("width", C.c_int), ("height", C.c_int), ("plates", C.c_int), ("steps", C.c_int),
        ("velRange", C.c_float), ("genSeed", C.c_uint64), ("worldSeed", C.c_uint32),
        ("arrival_s", C.c_double),
    ]


class RequestResult(C.Structure):
    _fields_ = [
        ("status", C.c_int), ("arrival_s", C.c_double), ("admit_s", C.c_double), ("finish_s", C.c_double),
        ("height_checksum", C.c_float),
    ]


class ServerStats(C.Structure):
    _fields_ = [
        ("completed", C.c_int), ("rejected", C.c_int), ("ticks", C.c_int), ("max_active", C.c_int),
        ("wall_s", C.c_double), ("cell_updates", C.c_double), ("cell_updates_per_s", C.c_double),
        ("latency_p50_s", C.c_double), ("latency_p99_s", C.c_double), ("latency_mean_s", C.c_double),
        ("peak_bytes", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Tuning(C.Structure):
    """tecto_tuning: the autotuner's choice and the per-candidate timings."""
    _fields_ = [
        ("hydraulicTile", C.c_int), ("sortRadixBits", C.c_int), ("thermalTile", C.c_int),
        ("hydraulic_ms", C.c_float * 9), ("sort_ms", C.c_float * 4), ("thermal_ms", C.c_float * 5),
    ]

    def as_dict(self) -> dict:
        return {"hydraulicTile": self.hydraulicTile, "sortRadixBits": self.sortRadixBits,
                "thermalTile": self.thermalTile,
                "hydraulic_ms": [round(x, 4) for x in self.hydraulic_ms],
                "sort_ms": [round(x, 4) for x in self.sort_ms],
                "thermal_ms": [round(x, 4) for x in self.thermal_ms]}


SERVER_DRY_RUN = 1

PLATE_DTYPE = np.dtype(
    [("velocity", "<f4"), ("direction_x", "<f4"), ("direction_y", "<f4"),
     ("pixelCenter_x", "<f4"), ("pixelCenter_y", "<f4")]
)

PLATE_DYNAMICS_DTYPE = np.dtype(
    [("velocitySmoothed", "<f4"), ("directionSmoothed_x", "<f4"), ("directionSmoothed_y", "<f4"),
     ("geometricCenter_x", "<f4"), ("geometricCenter_y", "<f4"), ("mass", "<f4"), ("size", "<i4"),
     ("mergeWaitTime", "<i4"), ("frictionLoss", "<f4")]
)

_lib = None


class TectoError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str = ""):
        super().__init__(f"{where}: {ERRORS.get(code, code)} {msg}")
        self.code = code


def _declare(L: C.CDLL) -> None:
    P = C.c_void_p
    sig = {
        "tecto_settings_default": ([C.POINTER(Settings)], C.c_int),
        "tecto_settings_baseline": ([C.POINTER(Settings)], C.c_int),
        "tecto_settings_from_json": ([C.c_char_p, C.POINTER(Settings), C.POINTER(C.c_int), C.POINTER(C.c_int)], C.c_int),
        "tecto_world_create": ([C.POINTER(Settings), C.c_int, C.c_int, C.c_uint32, C.POINTER(P)], C.c_int),
        "tecto_world_destroy": ([P], C.c_int),
        "tecto_world_set_settings": ([P, C.POINTER(Settings)], C.c_int),
        "tecto_world_get_settings": ([P, C.POINTER(Settings)], C.c_int),
        "tecto_world_size": ([P, C.POINTER(C.c_int), C.POINTER(C.c_int)], C.c_int),
        "tecto_generate_world_host": ([C.c_int, C.c_int, C.c_int, C.c_float, C.c_uint64, P, P, P], C.c_int),
        "tecto_world_init_synthetic": ([P, C.c_int, C.c_float, C.c_uint64, P], C.c_int),
        "tecto_world_upload": ([P, C.c_int, P, C.c_size_t, P], C.c_int),
        "tecto_world_download": ([P, C.c_int, P, C.c_size_t, P], C.c_int),
        "tecto_world_upload_async": ([P, C.c_int, P, C.c_size_t, P], C.c_int),
        "tecto_world_download_async": ([P, C.c_int, P, C.c_size_t, P], C.c_int),
        "tecto_world_field": ([P, C.c_int, C.POINTER(P), C.POINTER(C.c_size_t)], C.c_int),
        "tecto_world_set_plates": ([P, P, C.c_int, P], C.c_int),
        "tecto_world_get_plates": ([P, P, C.c_int, P], C.c_int),
        "tecto_world_set_iteration": ([P, C.c_uint32], C.c_int),
        "tecto_world_set_plate_dynamics": ([P, P, C.c_int, P], C.c_int),
        "tecto_world_get_plate_dynamics": ([P, P, C.c_int, P], C.c_int),
        "tecto_world_set_asthenosphere": ([P, P, C.c_int, C.c_int, P], C.c_int),
        "tecto_world_get_iteration": ([P, C.POINTER(C.c_uint32)], C.c_int),
        "tecto_world_step": ([P, C.c_int, P], C.c_int),
        "tecto_phase_collide": ([P, P], C.c_int),
        "tecto_phase_resolve": ([P, P], C.c_int),
        "tecto_phase_thermal": ([P, C.c_int, P], C.c_int),
        "tecto_phase_hydraulic": ([P, C.c_int, C.c_float, P], C.c_int),
        "tecto_phase_finish": ([P, P], C.c_int),
        "tecto_phase_ccl": ([P, C.c_int, P], C.c_int),
        "tecto_sort_scratch_bytes": ([C.c_size_t, C.c_int], C.c_size_t),
        "tecto_sort_pairs": ([P, P, P, P, C.c_size_t, C.c_int, P, C.c_size_t, P], C.c_int),
        "tecto_sort_scratch_bytes_radix": ([C.c_size_t, C.c_int, C.c_int], C.c_size_t),
        "tecto_sort_pairs_radix": ([P, P, P, P, C.c_size_t, C.c_int, C.c_int, P, C.c_size_t, P], C.c_int),
        "tecto_sort_wide_pass": ([C.c_size_t], C.c_int),
        "tecto_sort_pairs_noalloc": ([P, P, P, P, C.c_size_t, C.c_int, P], C.c_int),
        "tecto_world_check": ([P, P], C.c_int),
        "tecto_world_launch_count": ([P, C.POINTER(C.c_uint64)], C.c_int),
        "tecto_world_bytes": ([C.c_int, C.c_int], C.c_size_t),
        "tecto_world_init_synthetic_device": ([P, C.c_int, C.c_float, C.c_uint64, P], C.c_int),
        "tecto_world_init_reference": ([P, P], C.c_int),
        "tecto_world_init": ([P, C.c_int, P, C.c_int, P], C.c_int),
        "tecto_reference_seeds": ([C.c_int, C.c_int, C.c_uint32, C.c_int, P, C.c_int, P, P, P, C.c_int,
                                   C.POINTER(C.c_int), P, P], C.c_int),
        "tecto_batch_create": ([C.POINTER(P)], C.c_int),
        "tecto_batch_destroy": ([P], C.c_int),
        "tecto_batch_add": ([P, P, P], C.c_int),
        "tecto_batch_remove": ([P, P], C.c_int),
        "tecto_batch_step": ([P, C.c_int, P], C.c_int),
        "tecto_batch_size": ([P, C.POINTER(C.c_int), C.POINTER(C.c_size_t)], C.c_int),
        "tecto_batch_launch_count": ([P, C.POINTER(C.c_uint64)], C.c_int),
        "tecto_batch_check": ([P, P], C.c_int),
        "tecto_batch_phase_hydraulic": ([P, C.c_int, C.c_float, P], C.c_int),
        "tecto_batch_phase_thermal": ([P, C.c_int, P], C.c_int),
        "tecto_batch_upload_async": ([P, C.c_int, P, C.c_size_t, P], C.c_int),
        "tecto_batch_download_async": ([P, C.c_int, P, C.c_size_t, P], C.c_int),
        "tecto_batch_offsets": ([P, C.POINTER(C.c_size_t), C.c_int], C.c_int),
        "tecto_batch_stage_upload_async": ([P, C.c_int, P, C.c_size_t, P], C.c_int),
        "tecto_batch_commit_upload": ([P, C.c_int, P], C.c_int),
        "tecto_batch_gather_download": ([P, C.c_int, P], C.c_int),
        "tecto_batch_fetch_download_async": ([P, C.c_int, P, C.c_size_t, P], C.c_int),
        "tecto_autotune": ([C.POINTER(Settings), P, P, C.c_int, P, C.POINTER(Tuning)], C.c_int),
        "tecto_batch_autotune": ([P, P, C.POINTER(Tuning)], C.c_int),
        "tecto_world_autotune": ([P, P, C.POINTER(Tuning)], C.c_int),
        "tecto_autotune_record": ([C.c_int, C.c_size_t, C.c_int, C.c_int, C.c_int, C.c_int], C.c_int),
        "tecto_autotune_lookup": ([C.c_int, C.c_size_t, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.c_int)], C.c_int),
        "tecto_autotune_clear": ([], C.c_int),
        "tecto_server_create": ([C.POINTER(Settings), C.c_size_t, C.c_int, C.c_int, C.POINTER(P)], C.c_int),
        "tecto_server_destroy": ([P], C.c_int),
        "tecto_server_run_trace": ([P, C.POINTER(Request), C.c_int, P, C.POINTER(RequestResult),
                                    C.POINTER(ServerStats)], C.c_int),
        "tecto_server_run_trace_sequential": ([P, C.POINTER(Request), C.c_int, P, C.POINTER(RequestResult),
                                               C.POINTER(ServerStats)], C.c_int),
        "tecto_server_set_dry_cost": ([P, C.c_double], C.c_int),
        "tecto_server_set_policy": ([P, C.c_size_t, C.c_int], C.c_int),
        "tecto_server_set_init": ([P, C.c_int], C.c_int),
        "tecto_server_set_output": ([P, C.c_char_p, C.c_int, C.c_float, C.c_float], C.c_int),
        "tecto_server_submit": ([P, C.POINTER(Request), C.POINTER(C.c_int)], C.c_int),
        "tecto_server_tick": ([P, P, C.POINTER(C.c_int), C.POINTER(C.c_int)], C.c_int),
        "tecto_server_poll": ([P, C.c_int, C.POINTER(C.c_int), C.POINTER(RequestResult)], C.c_int),
        "tecto_server_live_stats": ([P, C.POINTER(ServerStats)], C.c_int),
        "tecto_selftest_div": ([P, P, P, C.c_size_t, P], C.c_int),
        "tecto_selftest_div_var": ([P, P, P, C.c_size_t, P], C.c_int),
        "tecto_selftest_rcp_sqrt": ([P, P], C.c_int),
        "tecto_png_encode": ([P, C.c_int, C.c_int, C.c_int, P, C.c_size_t, C.POINTER(C.c_size_t)], C.c_int),
        "tecto_plate_palette": ([P], C.c_int),
        "tecto_world_export_png": ([P, C.c_int, C.c_char_p, C.c_float, C.c_float, P], C.c_int),
        "tecto_world_save_snapshot": ([P, C.c_char_p, P], C.c_int),
        "tecto_world_load_snapshot": ([P, C.c_char_p, P], C.c_int),
        "tecto_snapshot_info": ([C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(Settings)], C.c_int),
        "tecto_last_error_string": ([], C.c_char_p),
        "tecto_version": ([], C.c_char_p),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res


def lib() -> C.CDLL:
    """The loaded engine library.  Raises if it has not been built (no fallback exists)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
            )
        L = C.CDLL(str(LIB_PATH))
        _declare(L)
        _lib = L
    return _lib


def check(code: int, where: str) -> None:
    if code != TECTO_OK:
        raise TectoError(code, where, lib().tecto_last_error_string().decode(errors="replace"))


def default_settings() -> Settings:
    s = Settings()
    check(lib().tecto_settings_default(C.byref(s)), "tecto_settings_default")
    return s


def baseline_settings() -> Settings:
    s = Settings()
    check(lib().tecto_settings_baseline(C.byref(s)), "tecto_settings_baseline")
    return s


def settings_from_json(text: str, base: Settings | None = None) -> tuple[Settings, int, int]:
    s = (base or default_settings()).copy()
    w, h = C.c_int(0), C.c_int(0)
    check(lib().tecto_settings_from_json(text.encode(), C.byref(s), C.byref(w), C.byref(h)),
          "tecto_settings_from_json")
    return s, w.value, h.value


def generate_world(W: int, H: int, plates: int, vel_range: float, gen_seed: int):
    """Host-only synthetic world: (height f32[H,W], plate id u8[H,W], plates structured[255])."""
    h = np.empty((H, W), np.float32)
    ids = np.empty((H, W), np.uint8)
    pl = np.zeros(MAX_PLATES, PLATE_DTYPE)
    check(lib().tecto_generate_world_host(W, H, plates, vel_range, gen_seed, h.ctypes.data,
                                          ids.ctypes.data, pl.ctypes.data), "tecto_generate_world_host")
    return h, ids, pl


_FIELD_DT = {
    FIELD_HEIGHT: (np.float32, 1), FIELD_WATER: (np.float32, 1), FIELD_SEDIMENT: (np.float32, 1),
    FIELD_FLUX: (np.float32, 4), FIELD_PLATE_ID: (np.uint8, 1), FIELD_LABELS: (np.uint32, 1),
    FIELD_COLLISION: (np.uint32, 1), FIELD_SORT_KEYS: (np.uint32, 1), FIELD_SORT_VALS: (np.uint32, 1),
    FIELD_ACCRETION: (np.uint8, 1), FIELD_JFA_SEED: (np.int32, 1), FIELD_JFA_DIST: (np.int32, 1),
}


def _stream(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return int(getattr(stream, "cuda_stream", stream))


class World:
    """One simulated world on the current GPU (tecto_world)."""

    def __init__(self, settings: Settings, W: int, H: int, seed: int = 1000):
        self.W, self.H = W, H
        p = C.c_void_p()
        check(lib().tecto_world_create(C.byref(settings), W, H, seed, C.byref(p)), "tecto_world_create")
        self.ptr = p

    def close(self) -> None:
        if getattr(self, "ptr", None):
            lib().tecto_world_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def init_synthetic(self, plates: int, vel_range: float, gen_seed: int, stream=None) -> None:
        check(lib().tecto_world_init_synthetic(self.ptr, plates, vel_range, gen_seed, _stream(stream)),
              "tecto_world_init_synthetic")

    def set_settings(self, s: Settings) -> None:
        check(lib().tecto_world_set_settings(self.ptr, C.byref(s)), "tecto_world_set_settings")

    def download(self, field: int, stream=None) -> np.ndarray:
        if field == FIELD_TYPE_BITMAP:
            out = np.empty(NUM_PAIRS, np.uint8)
        elif field == FIELD_DIV_BITMAP:
            out = np.empty(NUM_DIV_WORDS, np.uint32)
        else:
            dt, k = _FIELD_DT[field]
            out = np.empty((self.H, self.W, k) if k > 1 else (self.H, self.W), dt)
        check(lib().tecto_world_download(self.ptr, field, out.ctypes.data, out.nbytes, _stream(stream)),
              "tecto_world_download")
        return out

    def upload(self, field: int, arr: np.ndarray, stream=None) -> None:
        a = np.ascontiguousarray(arr)
        check(lib().tecto_world_upload(self.ptr, field, a.ctypes.data, a.nbytes, _stream(stream)),
              "tecto_world_upload")

    def plates(self, stream=None) -> np.ndarray:
        out = np.zeros(MAX_PLATES, PLATE_DTYPE)
        check(lib().tecto_world_get_plates(self.ptr, out.ctypes.data, MAX_PLATES, _stream(stream)),
              "tecto_world_get_plates")
        return out

    def set_plates(self, plates: np.ndarray, stream=None) -> None:
        a = np.ascontiguousarray(plates, dtype=PLATE_DTYPE)
        check(lib().tecto_world_set_plates(self.ptr, a.ctypes.data, len(a), _stream(stream)),
              "tecto_world_set_plates")

    def plate_dynamics(self, stream=None) -> np.ndarray:
        out = np.zeros(MAX_PLATES, PLATE_DYNAMICS_DTYPE)
        check(lib().tecto_world_get_plate_dynamics(self.ptr, out.ctypes.data, MAX_PLATES, _stream(stream)),
              "tecto_world_get_plate_dynamics")
        return out

    def set_plate_dynamics(self, records: np.ndarray, stream=None) -> None:
        a = np.ascontiguousarray(records, dtype=PLATE_DYNAMICS_DTYPE)
        check(lib().tecto_world_set_plate_dynamics(self.ptr, a.ctypes.data, len(a), _stream(stream)),
              "tecto_world_set_plate_dynamics")

    def set_asthenosphere(self, pressure: np.ndarray | None, stream=None) -> None:
        """The asthenosphere pressure texture (float [ph, pw]); None removes it."""
        if pressure is None:
            check(lib().tecto_world_set_asthenosphere(self.ptr, None, 0, 0, _stream(stream)),
                  "tecto_world_set_asthenosphere")
            return
        a = np.ascontiguousarray(pressure, dtype=np.float32)
        check(lib().tecto_world_set_asthenosphere(self.ptr, a.ctypes.data, a.shape[1], a.shape[0], _stream(stream)),
              "tecto_world_set_asthenosphere")

    @property
    def iteration(self) -> int:
        v = C.c_uint32()
        check(lib().tecto_world_get_iteration(self.ptr, C.byref(v)), "tecto_world_get_iteration")
        return v.value

    @iteration.setter
    def iteration(self, v: int) -> None:
        check(lib().tecto_world_set_iteration(self.ptr, v), "tecto_world_set_iteration")

    def step(self, n: int = 1, stream=None) -> None:
        check(lib().tecto_world_step(self.ptr, n, _stream(stream)), "tecto_world_step")

    def collide(self, stream=None):
        check(lib().tecto_phase_collide(self.ptr, _stream(stream)), "tecto_phase_collide")

    def resolve(self, stream=None):
        check(lib().tecto_phase_resolve(self.ptr, _stream(stream)), "tecto_phase_resolve")

    def thermal(self, iters: int, stream=None):
        check(lib().tecto_phase_thermal(self.ptr, iters, _stream(stream)), "tecto_phase_thermal")

    def hydraulic(self, iters: int, dt: float, stream=None):
        check(lib().tecto_phase_hydraulic(self.ptr, iters, dt, _stream(stream)), "tecto_phase_hydraulic")

    def autotune(self, stream=None) -> Tuning:
        t = Tuning()
        check(lib().tecto_world_autotune(self.ptr, _stream(stream), C.byref(t)), "tecto_world_autotune")
        return t

    def finish(self, stream=None):
        check(lib().tecto_phase_finish(self.ptr, _stream(stream)), "tecto_phase_finish")

    def ccl(self, connectivity: int, stream=None):
        check(lib().tecto_phase_ccl(self.ptr, connectivity, _stream(stream)), "tecto_phase_ccl")

    @property
    def launches(self) -> int:
        v = C.c_uint64()
        check(lib().tecto_world_launch_count(self.ptr, C.byref(v)), "tecto_world_launch_count")
        return v.value

    def check(self, stream=None):
        check(lib().tecto_world_check(self.ptr, _stream(stream)), "tecto_world_check")

    def export_png(self, kind: int, path, min_value: float = 0.0, max_value: float = 1.0, stream=None) -> None:
        """Write the height map (EXPORT_HEIGHT_GRAY16, normalised over [min_value, max_value]) or
        the plate ids (EXPORT_PLATES_RGB) as a PNG file."""
        check(lib().tecto_world_export_png(self.ptr, kind, os.fsencode(path), min_value, max_value,
                                           _stream(stream)), "tecto_world_export_png")

    def save_snapshot(self, path, stream=None) -> None:
        check(lib().tecto_world_save_snapshot(self.ptr, os.fsencode(path), _stream(stream)),
              "tecto_world_save_snapshot")

    def load_snapshot(self, path, stream=None) -> None:
        check(lib().tecto_world_load_snapshot(self.ptr, os.fsencode(path), _stream(stream)),
              "tecto_world_load_snapshot")

    @classmethod
    def from_snapshot(cls, path, stream=None) -> "World":
        """A new world of the snapshot's size and settings, holding its state."""
        W, H, s = snapshot_info(path)
        w = cls(s, W, H)
        w.load_snapshot(path, stream)
        return w


def snapshot_info(path) -> tuple[int, int, Settings]:
    W, H, s = C.c_int(0), C.c_int(0), Settings()
    check(lib().tecto_snapshot_info(os.fsencode(path), C.byref(W), C.byref(H), C.byref(s)),
          "tecto_snapshot_info")
    return W.value, H.value, s


def plate_palette() -> np.ndarray:
    """The RGB colour of each plate id in the plate export: uint8[256, 3]."""
    out = np.empty((256, 3), np.uint8)
    check(lib().tecto_plate_palette(out.ctypes.data), "tecto_plate_palette")
    return out


def png_encode(pixels: np.ndarray, kind: int) -> bytes:
    """PNG file bytes of a host image: PNG_GRAY16 (uint16 [H,W]), PNG_RGB8 (uint8 [H,W,3]) or
    PNG_GRAY8 (uint8 [H,W])."""
    dt, nd = {PNG_GRAY16: (np.uint16, 2), PNG_RGB8: (np.uint8, 3), PNG_GRAY8: (np.uint8, 2)}[kind]
    a = np.ascontiguousarray(pixels, dtype=dt)
    if a.ndim != nd or (kind == PNG_RGB8 and a.shape[2] != 3):
        raise ValueError(f"png_encode: bad image shape {a.shape} for kind {kind}")
    n = C.c_size_t(0)
    H, W = a.shape[0], a.shape[1]
    check(lib().tecto_png_encode(a.ctypes.data, W, H, kind, None, 0, C.byref(n)), "tecto_png_encode")
    out = C.create_string_buffer(n.value)
    check(lib().tecto_png_encode(a.ctypes.data, W, H, kind, out, n.value, C.byref(n)), "tecto_png_encode")
    return out.raw[: n.value]


def _world_init_device(self, plates: int, vel_range: float, gen_seed: int, stream=None) -> None:
    check(lib().tecto_world_init_synthetic_device(self.ptr, plates, vel_range, gen_seed, _stream(stream)),
          "tecto_world_init_synthetic_device")


World.init_synthetic_device = _world_init_device


def _world_init_reference(self, stream=None) -> None:
    """The reference's initialisation (initializeTectonics) from the world's settings and seed."""
    check(lib().tecto_world_init_reference(self.ptr, _stream(stream)), "tecto_world_init_reference")


World.init_reference = _world_init_reference


def reference_seeds(W: int, H: int, seed: int, num_plates: int, gens):
    """The host draws of the reference's initialisation: (seed x, seed y, seed plate id, plates,
    plate dynamics records)."""
    g = np.ascontiguousarray(gens, np.int32)
    cap = max([num_plates] + [int(v) for v in g])
    sx, sy = np.zeros(cap, np.float32), np.zeros(cap, np.float32)
    sid = np.zeros(cap, np.uint8)
    n = C.c_int(0)
    pl = np.zeros(MAX_PLATES, PLATE_DTYPE)
    dy = np.zeros(MAX_PLATES, PLATE_DYNAMICS_DTYPE)
    check(lib().tecto_reference_seeds(W, H, seed, num_plates, g.ctypes.data if len(g) else None, len(g),
                                      sx.ctypes.data, sy.ctypes.data, sid.ctypes.data, cap, C.byref(n),
                                      pl.ctypes.data, dy.ctypes.data), "tecto_reference_seeds")
    k = n.value
    return sx[:k].copy(), sy[:k].copy(), sid[:k].copy(), pl, dy


def world_bytes(W: int, H: int) -> int:
    return int(lib().tecto_world_bytes(W, H))


class Batch:
    """Many worlds advanced together, one kernel launch per phase (tecto_batch)."""

    def __init__(self):
        p = C.c_void_p()
        check(lib().tecto_batch_create(C.byref(p)), "tecto_batch_create")
        self.ptr = p
        self.worlds: list[World] = []

    def add(self, world: World, stream=None) -> None:
        check(lib().tecto_batch_add(self.ptr, world.ptr, _stream(stream)), "tecto_batch_add")
        self.worlds.append(world)

    def remove(self, world: World) -> None:
        check(lib().tecto_batch_remove(self.ptr, world.ptr), "tecto_batch_remove")
        self.worlds.remove(world)

    def step(self, n: int = 1, stream=None) -> None:
        check(lib().tecto_batch_step(self.ptr, n, _stream(stream)), "tecto_batch_step")

    def size(self) -> tuple[int, int]:
        nw, nc = C.c_int(), C.c_size_t()
        check(lib().tecto_batch_size(self.ptr, C.byref(nw), C.byref(nc)), "tecto_batch_size")
        return nw.value, nc.value

    @property
    def launches(self) -> int:
        v = C.c_uint64()
        check(lib().tecto_batch_launch_count(self.ptr, C.byref(v)), "tecto_batch_launch_count")
        return v.value

    def check(self, stream=None) -> None:
        check(lib().tecto_batch_check(self.ptr, _stream(stream)), "tecto_batch_check")

    def hydraulic(self, iters: int, dt: float, stream=None) -> None:
        check(lib().tecto_batch_phase_hydraulic(self.ptr, iters, dt, _stream(stream)), "tecto_batch_phase_hydraulic")

    def thermal(self, iters: int, stream=None) -> None:
        check(lib().tecto_batch_phase_thermal(self.ptr, iters, _stream(stream)), "tecto_batch_phase_thermal")

    def offsets(self) -> np.ndarray:
        """First cell of each member in the packed layout, then the total."""
        n, _ = self.size()
        out = (C.c_size_t * (n + 1))()
        check(lib().tecto_batch_offsets(self.ptr, out, n + 1), "tecto_batch_offsets")
        return np.array(out[:], np.int64)

    def upload_packed_async(self, field: int, host_ptr: int, nbytes: int, stream=None) -> None:
        check(lib().tecto_batch_upload_async(self.ptr, field, host_ptr, nbytes, _stream(stream)),
              "tecto_batch_upload_async")

    def download_packed_async(self, field: int, host_ptr: int, nbytes: int, stream=None) -> None:
        check(lib().tecto_batch_download_async(self.ptr, field, host_ptr, nbytes, _stream(stream)),
              "tecto_batch_download_async")

    def autotune(self, stream=None) -> Tuning:
        t = Tuning()
        check(lib().tecto_batch_autotune(self.ptr, _stream(stream), C.byref(t)), "tecto_batch_autotune")
        return t

    def close(self) -> None:
        if getattr(self, "ptr", None):
            lib().tecto_batch_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(settings: Settings, shapes, stream=None) -> Tuning:
    """Tune the hydraulic tile and sort digit width for worlds of these (width, height) shapes."""
    n = len(shapes)
    ws = (C.c_int * n)(*[int(w) for w, _ in shapes])
    hs = (C.c_int * n)(*[int(h) for _, h in shapes])
    t = Tuning()
    check(lib().tecto_autotune(C.byref(settings), ws, hs, n, _stream(stream), C.byref(t)), "tecto_autotune")
    return t


def autotune_record(device: int, total_cells: int, worlds: int, hydraulic_tile: int, radix_bits: int,
                    thermal_tile: int = 3) -> None:
    check(lib().tecto_autotune_record(device, total_cells, worlds, hydraulic_tile, radix_bits, thermal_tile),
          "tecto_autotune_record")


def autotune_lookup(device: int, total_cells: int, worlds: int):
    """(hydraulicTile, sortRadixBits, thermalTile) cached for the class, or None."""
    h, r, t = C.c_int(), C.c_int(), C.c_int()
    rc = lib().tecto_autotune_lookup(device, total_cells, worlds, C.byref(h), C.byref(r), C.byref(t))
    if rc == -7:
        return None
    check(rc, "tecto_autotune_lookup")
    return h.value, r.value, t.value


def autotune_clear() -> None:
    check(lib().tecto_autotune_clear(), "tecto_autotune_clear")


class Server:
    """Continuous-batching server for world-generation requests (tecto_server)."""

    def __init__(self, settings: Settings, budget_bytes: int, max_worlds: int = 0, dry_run: bool = False):
        p = C.c_void_p()
        check(lib().tecto_server_create(C.byref(settings), budget_bytes, max_worlds,
                                        SERVER_DRY_RUN if dry_run else 0, C.byref(p)), "tecto_server_create")
        self.ptr = p

    def set_output(self, directory, what: int, height_min: float = 0.0, height_max: float = 1.0) -> None:
        """Write finished requests' exports and snapshots (SERVER_OUT_* bits) into `directory`."""
        d = os.fsencode(directory) if directory is not None else None
        check(lib().tecto_server_set_output(self.ptr, d, what, height_min, height_max), "tecto_server_set_output")

    def set_init(self, mode: int) -> None:
        """SERVER_INIT_SYNTHETIC (default) or SERVER_INIT_REFERENCE for admitted worlds."""
        check(lib().tecto_server_set_init(self.ptr, mode), "tecto_server_set_init")

    def set_dry_cost(self, seconds_per_mcell_step: float) -> None:
        check(lib().tecto_server_set_dry_cost(self.ptr, seconds_per_mcell_step), "tecto_server_set_dry_cost")

    def set_policy(self, heavy_cells: int, heavy_slots: int) -> None:
        """Requests of at least heavy_cells cells are live at most heavy_slots at a time (0: no limit)."""
        check(lib().tecto_server_set_policy(self.ptr, heavy_cells, heavy_slots), "tecto_server_set_policy")

    def _run(self, fn, requests, stream):
        n = len(requests)
        reqs = (Request * max(n, 1))(*requests)
        res = (RequestResult * max(n, 1))()
        st = ServerStats()
        check(fn(self.ptr, reqs, n, _stream(stream), res, C.byref(st)), fn.__name__)
        return list(res)[:n], st

    def run_trace(self, requests, stream=None):
        return self._run(lib().tecto_server_run_trace, requests, stream)

    def run_trace_sequential(self, requests, stream=None):
        return self._run(lib().tecto_server_run_trace_sequential, requests, stream)

    # live serving: submit as requests come, drive the ticks, poll for results
    def submit(self, request) -> int:
        """Queue a request; returns its ticket (arrival time = now on the server clock)."""
        t = C.c_int()
        check(lib().tecto_server_submit(self.ptr, C.byref(request), C.byref(t)), "tecto_server_submit")
        return t.value

    def tick(self, stream=None):
        """Admit, advance every admitted world one step, retire; returns (active, waiting)."""
        a, w = C.c_int(), C.c_int()
        check(lib().tecto_server_tick(self.ptr, _stream(stream), C.byref(a), C.byref(w)), "tecto_server_tick")
        return a.value, w.value

    def poll(self, ticket: int):
        """(state, RequestResult) of a ticket; state is REQUEST_WAITING / RUNNING / DONE."""
        st, r = C.c_int(), RequestResult()
        check(lib().tecto_server_poll(self.ptr, ticket, C.byref(st), C.byref(r)), "tecto_server_poll")
        return st.value, r

    def drain(self, stream=None, max_ticks: int = 1 << 30) -> int:
        """Tick until nothing is admitted or waiting; returns the ticks taken."""
        n = 0
        while n < max_ticks:
            a, w = self.tick(stream)
            n += 1
            if a == 0 and w == 0:
                break
        return n

    def live_stats(self) -> ServerStats:
        st = ServerStats()
        check(lib().tecto_server_live_stats(self.ptr, C.byref(st)), "tecto_server_live_stats")
        return st

    def close(self) -> None:
        if getattr(self, "ptr", None):
            lib().tecto_server_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def load_config(path: str | os.PathLike) -> tuple[Settings, int, int]:
    """Read a reference-style config.json (plus optional settings objects)."""
    return settings_from_json(Path(path).read_text())


__all__ = [n for n in dir() if not n.startswith("_")]
