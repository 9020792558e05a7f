"""Python access to the CPU oracle (oracle/_build/liboracle.so) and, where it has been built here,
to the reference's own kernels compiled for the CPU (oracle/_ref/libtecto_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline and reference legs; never by the engine.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libtecto_ref.so"

_o = None
_r = None


def reference_root() -> str:
    """Where the reference's sources are read from: $TECTO_REFERENCE, else /root/reference."""
    return os.environ.get("TECTO_REFERENCE", "/root/reference")


def build(ref: bool = False) -> None:
    """make the oracle and the reference-GPU timing harness (and, with ref=True, the
    reference-on-CPU library and the reference's device code for the GPU, from the sources under
    reference_root())."""
    targets = ["all", "harness"] + (["ref", "refgpu", "refexport"] if ref else [])
    subprocess.run(["make", "-s", "-C", str(HERE), f"REF={reference_root()}", *targets], check=True)


# ---- the C ABI's settings and plate layouts (include/tecto.h), mirrored here so that the CPU-only
# legs never import or load the engine; tests/test_oracle_units.py checks them against the engine's

MAX_PLATES = 255

_KERNEL_FLOATS_INTS = (
    "f:inelasticCollisionMultiplierContinental f:inelasticCollisionMultiplierSubduction "
    "f:inelasticCollisionMultiplierAccretion f:frictionCoefficientContinental f:frictionCoefficientSubduction "
    "f:frictionCoefficientAccretion f:environmentalDragCoefficient f:velocitySmoothingFactor "
    "f:directionSmoothingFactor f:breakScoreSmoothingFactor f:mergeDotDirectionThreshold "
    "f:mergeVelocityDiffThreshold f:mergeMinVelocity i:mergeWaitAfterSplit i:minPlateSize "
    "f:continentalCrustThreshold f:divergence_height_target_min f:divergence_height_target_max "
    "f:divergence_interpolation_factor i:collisionTypeUpdateCooldown i:minCollisionSize "
    "f:subductionOverUpliftMultiplier f:subductionUnderUpliftMultiplier f:continentalUpliftMultiplier "
    "f:minUpliftClamp f:maxUpliftClamp i:upliftRange i:subductionOverRange i:continentalPropMaxIters "
    "f:continentalPropThreshold f:hydrationPipeCrossSection f:hydrationPipeLength f:hydrationRainfall "
    "f:hydrationEvaporation f:gravity f:sedimentCapacity f:sedimentErosionRate f:sedimentDepositionRate "
    "f:pressureAccumulation f:pressureDecayRate i:pressureBlurRange f:pressureMultiplier f:curlNoiseMultiplier "
    "f:stressSplitThreshold i:targetMinimumPlateArea i:targetMaximumPlateArea f:thermalErosionStrength "
    "f:thermalErosionAmplitude f:thermalCellSize f:thermalThresholdAngle"
)


class KernelSettings(C.Structure):
    """tecto_kernel_settings: the reference's KernelSettings, field for field."""
    _fields_ = [(f.split(":")[1], C.c_float if f[0] == "f" else C.c_int) for f in _KERNEL_FLOATS_INTS.split()]


class SimulationSettings(C.Structure):
    _fields_ = [("numStartingPlates", C.c_int), ("seed", C.c_uint32), ("numVoronoiSeeds", C.c_int * 8),
                ("numVoronoiGenerations", C.c_int), ("iterationsForCCL", C.c_int)]


class StepSettings(C.Structure):
    _fields_ = [("hydraulicIterations", C.c_int), ("hydraulicDt", C.c_float), ("thermalIterations", C.c_int),
                ("upliftMode", C.c_int), ("upliftAmount", C.c_float), ("upliftSigma", C.c_float),
                ("upliftRadius", C.c_int), ("cclConnectivity", C.c_int), ("sortRadixBits", C.c_int),
                ("hydraulicTile", C.c_int), ("thermalTile", C.c_int), ("plateDynamics", C.c_int),
                ("platePolicy", C.c_int), ("reserved", C.c_int * 3)]


class Settings(C.Structure):
    _fields_ = [("kernel", KernelSettings), ("sim", SimulationSettings), ("step", StepSettings)]


PLATE_DTYPE = np.dtype([("velocity", "<f4"), ("direction_x", "<f4"), ("direction_y", "<f4"),
                        ("pixelCenter_x", "<f4"), ("pixelCenter_y", "<f4")])
PLATE_DYNAMICS_DTYPE = np.dtype(
    [("velocitySmoothed", "<f4"), ("directionSmoothed_x", "<f4"), ("directionSmoothed_y", "<f4"),
     ("geometricCenter_x", "<f4"), ("geometricCenter_y", "<f4"), ("mass", "<f4"), ("size", "<i4"),
     ("mergeWaitTime", "<i4"), ("frictionLoss", "<f4")]
)


def default_settings() -> Settings:
    """The reference's defaults (or_settings_default)."""
    s = Settings()
    lib().or_settings_default(C.addressof(s))
    return s


def baseline_settings() -> Settings:
    """The benchmark physics on the reference's parameters (or_settings_baseline)."""
    s = Settings()
    lib().or_settings_baseline(C.addressof(s))
    return s


def generate_world(W: int, H: int, plates: int, vel_range: float, gen_seed: int):
    """The benchmark's synthetic world (or_generate_world): (height f32[H,W], plate id u8[H,W],
    plates[255])."""
    h = np.empty((H, W), np.float32)
    ids = np.empty((H, W), np.uint8)
    pl = np.zeros(MAX_PLATES, PLATE_DTYPE)
    if lib().or_generate_world(W, H, plates, vel_range, gen_seed, h.ctypes.data, ids.ctypes.data, pl.ctypes.data):
        raise ValueError("or_generate_world: invalid size or plate count (1..255)")
    return h, ids, pl


REF_CUBIN = HERE / "_ref" / "ref_kernels.cubin"
REF_GPU_LIB = HERE / "_build" / "libref_gpu.so"


def ref_gpu_time(W, H, h, ids, plates, settings, steps=5, warmup=2):
    """Milliseconds per step of the reference's own CUDA kernels (refgpu/ref_gpu_harness.cpp) on
    this GPU for the world (h, ids, plates) with `settings` (benchmark physics mapped onto the
    reference's parameters); raises RuntimeError when the cubin or the GPU is unavailable."""
    if not REF_CUBIN.exists():
        raise RuntimeError("the reference's device code was not built (oracle/_ref/ref_kernels.cubin is absent)")
    L = C.CDLL(str(REF_GPU_LIB))
    L.refgpu_error.restype = C.c_char_p
    L.refgpu_load.argtypes = [C.c_char_p]
    L.refgpu_time_steps.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                    C.c_float, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]
    if L.refgpu_load(str(REF_CUBIN).encode()) != 0:
        raise RuntimeError(L.refgpu_error().decode())
    ms = C.c_double()
    rc = L.refgpu_time_steps(W, H, _P(h), _P(ids), _P(plates), C.addressof(settings.kernel),
                             settings.step.hydraulicIterations, settings.step.hydraulicDt,
                             settings.step.thermalIterations, settings.sim.iterationsForCCL, steps, warmup,
                             C.byref(ms))
    if rc != 0:
        raise RuntimeError(L.refgpu_error().decode())
    return ms.value


def ref_gpu_relabel(ids, plate_sizes, settings, max_rounds=16):
    """The reference's own CCL relabel (refgpu/ref_relabel.cu: its CCL, createPlateIdLabelMap, the
    thrust ranking, getMaxSizeLabels, createLabelIdLookup, postCClIdReassign and the
    assignUnassignedIdsToNeighbor passes) on this GPU.  Returns (ids, labels, markers, rounds,
    unassigned): markers[k] is the plate whose record slot k holds afterwards."""
    if not REF_CUBIN.exists():
        raise RuntimeError("the reference's device code was not built (oracle/_ref/ref_kernels.cubin is absent)")
    L = C.CDLL(str(REF_GPU_LIB))
    L.refgpu_relabel_error.restype = C.c_char_p
    L.refgpu_relabel.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    out = np.ascontiguousarray(ids, np.uint8).copy()
    H, W = out.shape
    sizes = np.ascontiguousarray(plate_sizes, np.int32)
    assert sizes.shape == (255,)
    labels = np.zeros((H, W), np.uint32)
    markers = np.zeros(255, np.float32)
    rounds, left = C.c_int(), C.c_int()
    rc = L.refgpu_relabel(str(REF_CUBIN).encode(), W, H, _P(out), _P(sizes), C.addressof(settings.kernel),
                          _P(labels), _P(markers), max_rounds, C.byref(rounds), C.byref(left))
    if rc != 0:
        raise RuntimeError(L.refgpu_relabel_error().decode())
    return out, labels, markers, rounds.value, left.value


REF_EXPORT_CUBIN = HERE / "_ref" / "ref_export.cubin"


def _ref_export_lib():
    if not REF_EXPORT_CUBIN.exists():
        raise RuntimeError("the reference's export kernels were not built (oracle/_ref/ref_export.cubin is absent)")
    L = C.CDLL(str(REF_GPU_LIB))
    L.refgpu_error.restype = C.c_char_p
    L.refgpu_export_load.argtypes = [C.c_char_p]
    L.refgpu_gray16.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_void_p]
    L.refgpu_ids_rgb.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    if L.refgpu_export_load(str(REF_EXPORT_CUBIN).encode()) != 0:
        raise RuntimeError(L.refgpu_error().decode())
    return L


def ref_gpu_gray16(h, minv, maxv):
    """The reference's convertFloatToGray16Kernel run on this GPU: uint16[H, W]."""
    L = _ref_export_lib()
    h = np.ascontiguousarray(h, np.float32)
    out = np.empty(h.shape, np.uint16)
    if L.refgpu_gray16(h.ctypes.data, h.shape[1], h.shape[0], minv, maxv, out.ctypes.data) != 0:
        raise RuntimeError(L.refgpu_error().decode())
    return out


def ref_gpu_ids_rgb(ids):
    """The reference's convertGrayscaleToRgbKernel run on this GPU: uint8[H, W, 3]."""
    L = _ref_export_lib()
    ids = np.ascontiguousarray(ids, np.uint8)
    out = np.empty(ids.shape + (3,), np.uint8)
    if L.refgpu_ids_rgb(ids.ctypes.data, ids.shape[1], ids.shape[0], out.ctypes.data) != 0:
        raise RuntimeError(L.refgpu_error().decode())
    return out


def _P(a):
    return a.ctypes.data if a is not None else None


def lib() -> C.CDLL:
    global _o
    if _o is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        V = C.c_void_p
        L.or_plate_offsets.argtypes = [V, V, V, V]
        L.or_collision_words.argtypes = [C.c_int, C.c_int, V, V, V, V, V, V, V]
        L.or_collision_types.argtypes = [C.c_int, C.c_int, V, V, V, V, V, V]
        L.or_resolve.argtypes = [C.c_int, C.c_int, V, V, V, V, V, V, V, V, C.c_uint32, C.c_uint32, V, V, V]
        L.or_resolve_ex.argtypes = [C.c_int, C.c_int, V, V, V, V, V, V, V, V, C.c_uint32, C.c_uint32, V, V, V,
                                    V, V]
        L.or_uplift_ref.argtypes = [C.c_int, C.c_int, V, V, V, V, V, V, V, V, V, V]
        L.or_expf.argtypes = [C.c_float]
        L.or_expf.restype = C.c_float
        L.or_log10f.argtypes = [C.c_float]
        L.or_log10f.restype = C.c_float
        L.or_gray16.argtypes = [C.c_size_t, V, C.c_float, C.c_float, V]
        L.or_plate_palette.argtypes = [V]
        L.or_thermal.argtypes = [C.c_int, C.c_int, V, C.c_int, V]
        L.or_hydraulic.argtypes = [C.c_int, C.c_int, V, V, V, V, C.c_int, C.c_float, C.c_uint32, V]
        L.or_accretion.argtypes = [C.c_int, C.c_int, V, V, V, V]
        L.or_ccl.argtypes = [C.c_int, C.c_int, V, V, C.c_int]
        L.or_step.argtypes = [C.c_int, C.c_int, V, V, V, V, V, V, V, V, V, V, V, V, C.c_uint32, V]
        L.or_step_dyn.argtypes = [C.c_int, C.c_int, V, V, V, V, V, V, V, V, V, V, V, V, V, C.c_int, C.c_int, V,
                                  C.c_uint32, V]
        L.or_resolve_dyn.argtypes = [C.c_int, C.c_int, V, V, V, V, V, V, V, V, C.c_uint32, C.c_uint32, V, V, V,
                                     V, V, V, V, V]
        L.or_plate_stats.argtypes = [C.c_int, C.c_int, V, V, C.c_uint32, V]
        L.or_curl_at.argtypes = [V, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, V, V]
        L.or_plate_motion.argtypes = [C.c_int, C.c_int, V, V, V, V, C.c_int, C.c_int, V]
        L.or_reference_seeds.argtypes = [C.c_int, C.c_int, C.c_uint32, C.c_int, V, C.c_int, V, V, V, C.c_int, V, V, V]
        L.or_init_reference.argtypes = [C.c_int, C.c_int, C.c_uint32, V, V, V, C.c_int, V, V]
        L.or_relabel.argtypes = [C.c_int, C.c_int, V, V, V, V, C.c_int]
        L.or_merge.argtypes = [C.c_int, C.c_int, V, V, V, V, V]
        L.or_hash.argtypes = [C.c_uint32]
        L.or_hash.restype = C.c_uint32
        L.or_simplex3.argtypes = [C.c_float] * 4 + [C.c_int]
        L.or_simplex3.restype = C.c_float
        L.or_rain_noise.argtypes = [C.c_int, C.c_int, C.c_int]
        L.or_rain_noise.restype = C.c_float
        L.or_lerp.argtypes = [C.c_float] * 3
        L.or_lerp.restype = C.c_float
        L.or_sinf.argtypes = [C.c_float]
        L.or_sinf.restype = C.c_float
        L.or_gaussian_weights.argtypes = [C.c_float, C.c_int, V]
        L.or_settings_default.argtypes = [V]
        L.or_settings_baseline.argtypes = [V]
        L.or_generate_world.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_uint64, V, V, V]
        L.or_use_libm_sin.argtypes = [C.c_int]
        _o = L
    return _o


def use_libm_sin(on: bool) -> None:
    """Pinning mode: the oracle calls libm's sinf, as the reference's kernels do on the CPU."""
    lib().or_use_libm_sin(1 if on else 0)


def ref_available() -> bool:
    return REF_LIB.exists()


def ref() -> C.CDLL:
    """The reference's own kernels compiled for the CPU (only where oracle/Makefile `ref` ran)."""
    global _r
    if _r is None:
        L = C.CDLL(str(REF_LIB))
        V = C.c_void_p
        L.ref_set_settings.argtypes = [V]
        L.ref_pixel_movements.argtypes = [C.c_int, C.c_int, V, V, V]
        L.ref_register_collisions.argtypes = [C.c_int, C.c_int, V, V, V]
        L.ref_collision_types.argtypes = [C.c_int, C.c_int, V, V, V, V, V]
        L.ref_process_collisions.argtypes = [C.c_int, C.c_int, V, V, V, V, V, V, C.c_int, C.c_uint, V, V, V, V, V]
        L.ref_uplift.argtypes = [C.c_int, C.c_int, V, V, V, V, V, V, V, V, V]
        L.ref_thermal.argtypes = [C.c_int, C.c_int, V]
        L.ref_hydraulic.argtypes = [C.c_int, C.c_int, V, V, V, V, C.c_int, C.c_float, C.c_uint]
        L.ref_hydraulic.restype = C.c_int
        L.ref_accretion.argtypes = [C.c_int, C.c_int, V, V, V]
        L.ref_ccl.argtypes = [C.c_int, C.c_int, V, V]
        L.ref_gray16.argtypes = [C.c_int, C.c_int, V, C.c_float, C.c_float, V]
        L.ref_collision_friction.argtypes = [C.c_int, C.c_int, V, V, V, V, V, V, V, C.c_int, C.c_uint, V]
        L.ref_plate_centres.argtypes = [C.c_int, C.c_int, V, V]
        L.ref_curl.argtypes = [C.c_int, C.c_int, V, C.c_int, C.c_int, V]
        L.ref_plate_motion.argtypes = [C.c_int, C.c_int, V, V, V, V]
        L.ref_init.argtypes = [C.c_int, C.c_int, C.c_int, V, V, V, C.c_int, V, V]
        L.ref_merges.argtypes = [C.c_int, C.c_int, V, V, V, V, V]
        L.ref_ids_rgb.argtypes = [C.c_int, C.c_int, V, V]
        _r = L
    return _r


# ---- oracle phases on numpy arrays ---------------------------------------------------------

def plate_offsets(plates: np.ndarray):
    offx = np.zeros(255, np.int32)
    offy = np.zeros(255, np.int32)
    nxt = np.zeros_like(plates)
    lib().or_plate_offsets(_P(plates), _P(offx), _P(offy), _P(nxt))
    return offx, offy, nxt


def collision_words(ids: np.ndarray, offx, offy):
    H, W = ids.shape
    N = W * H
    dest = np.zeros(N, np.uint32)
    word = np.zeros(N, np.uint32)
    sk = np.zeros(N, np.uint32)
    sv = np.zeros(N, np.uint32)
    lib().or_collision_words(W, H, _P(ids), _P(offx), _P(offy), _P(dest), _P(word), _P(sk), _P(sv))
    return dest.reshape(H, W), word.reshape(H, W), sk, sv


def collision_types(word, h_old, offx, offy, settings, bitmap):
    H, W = word.shape
    bm = bitmap.copy()
    lib().or_collision_types(W, H, _P(word), _P(h_old), _P(offx), _P(offy), C.addressof(settings.kernel), _P(bm))
    return bm


def resolve(id_old, h_old, word, offx, offy, bitmap, div_bitmap, settings, seed, iteration):
    H, W = id_old.shape
    div = div_bitmap.copy()
    h_new = np.zeros_like(h_old)
    id_new = np.zeros_like(id_old)
    acc = np.zeros_like(id_old)
    lib().or_resolve(W, H, _P(id_old), _P(h_old), _P(word), _P(offx), _P(offy), _P(bitmap), _P(div),
                     C.addressof(settings), seed, iteration, _P(h_new), _P(id_new), _P(acc))
    return h_new, id_new, acc, div


def resolve_ex(id_old, h_old, word, offx, offy, bitmap, div_bitmap, settings, seed, iteration):
    """resolve() plus the processConvergence records (heightAddition, typeByte) of convergent cells."""
    H, W = id_old.shape
    div = div_bitmap.copy()
    h_new = np.zeros_like(h_old)
    id_new = np.zeros_like(id_old)
    acc = np.zeros_like(id_old)
    up_h = np.zeros((H, W), np.float32)
    up_t = np.zeros((H, W), np.uint8)
    lib().or_resolve_ex(W, H, _P(id_old), _P(h_old), _P(word), _P(offx), _P(offy), _P(bitmap), _P(div),
                        C.addressof(settings), seed, iteration, _P(h_new), _P(id_new), _P(acc), _P(up_h), _P(up_t))
    return h_new, id_new, acc, div, up_h, up_t


def uplift_ref(word, up_h, up_t, h_old, plates, id_new, h_new, settings):
    """The reference uplift on resolved heights: (heights, JFA nearest seed, JFA distance)."""
    H, W = h_old.shape
    out = h_new.copy()
    seed = np.zeros((H, W), np.int32)
    dist = np.zeros((H, W), np.int32)
    lib().or_uplift_ref(W, H, _P(word), _P(up_h), _P(up_t), _P(h_old), _P(plates), _P(id_new), _P(out),
                        C.addressof(settings.kernel), _P(seed), _P(dist))
    return out, seed, dist


def expf(x: float) -> float:
    return lib().or_expf(x)


def log10f(x: float) -> float:
    return lib().or_log10f(x)


def reference_seeds(W, H, seed, num_plates, gens):
    """or_reference_seeds: (x, y, id) of the seeds, plate records, plate dynamics records."""
    g = np.ascontiguousarray(gens, np.int32)
    cap = max([num_plates] + [int(v) for v in g])
    sx, sy = np.zeros(cap, np.float32), np.zeros(cap, np.float32)
    sid = np.zeros(cap, np.uint8)
    n = C.c_int(0)
    pl = np.zeros(MAX_PLATES, PLATE_DTYPE)
    dy = np.zeros(MAX_PLATES, PLATE_DYNAMICS_DTYPE)
    if lib().or_reference_seeds(W, H, seed, num_plates, _P(g), len(g), _P(sx), _P(sy), _P(sid), cap, C.byref(n),
                                _P(pl), _P(dy)) != 0:
        raise ValueError("invalid reference seed settings")
    k = n.value
    return sx[:k].copy(), sy[:k].copy(), sid[:k].copy(), pl, dy


def init_reference(W, H, seed, sx, sy, sid):
    """or_init_reference: (heights f32[H, W], plate ids u8[H, W])."""
    h = np.zeros((H, W), np.float32)
    ids = np.zeros((H, W), np.uint8)
    sx, sy, sid = (np.ascontiguousarray(a, t) for a, t in ((sx, np.float32), (sy, np.float32), (sid, np.uint8)))
    lib().or_init_reference(W, H, seed, _P(sx), _P(sy), _P(sid), len(sx), _P(h), _P(ids))
    return h, ids


def relabel(ids, labels, plates, dyn, min_plate_size):
    """or_relabel on copies: (ids, plates, dyn, cells left without an id)."""
    i, pl, dy = np.ascontiguousarray(ids, np.uint8).copy(), plates.copy(), dyn.copy()
    lab = np.ascontiguousarray(labels, np.uint32)
    H, W = i.shape
    left = lib().or_relabel(W, H, _P(i), _P(lab), _P(pl), _P(dy), min_plate_size)
    return i, pl, dy, left


def merge(ids, plates, dyn, bitmap, settings):
    """or_merge on copies: (ids, bitmap, merges)."""
    i, bm = np.ascontiguousarray(ids, np.uint8).copy(), np.ascontiguousarray(bitmap, np.uint8).copy()
    H, W = i.shape
    n = lib().or_merge(W, H, _P(i), _P(plates), _P(dyn), _P(bm), C.addressof(settings.kernel))
    return i, bm, n


def plate_stats(h, ids, iteration, dyn=None):
    """or_plate_stats: mass, size and geometric centre per plate (updates a copy of dyn)."""
    H, W = h.shape
    out = np.zeros(MAX_PLATES, PLATE_DYNAMICS_DTYPE) if dyn is None else dyn.copy()
    lib().or_plate_stats(W, H, _P(np.ascontiguousarray(h, np.float32)), _P(np.ascontiguousarray(ids, np.uint8)),
                         iteration, _P(out))
    return out


def curl_at(pressure, W, H, cx, cy):
    pr = np.ascontiguousarray(pressure, np.float32)
    ox, oy = C.c_float(), C.c_float()
    lib().or_curl_at(_P(pr), pr.shape[1], pr.shape[0], W, H, cx, cy, C.byref(ox), C.byref(oy))
    return ox.value, oy.value


def plate_motion(W, H, plates, dyn, fric, pressure, settings):
    """or_plate_motion on copies: returns (plates, dyn)."""
    pl, dd = plates.copy(), dyn.copy()
    fr = np.ascontiguousarray(fric, np.int64)
    pr = None if pressure is None else np.ascontiguousarray(pressure, np.float32)
    pw, ph = (pr.shape[1], pr.shape[0]) if pr is not None else (0, 0)
    lib().or_plate_motion(W, H, _P(pl), _P(dd), _P(fr), _P(pr), pw, ph, C.addressof(settings.kernel))
    return pl, dd


def gray16(h, minv, maxv):
    """convertFloatToGray16Kernel (texture_save.cu:80-96) on the CPU."""
    h = np.ascontiguousarray(h, np.float32)
    out = np.empty(h.shape, np.uint16)
    lib().or_gray16(h.size, h.ctypes.data, minv, maxv, out.ctypes.data)
    return out


def plate_palette():
    """convertGrayscaleToRgbKernel's colour of each plate id (texture_save.cu:16-70): uint8[256, 3]."""
    out = np.empty((256, 3), np.uint8)
    lib().or_plate_palette(out.ctypes.data)
    return out


def thermal(h, iters, settings):
    H, W = h.shape
    out = h.copy()
    lib().or_thermal(W, H, _P(out), iters, C.addressof(settings.kernel))
    return out


def hydraulic(h, w, s, flux, iters, dt, rain_seed, settings):
    H, W = h.shape
    h, w, s, flux = h.copy(), w.copy(), s.copy(), flux.copy()
    lib().or_hydraulic(W, H, _P(h), _P(w), _P(s), _P(flux), iters, dt, rain_seed, C.addressof(settings.kernel))
    return h, w, s, flux


def accretion(h, acc, ids, settings):
    H, W = h.shape
    out = ids.copy()
    lib().or_accretion(W, H, _P(h), _P(acc), _P(out), C.addressof(settings.kernel))
    return out


def ccl(ids, mode):
    H, W = ids.shape
    labels = np.zeros((H, W), np.uint32)
    lib().or_ccl(W, H, _P(ids), _P(labels), mode)
    return labels


class OracleWorld:
    """A full world state stepped by or_step."""

    def __init__(self, settings, h, ids, plates, seed, w=None, s=None, flux=None):
        H, W = h.shape
        self.W, self.H = W, H
        self.settings = settings
        self.h = h.astype(np.float32).copy()
        self.id = ids.astype(np.uint8).copy()
        self.w = np.zeros((H, W), np.float32) if w is None else w.copy()
        self.s = np.zeros((H, W), np.float32) if s is None else s.copy()
        self.flux = np.zeros((H, W, 4), np.float32) if flux is None else flux.copy()
        self.labels = np.zeros((H, W), np.uint32)
        self.word = np.zeros((H, W), np.uint32)
        self.acc = np.zeros((H, W), np.uint8)
        self.bitmap = np.zeros(32385, np.uint8)
        self.div = np.zeros(1013, np.uint32)
        self.plates = plates.copy()
        self.seed = seed
        self.iteration = C.c_uint32(0)

        self.dyn = np.zeros(MAX_PLATES, PLATE_DYNAMICS_DTYPE)
        self.pressure = None

    def step(self, n: int = 1) -> None:
        pr = self.pressure
        pw, ph = (pr.shape[1], pr.shape[0]) if pr is not None else (0, 0)
        for _ in range(n):
            lib().or_step_dyn(self.W, self.H, _P(self.h), _P(self.w), _P(self.s), _P(self.flux), _P(self.id),
                              _P(self.labels), _P(self.word), _P(self.acc), _P(self.bitmap), _P(self.div),
                              _P(self.plates), _P(self.dyn), _P(pr), pw, ph, C.addressof(self.settings),
                              self.seed, C.byref(self.iteration))
