/*
 * tecto.h - C ABI of the GB300 (sm_103a) engine for the plate-tectonics simulation step.
 *
 * This is the only boundary between callers and the engine: plain C types, plain pointers
 * and sizes, explicit CUDA streams (passed as opaque pointers), integer status codes.
 * Nothing here exits the process; every call returns TECTO_OK (0) or a negative code.
 *
 * Each entry point names the reference interface it replaces (MarWo22/master_thesis,
 * paths relative to the project root).
 *
 * Threading: one world per handle.  Calls on different worlds may run concurrently from
 * different host threads; calls on the same world must be serialised by the caller.
 * Device work is enqueued on the stream given; a NULL stream means the legacy default stream.
 */
#ifndef TECTO_H
#define TECTO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TECTO_MAX_PLATES 255          /* MAX_PLATE_COUNT, src/cuda_compute/plate_tectonics_kernel.cuh:13 */
#define TECTO_NUM_PAIRS 32385         /* 255*254/2, NUM_TRIANGLE_ENTRIES, plate_tectonic_sim.h:25 */
#define TECTO_NUM_DIV_WORDS 1013      /* NUM_WORDS_TRIANGLE_SINGLE_BITS, plate_tectonic_sim.h:30 */
#define TECTO_MAX_VORONOI_GENS 8

/* ---- status codes ------------------------------------------------------------------ */
#define TECTO_OK 0
#define TECTO_ERR_INVALID (-1)        /* bad argument (null handle, size out of range, ...) */
#define TECTO_ERR_CUDA (-2)           /* a CUDA runtime call failed; see tecto_last_error_string */
#define TECTO_ERR_OOM (-3)            /* device allocation failed */
#define TECTO_ERR_DEVICE_TIMEOUT (-4) /* a bounded device-side wait gave up (error flag set) */
#define TECTO_ERR_UNSUPPORTED (-5)    /* configuration the engine does not implement */
#define TECTO_ERR_BUDGET (-6)         /* admission refused: memory budget exhausted */
#define TECTO_ERR_NOT_FOUND (-7)      /* lookup found no entry (autotuner cache) */

typedef struct CUstream_st *tecto_stream_t; /* same type as cudaStream_t */
typedef struct tecto_world tecto_world;

/* ---- settings ---------------------------------------------------------------------- */

/* Field-for-field mirror of KernelSettings (src/cuda_compute/kernel_settings.cuh:4-81): same
 * names, same order, same 4-byte types, so a KernelSettings object can be copied in bytewise.
 * Defaults come from tecto_settings_default(). */
typedef struct tecto_kernel_settings {
    float inelasticCollisionMultiplierContinental;
    float inelasticCollisionMultiplierSubduction;
    float inelasticCollisionMultiplierAccretion;
    float frictionCoefficientContinental;
    float frictionCoefficientSubduction;
    float frictionCoefficientAccretion;
    float environmentalDragCoefficient;
    float velocitySmoothingFactor;
    float directionSmoothingFactor;
    float breakScoreSmoothingFactor;
    float mergeDotDirectionThreshold;
    float mergeVelocityDiffThreshold;
    float mergeMinVelocity;
    int mergeWaitAfterSplit;
    int minPlateSize;
    float continentalCrustThreshold;
    float divergence_height_target_min;
    float divergence_height_target_max;
    float divergence_interpolation_factor;
    int collisionTypeUpdateCooldown;
    int minCollisionSize;
    float subductionOverUpliftMultiplier;
    float subductionUnderUpliftMultiplier;
    float continentalUpliftMultiplier;
    float minUpliftClamp;
    float maxUpliftClamp;
    int upliftRange;
    int subductionOverRange;
    int continentalPropMaxIters;
    float continentalPropThreshold;
    float hydrationPipeCrossSection;
    float hydrationPipeLength;
    float hydrationRainfall;
    float hydrationEvaporation;
    float gravity;
    float sedimentCapacity;
    float sedimentErosionRate;
    float sedimentDepositionRate;
    float pressureAccumulation;
    float pressureDecayRate;
    int pressureBlurRange;
    float pressureMultiplier;
    float curlNoiseMultiplier;
    float stressSplitThreshold;
    int targetMinimumPlateArea;
    int targetMaximumPlateArea;
    float thermalErosionStrength;
    float thermalErosionAmplitude;
    float thermalCellSize;
    float thermalThresholdAngle;
} tecto_kernel_settings;

/* SimulationSettings (src/generation_settings.h:67-76); the std::vector of Voronoi generation
 * sizes becomes a fixed array plus a count. */
typedef struct tecto_simulation_settings {
    int numStartingPlates;
    uint32_t seed;
    int numVoronoiSeeds[TECTO_MAX_VORONOI_GENS];
    int numVoronoiGenerations;
    int iterationsForCCL;
} tecto_simulation_settings;

/* Uplift modes. */
#define TECTO_UPLIFT_GAUSSIAN 0  /* +upliftAmount on convergent cells, separable Gaussian blur */
#define TECTO_UPLIFT_NONE 1      /* no uplift phase */
#define TECTO_UPLIFT_REFERENCE 2 /* the reference's uplift: continental collisions propagated against the
                                    plate motion, a jump-flooding distance field to the nearest
                                    collision, distance profiles applied (plate_tectonic_sim.cu:270-317) */

/* CCL connectivity modes. */
#define TECTO_CCL_4 4
#define TECTO_CCL_8 8
#define TECTO_CCL_REF8 9 /* the union set the reference's kernels build (src/cuda_compute/ccl.cu:
                            90-177): init's link to the first equal of (tl, t, tr, l), then l and tl
                            unions on every row and t and tr unions on row 0 */

/* Knobs the reference hard-codes (plate_tectonic_sim.cu:73, :336-363) or does not have. */
typedef struct tecto_step_settings {
    int hydraulicIterations;  /* reference: 10 (literal loop bound, plate_tectonic_sim.cu:336) */
    float hydraulicDt;        /* reference: 1.0 (literal, plate_tectonic_sim.cu:338-363) */
    int thermalIterations;    /* reference: 1 (single launch, plate_tectonic_sim.cu:73) */
    int upliftMode;           /* TECTO_UPLIFT_* */
    float upliftAmount;       /* added on convergent cells before the blur */
    float upliftSigma;        /* Gaussian sigma in cells */
    int upliftRadius;         /* taps on each side (<= 8) */
    int cclConnectivity;      /* TECTO_CCL_* */
    int sortRadixBits;        /* collision sort digit width 8..11; 0 = autotuner's choice, else 8 */
    int hydraulicTile;        /* 0 = autotuner's choice, else 4; 1: 64x16/256 threads, 2: 64x32/256,
                                 3: 64x32/512, 4: 64x32/1024, 5: 64x64/1024, 6: 64x16/512 (3 blocks
                                 per SM), 7: 64x16/384 (4 blocks per SM), 8: column strips of 56
                                 cells marched down by one warp each, no block barriers, 9: column
                                 strips of 120 cells marched down 8 rows at a time by a block of 512
                                 threads, rows kept in shared memory (8 and 9: the split path,
                                 50 dt >= 1.5, runs variant 4) */
    int thermalTile;          /* 0 = autotuner's choice, else 4; 1: 64x32 tiles / 1024 threads, up to 5
                                 iterations per launch; 2: 64x16 / 512, 2 blocks per SM, up to 4;
                                 3: 64x16 / 768, 2 blocks per SM, up to 3; 4: 64x16 / 512, 3 blocks
                                 per SM, up to 2; 5: column strips of up to 124 cells marched down
                                 8 rows at a time by a block of 512 threads, one iteration per launch */
    int plateDynamics;        /* TECTO_PLATE_DYNAMICS_*: 0 fixed plate velocities (the benchmark), 1 the
                                 reference's applyPlateMovementChanges after every step */
    int platePolicy;          /* TECTO_PLATE_RELABEL | TECTO_PLATE_MERGE bits, 0 = neither */
    int reserved[3];
} tecto_step_settings;

/* Plate policy after a step (bits of platePolicy). */
#define TECTO_PLATE_RELABEL 1 /* after each CCL: fragments of a plate other than its largest take free
                                 plate ids or their neighbours' (applyCCL, plate_tectonic_sim.cu:391-467) */
#define TECTO_PLATE_MERGE 2   /* after every step: touching plates that move alike merge (mergePlates,
                                 plate_tectonic_sim.cu:470-494) */

/* Plate dynamics modes. */
#define TECTO_PLATE_DYNAMICS_OFF 0
#define TECTO_PLATE_DYNAMICS_REFERENCE 1 /* collision friction, asthenosphere drag and smoothing
                                            (plate_tectonics_kernel.cu:1863-1925), see
                                            tecto_plate_dynamics */

typedef struct tecto_settings {
    tecto_kernel_settings kernel;
    tecto_simulation_settings sim;
    tecto_step_settings step;
} tecto_settings;

/* Reference defaults: KernelSettings initialisers (kernel_settings.cuh:6-71), SimulationSettings
 * initialisers (generation_settings.h:69-72), and the reference's literal step constants. */
int tecto_settings_default(tecto_settings *out);

/* The synthetic benchmark parameterisation: rain 0.01, evaporation 0.05, Kc 0.1, Ks 0.3, Kd 0.1,
 * dt 0.02, 20 hydraulic and 10 thermal iterations, talus 0.01, rate 0.5, Gaussian uplift 0.01 with
 * sigma 1.5 radius 3, continental threshold 0, 4-connected CCL every 10 steps.  Everything else
 * keeps the reference default. */
int tecto_settings_baseline(tecto_settings *out);

/* Parse a config.json (src/config.h:23-33 keys "heightmap_dimensions" {x,y} and "use_renderer",
 * plus optional "kernel_settings", "simulation_settings" and "step_settings" objects whose keys are
 * the field names above) on top of *inout.  width/height receive heightmap_dimensions when present
 * (may be NULL). */
int tecto_settings_from_json(const char *json_text, tecto_settings *inout, int *width, int *height);

/* ---- per-plate kinematics ---------------------------------------------------------- */

/* The hot-path subset of PlateData (src/cuda_compute/types/plate_data.h:5-38). */
typedef struct tecto_plate {
    float velocity;      /* PlateData::velocity (cells per step) */
    float direction_x;   /* PlateData::direction */
    float direction_y;
    float pixelCenter_x; /* PlateData::pixelCenter, sub-cell position in [0,1) */
    float pixelCenter_y;
} tecto_plate;

/* The rest of a plate's PlateData (types/plate_data.h) that plate dynamics reads and writes.
 * With TECTO_PLATE_DYNAMICS_REFERENCE each step
 *  - first recomputes mass, size and the geometric centre from the current cells (the values
 *    mergePlates and calculatePlateCenters leave at the end of the reference's previous iteration,
 *    plate_tectonic_sim.cu:95-111; mass and centre sums are accumulated in 64-bit fixed point so
 *    that every run gives the same bits); the first iteration keeps the stored centre, as the
 *    reference computes no centre before its first iteration ends;
 *  - accumulates each plate's collision friction in the resolve (applyElasticVelocityChange,
 *    plate_tectonics_kernel.cu:371-394: velocity x coefficient x source height / plate mass per
 *    arrival at a convergent cell);
 *  - then applies applyPlateMovementChanges: friction loss, drag towards the asthenosphere flow
 *    sampled at the geometric centre, smoothing, merge wait countdown. */
typedef struct tecto_plate_dynamics {
    float velocitySmoothed;
    float directionSmoothed_x, directionSmoothed_y;
    float geometricCenter_x, geometricCenter_y;
    float mass;          /* sum of the plate's cell heights */
    int size;            /* cells */
    int mergeWaitTime;
    float frictionLoss;  /* CollisionVelocityChanges::frictionLoss of the last step (read only) */
} tecto_plate_dynamics;

/* ---- fields ------------------------------------------------------------------------ */
#define TECTO_FIELD_HEIGHT 0       /* f32[W*H]  m_heightMapTexture */
#define TECTO_FIELD_WATER 1        /* f32[W*H]  m_hydrationLevel */
#define TECTO_FIELD_SEDIMENT 2     /* f32[W*H]  m_sedimentLevel */
#define TECTO_FIELD_FLUX 3         /* f32x4[W*H] m_hydrationFlux (left, +y, right, -y) */
#define TECTO_FIELD_PLATE_ID 4     /* u8[W*H]   m_plateIdsTexture */
#define TECTO_FIELD_LABELS 5       /* u32[W*H]  CCL labels (minimum linear index per component) */
#define TECTO_FIELD_COLLISION 6    /* u32[W*H]  packed arrival word of the last step (m_plateCollisions) */
#define TECTO_FIELD_TYPE_BITMAP 7  /* u8[32385] m_collisionTypeBitmap */
#define TECTO_FIELD_DIV_BITMAP 8   /* u32[1013] m_divergenceBitmap */
#define TECTO_FIELD_SORT_KEYS 9    /* u32[W*H]  destination cells of the last step, sorted */
#define TECTO_FIELD_SORT_VALS 10   /* u32[W*H]  source cells, in the same order */
#define TECTO_FIELD_ACCRETION 11   /* u8[W*H]   accretion marks of the last resolve (0 = none) */
#define TECTO_FIELD_JFA_SEED 12    /* i32[W*H]  reference uplift of the last step: nearest propagated
                                      collision cell (JFA seed), -1 none (read only) */
#define TECTO_FIELD_JFA_DIST 13    /* i32[W*H]  its distance in whole cells (JFAComputeDistance), -1 none */
#define TECTO_FIELD_COUNT 14

/* ---- world lifecycle (replaces PlateTectonicSim, plate_tectonic_sim.h:110-130) ------ */

/* PlateTectonicSim::PlateTectonicSim(width, height, seed, interop) + initializeTextures()
 * (plate_tectonic_sim.cu:28-36, :844-872): allocates the world's device state (zeroed) on the
 * current device and uploads settings (the reference never uploads them headless).  Also loads
 * the reference's seed convention: the step's noise seed is seed + iteration. */
int tecto_world_create(const tecto_settings *settings, int width, int height, uint32_t seed,
                       tecto_world **out);
int tecto_world_destroy(tecto_world *world);

/* Replace the settings of a live world (Gui::simulationSettingsSection ->
 * copyHostKernelSettingsToDevice, kernel_settings.cu:7-9, gui.cpp:435-441). */
int tecto_world_set_settings(tecto_world *world, const tecto_settings *settings);
int tecto_world_get_settings(const tecto_world *world, tecto_settings *out);
int tecto_world_size(const tecto_world *world, int *width, int *height);

/* Synthetic world generator (host-only, needs no GPU): numPlates plates from a toroidal Voronoi
 * of numPlates uniform seed points, per-plate velocity vector uniform in [-velRange, velRange]^2,
 * half the plates continental (0.5 + N(0, 0.05)) and half oceanic (-0.5 + N(0, 0.02)), water,
 * sediment and flux zero.  Deterministic in genSeed on every platform.  Any output may be NULL. */
int tecto_generate_world_host(int width, int height, int numPlates, float velRange, uint64_t genSeed,
                              float *height_out, uint8_t *plate_id_out, tecto_plate *plates_out);

/* PlateTectonicSim::initialize (plate_tectonic_sim.cu:40-51) for the synthetic generator above:
 * generates on the host, uploads, resets water/sediment/flux/bitmaps and the iteration count. */
int tecto_world_init_synthetic(tecto_world *world, int numPlates, float velRange, uint64_t genSeed,
                               tecto_stream_t stream);

/* Host <-> device copies of one field (synchronous w.r.t. the stream: the call returns after
 * the copy completed).  bytes must equal the field's size. */
int tecto_world_upload(tecto_world *world, int field, const void *host, size_t bytes,
                       tecto_stream_t stream);
int tecto_world_download(tecto_world *world, int field, void *host, size_t bytes,
                         tecto_stream_t stream);
/* The same copies ordered on the stream without waiting for them: the host buffer (pinned for
 * asynchrony) must stay valid, and a download's unread, until the stream reaches the copy. */
int tecto_world_upload_async(tecto_world *world, int field, const void *host, size_t bytes,
                             tecto_stream_t stream);
int tecto_world_download_async(tecto_world *world, int field, void *host, size_t bytes, tecto_stream_t stream);
/* Borrow the device pointer of a field (valid until the next call that steps the world). */
int tecto_world_field(tecto_world *world, int field, void **device_ptr, size_t *bytes);

int tecto_world_set_plates(tecto_world *world, const tecto_plate *plates, int count,
                           tecto_stream_t stream);
int tecto_world_get_plates(tecto_world *world, tecto_plate *plates, int count,
                           tecto_stream_t stream);
int tecto_world_set_plate_dynamics(tecto_world *world, const tecto_plate_dynamics *plates, int count,
                                   tecto_stream_t stream);
int tecto_world_get_plate_dynamics(tecto_world *world, tecto_plate_dynamics *plates, int count,
                                   tecto_stream_t stream);
/* The asthenosphere pressure texture (host floats, pw x ph, any size; the reference loads
 * assets/textures/noise.png as grey / 255, plate_tectonic_sim.cu:866-869).  Plate dynamics samples
 * its curl (computeCurl, plate_tectonics_kernel.cu:2788-2822, nearest-scaled to the world) at each
 * plate's geometric centre.  NULL removes it: the curl is then zero everywhere. */
int tecto_world_set_asthenosphere(tecto_world *world, const float *pressure, int pw, int ph,
                                  tecto_stream_t stream);
int tecto_world_set_iteration(tecto_world *world, uint32_t iteration);
int tecto_world_get_iteration(const tecto_world *world, uint32_t *iteration);

/* ---- stepping ---------------------------------------------------------------------- */

/* PlateTectonicSim::executeIteration (plate_tectonic_sim.cu:54-131), hot-path phases only:
 * plate offsets, advection + radix sort + segmented winner pick, collision typing, resolve,
 * uplift, thermal, hydraulic, accretion, CCL every iterationsForCCL steps, plate sub-cell
 * centre update.  Asynchronous on `stream`; nSteps steps are enqueued (as a CUDA graph once
 * warm). */
int tecto_world_step(tecto_world *world, int nSteps, tecto_stream_t stream);

/* Phase entry points (each a subset of executeIteration, for parity tests and custom drivers).
 * Calling them in the order below is equivalent to one tecto_world_step. */

/* getPlateCollisions (plate_tectonic_sim.cu:174-208) + determineCollisionType kernel and
 * createCollisionTypeMatrix (:232-241): plate offsets, advection, sort on destination, collision
 * words, collision-type evidence and the pair bitmap update. */
int tecto_phase_collide(tecto_world *world, tecto_stream_t stream);
/* processCollisions + flipDivergedBitmap (:246-262) and the uplift phase of upliftMode. */
int tecto_phase_resolve(tecto_world *world, tecto_stream_t stream);
/* thermalErosionKernel (:73), `iterations` deterministic gather iterations. */
int tecto_phase_thermal(tecto_world *world, int iterations, tecto_stream_t stream);
/* applyHydraulicErosion (:331-373) with `iterations` sub-iterations of step dt. */
int tecto_phase_hydraulic(tecto_world *world, int iterations, float dt, tecto_stream_t stream);
/* applyAccretion (:90-93) and the plate sub-cell centre update of applyPlateMovementChanges
 * (plate_tectonics_kernel.cu:1871-1878); advances the iteration counter. */
int tecto_phase_finish(tecto_world *world, tecto_stream_t stream);
/* applyCCL's labelling part (plate_tectonic_sim.cu:375-389): labels of equal-plate components
 * on the torus, each the minimum linear index of its component. */
int tecto_phase_ccl(tecto_world *world, int connectivity, tecto_stream_t stream);

/* Standalone stable LSD radix sort of (u32 key, u32 value) pairs on the device: the sort that
 * replaces registerPlateCollisions' atomic slotting (plate_tectonics_kernel.cu:273-298).
 * Keys must be < 2^key_bits.  scratch must hold tecto_sort_scratch_bytes(n, key_bits) bytes.
 * Result in keys_out/vals_out; inputs are not modified. */
size_t tecto_sort_scratch_bytes(size_t n, int key_bits);
int tecto_sort_pairs(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_out,
                     uint32_t *vals_out, size_t n, int key_bits, void *scratch,
                     size_t scratch_bytes, tecto_stream_t stream);

/* The same sort with the digit width chosen by the caller: radix_bits 8..11 (0 = 8), the widths
 * the collision sort's autotuner picks from (tecto_step_settings::sortRadixBits).  Scratch must
 * hold tecto_sort_scratch_bytes_radix(n, key_bits, radix_bits) bytes; other widths are
 * TECTO_ERR_INVALID (and 0 scratch bytes). */
size_t tecto_sort_scratch_bytes_radix(size_t n, int key_bits, int radix_bits);
int tecto_sort_pairs_radix(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_out,
                           uint32_t *vals_out, size_t n, int key_bits, int radix_bits, void *scratch,
                           size_t scratch_bytes, tecto_stream_t stream);
/* 1 when a sort of n pairs runs its passes in the form for large sorts (from 4096 tiles of 4096
 * keys, i.e. 16 777 216 pairs: three blocks per SM), 0 when it runs the form for smaller sorts.
 * The collision sort of a batch or world uses the same rule on its cell count. */
int tecto_sort_wide_pass(size_t n);

/* The same stable sort for callers that cannot allocate device memory: it needs no scratch
 * argument and makes no allocation of any kind (no cudaMalloc, cudaFree or allocating library
 * call).  This entry point has no counterpart in the reference.  Who needs it: a host that hands
 * the engine a fixed memory budget and owns every allocation (a plugin inside a renderer or game
 * engine), and a per-frame loop such as the reference's GUI loop, where cudaFree's implicit device
 * synchronisation would stall the frame.
 *
 * Its scratch is one fixed array in device memory, TECTO_SORT_NOALLOC_MAX_PAIRS pairs large
 * (9.4 MB), which every GPU that loads the library holds until the process exits.  Limits
 * and rules:
 *  - n > TECTO_SORT_NOALLOC_MAX_PAIRS is rejected with TECTO_ERR_INVALID (nothing runs);
 *  - outputs must not alias the inputs (TECTO_ERR_INVALID);
 *  - the first call on each device resolves the array's device address with that device current
 *    and keeps it for the life of that device's context; make that first call before any stream
 *    capture begins, and do not reset the device (cudaDeviceReset) while the library is in use;
 *  - all calls share the one array: two calls whose work overlaps on the GPU (different streams,
 *    or different host threads on the same device) race and corrupt each other's results, so
 *    serialise them.  Each call clears the parts that must start at zero itself.
 * Every call is synchronous: it reads the sort's error word back to the host and waits for the
 * stream, so it returns only after the result is in keys_out/vals_out. */
#define TECTO_SORT_NOALLOC_MAX_PAIRS ((size_t)1 << 20)
int tecto_sort_pairs_noalloc(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_out,
                             uint32_t *vals_out, size_t n, int key_bits, tecto_stream_t stream);

/* ---- batches: many worlds, one launch per phase ----------------------------------------
 *
 * The reference steps one world at a time; it has no counterpart for these calls.  A batch
 * advances all its worlds together: every phase is one kernel launch over a work list of
 * (world, tile) items, the sort runs once over all the batch's cells, and a step is replayed as
 * one CUDA graph.  Worlds keep their own device state and keep it between steps; results are
 * identical to stepping each world alone.  All worlds of a batch share one device and the settings
 * a step reads (kernel and step settings, the CCL period); the initialisation-only fields of
 * SimulationSettings (plate count, seed, Voronoi generations) may differ.  While a world is in a
 * batch, tecto_world_step and the phase calls refuse it. */
typedef struct tecto_batch tecto_batch;
int tecto_batch_create(tecto_batch **out);
int tecto_batch_destroy(tecto_batch *batch);  /* worlds stay alive and leave the batch */
int tecto_batch_add(tecto_batch *batch, tecto_world *world, tecto_stream_t stream);
int tecto_batch_remove(tecto_batch *batch, tecto_world *world);
int tecto_batch_step(tecto_batch *batch, int nSteps, tecto_stream_t stream);
int tecto_batch_size(const tecto_batch *batch, int *worlds, size_t *cells);
int tecto_batch_launch_count(const tecto_batch *batch, uint64_t *count);
int tecto_batch_check(tecto_batch *batch, tecto_stream_t stream);
/* One field of every member world to or from one packed host buffer, stream-ordered like
 * tecto_world_upload_async: member order (the order of tecto_batch_add, removed worlds taken out),
 * each world's W*H elements, bytes = the batch's cells x the element size (fields HEIGHT, WATER,
 * SEDIMENT, FLUX, PLATE_ID, LABELS).  One host<->device copy through a staging buffer the batch
 * keeps, and one device scatter or gather, instead of one copy per world. */
int tecto_batch_upload_async(tecto_batch *batch, int field, const void *host, size_t bytes, tecto_stream_t stream);
int tecto_batch_download_async(tecto_batch *batch, int field, void *host, size_t bytes, tecto_stream_t stream);
/* The same split in two so that copies overlap compute: stage_upload copies a packed field into a
 * staging buffer of the batch on copy_stream, commit_upload scatters it into the worlds on the
 * compute stream (after the copy); gather_download collects a field on the compute stream,
 * fetch_download copies it to the host on copy_stream (after the gather).  Each field has two
 * staging buffers in each direction, used in turn, so a stage may run up to two commits ahead (the
 * copy for step k+2 overlaps step k+1 and part of step k) and a gather up to two fetches ahead;
 * one more is TECTO_ERR_INVALID, and so is a commit with nothing staged or a fetch with nothing
 * gathered.  Events inside the batch order the streams: a stage waits for the commit that last read
 * its buffer, a gather for the fetch that last read its buffer.  Uploads and downloads may use
 * different copy streams (separate copy engines).  The host buffers must stay valid until the copy
 * stream has passed the copy. */
int tecto_batch_stage_upload_async(tecto_batch *batch, int field, const void *host, size_t bytes,
                                   tecto_stream_t copy_stream);
int tecto_batch_commit_upload(tecto_batch *batch, int field, tecto_stream_t stream);
int tecto_batch_gather_download(tecto_batch *batch, int field, tecto_stream_t stream);
int tecto_batch_fetch_download_async(tecto_batch *batch, int field, void *host, size_t bytes,
                                     tecto_stream_t copy_stream);
/* The first cell of each member in that packing, and the total (capacity >= worlds + 1). */
int tecto_batch_offsets(const tecto_batch *batch, size_t *cell_offsets, int capacity);
/* Phases over every world of the batch (one launch per sub-iteration): for measurement and
 * parity tests, like the per-world phase calls above. */
int tecto_batch_phase_hydraulic(tecto_batch *batch, int iterations, float dt, tecto_stream_t stream);
int tecto_batch_phase_thermal(tecto_batch *batch, int iterations, tecto_stream_t stream);

/* ---- autotuner ---------------------------------------------------------------------------
 *
 * No counterpart in the reference (fixed launch shapes, plate_tectonic_sim.cu).  Times every
 * hydraulic tile variant (one sub-iteration), every thermal tile variant (ten iterations) and every
 * sort digit width (the collision sort) on scratch worlds of the given shapes with synthetic
 * content, and returns the fastest of each.
 * The caller's worlds are not touched.  The choice is cached per device and batch shape class
 * (total cells and mean world cells, half-octave classes); batches whose settings leave
 * hydraulicTile / thermalTile / sortRadixBits at 0 use the choice cached for their class, else for
 * the nearest tuned class on their device, else the defaults (hydraulic variant 4, thermal
 * variant 4, 8-bit digits). */
typedef struct tecto_tuning {
    int hydraulicTile;       /* chosen variant, 1..9 */
    int sortRadixBits;       /* chosen digit width, 8..11 */
    int thermalTile;         /* chosen variant, 1..5 */
    float hydraulic_ms[9];   /* one hydraulic sub-iteration with variant 1..9 */
    float sort_ms[4];        /* the collision sort with 8..11-bit digits */
    float thermal_ms[5];     /* ten thermal iterations with variant 1..5 */
} tecto_tuning;
int tecto_autotune(const tecto_settings *settings, const int *widths, const int *heights, int count,
                   tecto_stream_t stream, tecto_tuning *out);
/* Tune for the batch's current member shapes and apply the choice to this batch. */
int tecto_batch_autotune(tecto_batch *batch, tecto_stream_t stream, tecto_tuning *out);
/* Tune for one world's shape and apply the choice to its plain stepping. */
int tecto_world_autotune(tecto_world *world, tecto_stream_t stream, tecto_tuning *out);
/* Cache access (no device work): record a choice for a class, look one up, clear the cache. */
int tecto_autotune_record(int device, size_t total_cells, int worlds, int hydraulicTile, int sortRadixBits,
                          int thermalTile);
int tecto_autotune_lookup(int device, size_t total_cells, int worlds, int *hydraulicTile, int *sortRadixBits,
                          int *thermalTile);
int tecto_autotune_clear(void);

/* Device bytes one world of width x height holds, including its share of batch buffers: the
 * admission cost used by the server below. */
size_t tecto_world_bytes(int width, int height);

/* ---- serving: continuous batching of world-generation requests -------------------------
 *
 * No counterpart in the reference (it runs one interactive world).  A request asks for a world of
 * width x height with `plates` plates (synthetic generator, seeds gen_seed / world_seed) to be
 * advanced `steps` steps.  The server keeps every admitted world resident in HBM, advances all of
 * them one step per tick as one batch, admits waiting requests first-come first-served whenever
 * their tecto_world_bytes fit the budget (and fewer than max_worlds are active), and retires
 * finished worlds at once, so new requests join while others are mid-flight.  A request larger
 * than the whole budget is rejected (TECTO_ERR_BUDGET).  Heavy requests (tecto_server_set_policy;
 * by default worlds of 2^20 cells or more, which already run near the GPU's full rate alone) are
 * live at most one at a time, first-come first-served among themselves; light requests join past
 * a heavy one that waits for its slot, but never past one that waits for budget. */
typedef struct tecto_server tecto_server;
typedef struct tecto_request {
    int width, height, plates, steps;
    float velRange;
    uint64_t genSeed;
    uint32_t worldSeed;
    double arrival_s;     /* arrival time, seconds from the start of a trace */
} tecto_request;
typedef struct tecto_request_result {
    int status;           /* TECTO_OK, TECTO_ERR_BUDGET (rejected) or another error */
    double arrival_s, admit_s, finish_s;
    float height_checksum; /* sum of the final height field (float64 accumulated, then rounded) */
} tecto_request_result;
typedef struct tecto_server_stats {
    int completed, rejected, ticks, max_active;
    double wall_s;                 /* trace start to last completion */
    double cell_updates;           /* sum over completed requests of cells x steps */
    double cell_updates_per_s;
    double latency_p50_s, latency_p99_s, latency_mean_s;
    double peak_bytes;             /* largest admitted footprint */
} tecto_server_stats;

#define TECTO_SERVER_DRY_RUN 1     /* flag: no device work; a tick costs `dry_tick_s_per_mcell` */

int tecto_server_create(const tecto_settings *settings, size_t budget_bytes, int max_worlds, int flags,
                        tecto_server **out);
int tecto_server_destroy(tecto_server *server);
/* Replay a trace in real time with continuous batching; results[i] belongs to requests[i]. */
int tecto_server_run_trace(tecto_server *server, const tecto_request *requests, int n,
                           tecto_stream_t stream, tecto_request_result *results,
                           tecto_server_stats *stats);
/* The same trace served one request at a time with the plain one-world path (the baseline). */
int tecto_server_run_trace_sequential(tecto_server *server, const tecto_request *requests, int n,
                                      tecto_stream_t stream, tecto_request_result *results,
                                      tecto_server_stats *stats);
/* Headless output of served results: each request that finishes writes, into `directory`,
 * request_<i>_height.png (TECTO_SERVER_OUT_HEIGHT_PNG: the 16-bit export over [height_min,
 * height_max]), request_<i>_plates.png (TECTO_SERVER_OUT_PLATES_PNG) and request_<i>.snap
 * (TECTO_SERVER_OUT_SNAPSHOT), i its index in the trace, before its world is released.  A failed
 * write sets that request's status.  what = 0 turns output off.  Dry runs write nothing. */
#define TECTO_SERVER_OUT_HEIGHT_PNG 1
#define TECTO_SERVER_OUT_PLATES_PNG 2
#define TECTO_SERVER_OUT_SNAPSHOT 4
int tecto_server_set_output(tecto_server *server, const char *directory, int what, float height_min,
                            float height_max);
/* How admitted worlds are initialised on the device: TECTO_SERVER_INIT_SYNTHETIC (default: the
 * engine's generator with the request's plates, velRange and genSeed) or TECTO_SERVER_INIT_REFERENCE
 * (tecto_world_init_reference with numStartingPlates = the request's plates, the server settings'
 * Voronoi generations and the request's worldSeed). */
#define TECTO_SERVER_INIT_SYNTHETIC 0
#define TECTO_SERVER_INIT_REFERENCE 1
int tecto_server_set_init(tecto_server *server, int mode);
/* Dry-run cost model: seconds one tick takes per million active cells (default 2e-4). */
int tecto_server_set_dry_cost(tecto_server *server, double seconds_per_mcell_step);
/* Size-aware admission: requests of at least heavy_cells cells are heavy, and at most heavy_slots
 * of them are live at a time (defaults 2^20 and 1).  heavy_slots = 0 lifts the limit: every
 * request joins as soon as it fits.  Applies to trace replays and live serving alike. */
int tecto_server_set_policy(tecto_server *server, size_t heavy_cells, int heavy_slots);

/* ---- live serving: requests submitted as they come, the caller drives the ticks ----------
 *
 * tecto_server_submit queues a copy of *request and returns its ticket (0, 1, 2, ... in submission
 * order); the request's arrival_s is replaced by the submission time on the server's clock (seconds
 * since tecto_server_create; the simulated clock in a dry run).  A request that can never be served
 * (invalid, or larger than the whole budget) is done at once with TECTO_ERR_INVALID or
 * TECTO_ERR_BUDGET as its status.  tecto_server_tick admits waiting requests first-come first-served
 * against the budget, advances every admitted world one step as one batch, and retires the worlds
 * that are done (checksum, and the outputs of tecto_server_set_output named request_<ticket>);
 * with nothing admitted it does no device work.  It reports the admitted and waiting counts after
 * the tick.  A request whose world cannot be created (out of device memory, say) is done with that
 * error as its status, in a trace replay too; if a tick fails, every pending request takes its
 * error as status and leaves.
 * tecto_server_poll gives a ticket's state and result; tecto_server_live_stats summarises the
 * submitted requests (wall_s = the server clock now).  One host thread owns a server;
 * tecto_server_run_trace is refused while live requests are pending. */
#define TECTO_REQUEST_WAITING 0
#define TECTO_REQUEST_RUNNING 1
#define TECTO_REQUEST_DONE 2
int tecto_server_submit(tecto_server *server, const tecto_request *request, int *ticket);
int tecto_server_tick(tecto_server *server, tecto_stream_t stream, int *active, int *waiting);
int tecto_server_poll(tecto_server *server, int ticket, int *state, tecto_request_result *result);
int tecto_server_live_stats(tecto_server *server, tecto_server_stats *stats);

/* The reference's world initialisation (PlateTectonicSim::initializeTectonics,
 * plate_tectonic_sim.cu:705-773) from the world's settings (sim.numStartingPlates,
 * sim.numVoronoiSeeds[0..numVoronoiGenerations)) and its seed: plate centres, Voronoi seed
 * generations and plate kinematics drawn on the host from std::default_random_engine through
 * std::uniform_real_distribution<float> in the reference's order; the nearest-seed plate ids
 * (initPlateIDs) and the simplex height map (initHeightmap, 5000..15000) on the device; CCL labels.
 * Everything else starts at zero, iteration 0.  Plate fragments keep their id (the reference's
 * post-CCL relabel is not part of this engine). */
int tecto_world_init_reference(tecto_world *world, tecto_stream_t stream);
/* PlateTectonicSim::initialize(numStartingPlates, numVoronoiSeeds) with its arguments: stores them in
 * the world's settings and runs tecto_world_init_reference. */
int tecto_world_init(tecto_world *world, int numPlates, const int *numVoronoiSeeds, int generations,
                     tecto_stream_t stream);
/* The host part alone: seed_x / seed_y / seed_id (capacity entries; *count = seeds of the last
 * generation, or the plate centres) and the plate records it draws. */
int tecto_reference_seeds(int width, int height, uint32_t seed, int numPlates, const int *numVoronoiSeeds,
                          int generations, float *seed_x, float *seed_y, uint8_t *seed_id, int capacity,
                          int *count, tecto_plate *plates, tecto_plate_dynamics *dynamics);

/* Device-side synthetic generator: same result as tecto_generate_world_host, computed on the GPU
 * (the on-device world init the server uses). */
int tecto_world_init_synthetic_device(tecto_world *world, int numPlates, float velRange,
                                      uint64_t genSeed, tecto_stream_t stream);

/* ---- output and checkpoints ------------------------------------------------------------ */

/* PNG encoding of a host image (kind: TECTO_PNG_GRAY16 = uint16 per pixel in host order,
 * TECTO_PNG_RGB8 = 3 bytes per pixel, TECTO_PNG_GRAY8 = 1 byte), rows top to bottom.  The encoder
 * writes stored deflate blocks (no compression).  out == NULL: only *written (the file size) is
 * set. */
#define TECTO_PNG_GRAY16 0
#define TECTO_PNG_RGB8 1
#define TECTO_PNG_GRAY8 2
int tecto_png_encode(const void *pixels, int width, int height, int kind, void *out, size_t capacity,
                     size_t *written);

/* The reference's two image exports (src/cuda_compute/texture_save.cu), written as a PNG file:
 *  TECTO_EXPORT_HEIGHT_GRAY16  saveFloatCudaTextureToDiskAsGray16: (uint16)(clamp((h - min) /
 *                              (max - min), 0, 1) * 65535), converted on the device; the reference
 *                              passes minUpliftClamp / maxUpliftClamp (plate_tectonic_sim.cu:635);
 *                              the file carries the reference's sRGB chunk (perceptual intent);
 *  TECTO_EXPORT_PLATES_RGB     saveGrayscale8BitCudaTextureToDiskAsRgb: one HSV colour per plate
 *                              id, id 255 the background (230, 235, 240); min/max unused.
 * Synchronous on `stream`. */
/* The colour of each plate id as the RGB export uses it (rgb768[3 * id + c]). */
int tecto_plate_palette(uint8_t *rgb768);
#define TECTO_EXPORT_HEIGHT_GRAY16 0
#define TECTO_EXPORT_PLATES_RGB 1
int tecto_world_export_png(tecto_world *world, int kind, const char *path, float min_value, float max_value,
                           tecto_stream_t stream);

/* Checkpoint / resume: the complete state a step reads (heights, water, sediment, flux, plate ids,
 * CCL labels, pair type bitmap, divergence bitmap, plate and plate dynamics records, the
 * asthenosphere pressure texture, settings, seed, iteration) as one file.  A world of the same size loaded from it steps bit-identically to the saved world.  The
 * reference has no counterpart (it restarts from config.json and its seed). */
int tecto_world_save_snapshot(tecto_world *world, const char *path, tecto_stream_t stream);
int tecto_world_load_snapshot(tecto_world *world, const char *path, tecto_stream_t stream);
/* Size and settings stored in a snapshot file, to create the world that loads it. */
int tecto_snapshot_info(const char *path, int *width, int *height, tecto_settings *settings);

/* ---- status -------------------------------------------------------------------------- */

/* Number of engine kernels enqueued for this world so far (graph replays count the kernels of the
 * captured step); the reference has no counterpart (it prints a per-step wall time,
 * plate_tectonic_sim.cu:128-130). */
int tecto_world_launch_count(const tecto_world *world, uint64_t *count);

/* Wait for the world's stream work and report device-side error flags (bounded waits that gave
 * up) as TECTO_ERR_DEVICE_TIMEOUT. */
int tecto_world_check(tecto_world *world, tecto_stream_t stream);
/* Self-test of the division the erosion kernels use where a divisor repeats (Markstein's
 * correction of a reciprocal product, with an IEEE-division fallback outside its safe range):
 * out[i] = a[i] / b[i] computed that way, on device buffers.  Tests compare it bit for bit with
 * the IEEE quotient. */
int tecto_selftest_div(const float *a, const float *b, float *out, size_t n, tecto_stream_t stream);
/* The same for the per-lane form the erosion kernels use where every cell has its own divisor:
 * the quotient from a correctly rounded reciprocal (one Newton-Raphson step from the hardware's
 * approximation), with the IEEE division outside its safe range. */
int tecto_selftest_div_var(const float *a, const float *b, float *out, size_t n, tecto_stream_t stream);
/* Exhaustive self-test of the erosion kernels' reciprocal and square root: for every positive
 * normal float, whether each equals the correctly rounded result.  bad (device, 512 counters)
 * receives the mismatches per exponent field: bad[e] for the reciprocal, bad[256 + e] for the
 * square root. */
int tecto_selftest_rcp_sqrt(unsigned long long *bad, tecto_stream_t stream);
const char *tecto_last_error_string(void);
const char *tecto_version(void);

#ifdef __cplusplus
}
#endif

#endif /* TECTO_H */
