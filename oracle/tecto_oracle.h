/*
 * tecto_oracle.h - CPU oracle for the plate-tectonics step.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's hot-path kernels (MarWo22/master_thesis,
 * src/cuda_compute/), one function per phase, each citing the reference lines it follows.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it; the engine
 * (master_thesis_gb300/) never does.
 *
 * Arithmetic: IEEE single precision in the reference's expression order, no multiply-add
 * contraction (built with -ffp-contract=off), sin from include/tecto_math.h.  Pinned against the
 * reference kernels themselves, compiled for the CPU from their own sources by oracle/Makefile
 * (target `ref`) and run with a sequential thread emulation (tests/golden/).
 *
 * Where the reference is order-dependent the oracle fixes one order, which the engine shares:
 *  - arrival slots at a destination cell: ascending source linear index (a stable sort);
 *  - accretion marks that hit the same cell: the mark of the highest destination index wins;
 *  - thermal erosion: Jacobi (gather) form, own outflows subtracted in direction order, then
 *    inflows added in direction order.
 */
#ifndef TECTO_ORACLE_H
#define TECTO_ORACLE_H

#include <stdint.h>
#include "../include/tecto.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Per-plate integer displacement of this step and the updated sub-cell centres. */
void or_plate_offsets(const tecto_plate *plates, int32_t *off_x, int32_t *off_y,
                      tecto_plate *plates_next);

/* Advection + canonical grouping: dest[i] for every cell, packed arrival words, and the
 * stably sorted (dest, src) pairs (any output may be NULL). */
void or_collision_words(int W, int H, const uint8_t *id, const int32_t *off_x, const int32_t *off_y,
                        uint32_t *dest, uint32_t *word, uint32_t *sorted_keys,
                        uint32_t *sorted_vals);

/* Collision-type evidence + pair bitmap update (type_bitmap in/out). */
void or_collision_types(int W, int H, const uint32_t *word, const float *h_old,
                        const int32_t *off_x, const int32_t *off_y,
                        const tecto_kernel_settings *ks, uint8_t *type_bitmap);

/* processCollisions + flipDivergedBitmap + uplift.  div_bitmap in/out; acc receives accretion
 * marks (zeroed first).  seed/iteration are the world's seed and step counter. */
void or_resolve(int W, int H, const uint8_t *id_old, const float *h_old, const uint32_t *word,
                const int32_t *off_x, const int32_t *off_y, const uint8_t *type_bitmap,
                uint32_t *div_bitmap, const tecto_settings *st, uint32_t seed, uint32_t iteration,
                float *h_new, uint8_t *id_new, uint8_t *acc);

/* Thermal erosion, `iters` gather iterations, in place. */
void or_resolve_ex(int W, int H, const uint8_t *id_old, const float *h_old, const uint32_t *word,
                   const int32_t *off_x, const int32_t *off_y, const uint8_t *bm, uint32_t *div_bitmap,
                   const tecto_settings *st, uint32_t seed, uint32_t iteration, float *h_new,
                   uint8_t *id_new, uint8_t *acc, float *up_h, uint8_t *up_t);

/* The reference uplift (continental propagation, JFA distance field, applyUplift). */
void or_uplift_ref(int W, int H, const uint32_t *word, const float *up_h, const uint8_t *up_t,
                   const float *h_old, const tecto_plate *plates, const uint8_t *id_new, float *h_new,
                   const tecto_kernel_settings *ks, int32_t *jfa_seed, int32_t *jfa_dist);
float or_expf(float x);
float or_log10f(float x);

void or_thermal(int W, int H, float *h, int iters, const tecto_kernel_settings *ks);

/* Hydraulic erosion, `iters` sub-iterations of step dt, in place; flux is 4 floats per cell. */
void or_hydraulic(int W, int H, float *h, float *w, float *s, float *flux, int iters, float dt,
                  uint32_t rain_seed, const tecto_kernel_settings *ks);

/* applyAccretion, in place on id. */
void or_accretion(int W, int H, const float *h, const uint8_t *acc, uint8_t *id,
                  const tecto_kernel_settings *ks);

/* CCL labels (TECTO_CCL_4 / _8 / _REF8), each the minimum linear index of its component. */
void or_ccl(int W, int H, const uint8_t *id, uint32_t *labels, int mode);

/* One full step.  Buffers are the world's state and are updated in place; word/acc/labels are
 * outputs (labels only written on CCL steps). *iteration is advanced. */
void or_step(int W, int H, float *h, float *w, float *s, float *flux, uint8_t *id,
             uint32_t *labels, uint32_t *word, uint8_t *acc, uint8_t *type_bitmap,
             uint32_t *div_bitmap, tecto_plate *plates, const tecto_settings *st, uint32_t seed,
             uint32_t *iteration);

/* processCollisions with plate dynamics' friction per plate (fixed point x 2^40 in fric[255]; plates:
 * velocities, dyn: masses); or_resolve_ex when fric is NULL. */
void or_resolve_dyn(int W, int H, const uint8_t *id_old, const float *h_old, const uint32_t *word,
                    const int32_t *off_x, const int32_t *off_y, const uint8_t *bm, uint32_t *div_bitmap,
                    const tecto_settings *st, uint32_t seed, uint32_t iteration, float *h_new,
                    uint8_t *id_new, uint8_t *acc, float *up_h, uint8_t *up_t, const tecto_plate *plates,
                    const tecto_plate_dynamics *dyn, int64_t *fric);
/* Plate dynamics: per-plate mass, size and geometric centre of a state; computeCurl at one cell;
 * applyPlateMovementChanges; a whole step with dynamics (dyn NULL or plateDynamics off: or_step). */
void or_plate_stats(int W, int H, const float *h, const uint8_t *id, uint32_t iteration,
                    tecto_plate_dynamics *dyn);
void or_curl_at(const float *pr, int pw, int ph, int W, int H, int cx, int cy, float *out_x, float *out_y);
void or_plate_motion(int W, int H, tecto_plate *plates, tecto_plate_dynamics *dyn, const int64_t *fric,
                     const float *pressure, int pw, int ph, const tecto_kernel_settings *ks);
void or_step_dyn(int W, int H, float *h, float *w, float *s, float *flux, uint8_t *id, uint32_t *labels,
                 uint32_t *word, uint8_t *acc, uint8_t *bm, uint32_t *div_bitmap, tecto_plate *plates,
                 tecto_plate_dynamics *dyn, const float *pressure, int pw, int ph, const tecto_settings *st,
                 uint32_t seed, uint32_t *iteration);

/* Image export (src/cuda_compute/texture_save.cu): convertFloatToGray16Kernel (:80-96) over n
 * heights, and convertGrayscaleToRgbKernel's colour (:16-70) of every plate id as a 256 x 3 palette. */
void or_gray16(size_t n, const float *h, float minv, float maxv, uint16_t *out);
void or_plate_palette(uint8_t *rgb768);

/* The reference's world initialisation: the host draws (seeds of the last Voronoi generation, plate
 * records) and the per-cell plate ids and height map. */
int or_reference_seeds(int W, int H, uint32_t seed, int numPlates, const int *gens, int ngens, float *seed_x,
                       float *seed_y, uint8_t *seed_id, int capacity, int *count, tecto_plate *plates,
                       tecto_plate_dynamics *dyn);
void or_init_reference(int W, int H, uint32_t seed, const float *sx, const float *sy, const uint8_t *sid, int S,
                       float *h, uint8_t *id);

/* Plate policy after a step: applyCCL's relabel of plate fragments (returns cells left without an
 * id) and mergePlates (returns merges). */
int or_relabel(int W, int H, uint8_t *id, const uint32_t *labels, tecto_plate *plates, tecto_plate_dynamics *dyn,
               int minPlateSize);
int or_merge(int W, int H, uint8_t *id, const tecto_plate *plates, const tecto_plate_dynamics *dyn,
             uint8_t *type_bitmap, const tecto_kernel_settings *ks);

/* Building blocks exposed for unit tests. */
uint32_t or_hash(uint32_t v);
float or_simplex3(float x, float y, float z, float scale, int seed);
float or_rain_noise(int x, int y, int seed);
float or_lerp(float a, float b, float t);
void or_gaussian_weights(float sigma, int radius, float *w_out);
float or_sinf(float x);
void or_use_libm_sin(int on);

/* The reference's default parameters and the benchmark's mapping of them (the same values as
 * tecto_settings_default / tecto_settings_baseline), and the benchmark's synthetic world generator
 * (the same worlds as tecto_generate_world_host), for the legs that must not load the engine. */
void or_settings_default(tecto_settings *out);
void or_settings_baseline(tecto_settings *out);
int or_generate_world(int W, int H, int P, float velRange, uint64_t genSeed, float *height_out, uint8_t *id_out,
                      tecto_plate *plates_out);

#ifdef __cplusplus
}
#endif

#endif /* TECTO_ORACLE_H */
