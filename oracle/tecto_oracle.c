/*
 * tecto_oracle.c - CPU oracle for the plate-tectonics step.  TEST INFRASTRUCTURE ONLY.
 * See tecto_oracle.h for the contract.  Reference paths are relative to MarWo22/master_thesis.
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off -fPIC -shared (oracle/Makefile).
 */
#include "tecto_oracle.h"
#include "../include/tecto_math.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NPLATE 255u
/* plate dynamics' fixed-point sums (the engine uses the same scales) */
#define OR_MASS_SCALE 65536.0f
#define OR_MASS_LIMIT 1099511627776.0f
#define OR_ANG_SCALE 4294967296.0f
#define OR_FRIC_SCALE 1099511627776.0f
#define OR_FRIC_LIMIT 4194304.0f
#define OR_TWO_PI_F 6.28318548202514648f

/* ---- addressing --------------------------------------------------------------------- */

/* CudaTexture::wrapCoordinate (src/cuda_compute/types/cuda_texture.cuh:67-76) */
static inline int wrapc(int c, int n)
{
    const int r = c % n;
    return r + (n & (r >> 31));
}

/* CudaTexture::coordinateToIndex (cuda_texture.cuh:55-60): wrapped y * W + x */
static inline uint32_t cidx(int x, int y, int W, int H)
{
    return (uint32_t)(wrapc(y, H) * W + wrapc(x, W));
}

/* upperTriangleIndexUnchecked(i, j, 255) (src/cuda_compute/cuda_helper.cuh:97-104), i < j */
static inline uint32_t tri_index(uint32_t i, uint32_t j)
{
    const uint32_t base = i * (2u * NPLATE - i - 1u) / 2u;
    return base + (j - i - 1u);
}

/* ---- noise (vendored cudaNoise, src/cuda_compute/cuda_noise.cuh) ---------------------- */

/* Robert Jenkins' 32-bit integer hash, as used by cuda_noise.cuh:44-54. */
uint32_t or_hash(uint32_t a)
{
    a = (a + 0x7ed55d16u) + (a << 12);
    a = (a ^ 0xc761c23cu) ^ (a >> 19);
    a = (a + 0x165667b1u) + (a << 5);
    a = (a + 0xd3a2646cu) ^ (a << 9);
    a = (a + 0xfd7046c5u) + (a << 3);
    a = (a ^ 0xb55a4f09u) ^ (a >> 16);
    return a;
}

/* float -> u32 with the GPU's conversion semantics (truncate, saturate, NaN -> 0). */
static inline uint32_t f2u_sat(float v)
{
    if (!(v > 0.0f)) return 0u;
    if (v >= 4294967296.0f) return 0xffffffffu;
    return (uint32_t)v;
}

/* randomFloat + randomGrid (cuda_noise.cuh:66-71, :108-111) */
static float random_grid(int x, int y, int z, int seed)
{
    float v = (float)x * 1723.0f;
    v = v + (float)y * 93241.0f;
    v = v + (float)z * 149812.0f;
    v = v + 3824.0f;
    v = v + (float)seed;
    const uint32_t hv = or_hash(f2u_sat(v));
    const float r = (float)hv / 4294967296.0f; /* (float)0xffffffff */
    return r * 2.0f - 1.0f;
}

/* discreteNoise(make_float3(x, 0, y), 1, seed) as called by rain (cuda_noise.cuh:470-477,
 * plate_tectonics_kernel.cu:2434). */
float or_rain_noise(int x, int y, int seed)
{
    const int ix = (int)((float)x * 1.0f);
    const int iy = 0;
    const int iz = (int)((float)y * 1.0f);
    return random_grid(ix, iy, iz, seed);
}

/* Gustavson's 3D simplex gradient set, in the order of cuda_noise.cuh:158-160 */
static const float GRAD3[12][3] = {
    {1, 1, 0}, {-1, 1, 0}, {1, -1, 0}, {-1, -1, 0},
    {1, 0, 1}, {-1, 0, 1}, {1, 0, -1}, {-1, 0, -1},
    {0, 1, 1}, {0, -1, 1}, {0, 1, -1}, {0, -1, -1}};

static inline float gdot(int g, float x, float y, float z)
{
    return (GRAD3[g][0] * x + GRAD3[g][1] * y) + GRAD3[g][2] * z;
}

static inline int perm12(uint32_t p) { return (int)(or_hash(p) % 12u); }

/* simplexNoise (cuda_noise.cuh:228-320): Gustavson 3D simplex with hashed gradients. */
float or_simplex3(float px, float py, float pz, float scale, int seed)
{
    const float xin = px * scale, yin = py * scale, zin = pz * scale;
    const float F3 = 1.0f / 3.0f, G3 = 1.0f / 6.0f;
    const float s = ((xin + yin) + zin) * F3;
    const int i = (int)floorf(xin + s);
    const int j = (int)floorf(yin + s);
    const int k = (int)floorf(zin + s);
    const float t = (float)(i + j + k) * G3;
    const float X0 = (float)i - t, Y0 = (float)j - t, Z0 = (float)k - t;
    const float x0 = xin - X0, y0 = yin - Y0, z0 = zin - Z0;
    int i1, j1, k1, i2, j2, k2;
    if (x0 >= y0) {
        if (y0 >= z0) { i1 = 1; j1 = 0; k1 = 0; i2 = 1; j2 = 1; k2 = 0; }
        else if (x0 >= z0) { i1 = 1; j1 = 0; k1 = 0; i2 = 1; j2 = 0; k2 = 1; }
        else { i1 = 0; j1 = 0; k1 = 1; i2 = 1; j2 = 0; k2 = 1; }
    } else {
        if (y0 < z0) { i1 = 0; j1 = 0; k1 = 1; i2 = 0; j2 = 1; k2 = 1; }
        else if (x0 < z0) { i1 = 0; j1 = 1; k1 = 0; i2 = 0; j2 = 1; k2 = 1; }
        else { i1 = 0; j1 = 1; k1 = 0; i2 = 1; j2 = 1; k2 = 0; }
    }
    const float x1 = (x0 - (float)i1) + G3, y1 = (y0 - (float)j1) + G3, z1 = (z0 - (float)k1) + G3;
    const float x2 = (x0 - (float)i2) + 2.0f * G3, y2 = (y0 - (float)j2) + 2.0f * G3,
                z2 = (z0 - (float)k2) + 2.0f * G3;
    const float x3 = (x0 - 1.0f) + 3.0f * G3, y3 = (y0 - 1.0f) + 3.0f * G3,
                z3 = (z0 - 1.0f) + 3.0f * G3;
    const uint32_t us = (uint32_t)seed, ui = (uint32_t)i, uj = (uint32_t)j, uk = (uint32_t)k;
    const int gi0 = perm12(us + ui * 607495u + uj * 359609u + uk * 654846u);
    const int gi1 = perm12(us + (ui + (uint32_t)i1) * 607495u + (uj + (uint32_t)j1) * 359609u +
                           (uk + (uint32_t)k1) * 654846u);
    const int gi2 = perm12(us + (ui + (uint32_t)i2) * 607495u + (uj + (uint32_t)j2) * 359609u +
                           (uk + (uint32_t)k2) * 654846u);
    const int gi3 = perm12(us + (ui + 1u) * 607495u + (uj + 1u) * 359609u + (uk + 1u) * 654846u);
    float n0, n1, n2, n3;
    float t0 = ((0.6f - x0 * x0) - y0 * y0) - z0 * z0;
    if (t0 < 0.0f) n0 = 0.0f; else { t0 = t0 * t0; n0 = (t0 * t0) * gdot(gi0, x0, y0, z0); }
    float t1 = ((0.6f - x1 * x1) - y1 * y1) - z1 * z1;
    if (t1 < 0.0f) n1 = 0.0f; else { t1 = t1 * t1; n1 = (t1 * t1) * gdot(gi1, x1, y1, z1); }
    float t2 = ((0.6f - x2 * x2) - y2 * y2) - z2 * z2;
    if (t2 < 0.0f) n2 = 0.0f; else { t2 = t2 * t2; n2 = (t2 * t2) * gdot(gi2, x2, y2, z2); }
    float t3 = ((0.6f - x3 * x3) - y3 * y3) - z3 * z3;
    if (t3 < 0.0f) n3 = 0.0f; else { t3 = t3 * t3; n3 = (t3 * t3) * gdot(gi3, x3, y3, z3); }
    return 32.0f * (((n0 + n1) + n2) + n3);
}

/* cuda::std::lerp (P0811R3 algorithm), used by processDivergence (plate_tectonics_kernel.cu:354) */
float or_lerp(float a, float b, float t)
{
    if ((a <= 0.0f && b >= 0.0f) || (a >= 0.0f && b <= 0.0f)) return t * b + (1.0f - t) * a;
    if (t == 1.0f) return b;
    const float x = a + t * (b - a);
    if ((t > 1.0f) == (b > a)) return b < x ? x : b;
    return x < b ? x : b;
}

/* The engine's sine (include/tecto_math.h) by default; libm's sinf when pinning against the
 * reference's kernels compiled for the CPU, which call the host sinf. */
static int g_libm_sin = 0;
void or_use_libm_sin(int on) { g_libm_sin = on; }
float or_sinf(float x) { return g_libm_sin ? sinf(x) : tecto_sinf(x); }
float or_expf(float x) { return tecto_expf(x); }
float or_log10f(float x) { return tecto_log10f(x); }

/* ---- plate kinematics ------------------------------------------------------------------ */

/* getPixelMovements' integer displacement (plate_tectonics_kernel.cu:248-257) and the sub-cell
 * centre update of applyPlateMovementChanges (:1871-1878). */
void or_plate_offsets(const tecto_plate *p, int32_t *off_x, int32_t *off_y, tecto_plate *next)
{
    for (unsigned k = 0; k < NPLATE; ++k) {
        const float mx = p[k].direction_x * p[k].velocity;
        const float my = p[k].direction_y * p[k].velocity;
        const float cx = p[k].pixelCenter_x + mx;
        const float cy = p[k].pixelCenter_y + my;
        const float fx = floorf(cx), fy = floorf(cy);
        off_x[k] = (int32_t)fx;
        off_y[k] = (int32_t)fy;
        if (next) {
            next[k] = p[k];
            next[k].pixelCenter_x = cx - fx;
            next[k].pixelCenter_y = cy - fy;
        }
    }
}

/* ---- advection + grouping --------------------------------------------------------------- */

/* getPixelMovements (plate_tectonics_kernel.cu:232-271) and registerPlateCollisions
 * (:273-298) with arrivals taken in ascending source order (the stable sort's order). */
void or_collision_words(int W, int H, const uint8_t *id, const int32_t *off_x, const int32_t *off_y,
                        uint32_t *dest, uint32_t *word, uint32_t *sorted_keys, uint32_t *sorted_vals)
{
    const size_t N = (size_t)W * (size_t)H;
    uint32_t *d = dest ? dest : (uint32_t *)malloc(N * sizeof(uint32_t));
    uint32_t *cnt = (uint32_t *)calloc(N + 1, sizeof(uint32_t));
    for (size_t i = 0; i < N; ++i) {
        const int x = (int)(i % (size_t)W), y = (int)(i / (size_t)W);
        const uint8_t p = id[i];
        d[i] = cidx(x + off_x[p], y + off_y[p], W, H);
    }
    if (word) {
        memset(word, 0, N * sizeof(uint32_t));
        for (size_t i = 0; i < N; ++i) {
            const uint32_t k = cnt[d[i]]++;
            if (k < 4u) word[d[i]] |= (uint32_t)(255u - id[i]) << (8u * k);
        }
    } else {
        for (size_t i = 0; i < N; ++i) cnt[d[i]]++;
    }
    if (sorted_keys || sorted_vals) {
        /* counting sort: exclusive prefix of arrival counts, then a stable scatter */
        uint32_t run = 0;
        for (size_t c = 0; c < N; ++c) { const uint32_t v = cnt[c]; cnt[c] = run; run += v; }
        for (size_t i = 0; i < N; ++i) {
            const uint32_t pos = cnt[d[i]]++;
            if (sorted_keys) sorted_keys[pos] = d[i];
            if (sorted_vals) sorted_vals[pos] = (uint32_t)i;
        }
    }
    free(cnt);
    if (!dest) free(d);
}

/* ---- collision typing ------------------------------------------------------------------- */

typedef struct { int32_t c[5]; } pair_counts; /* CollisionTypeCounts field order,
                                                 plate_tectonics_kernel.cuh:47-54 */

/* writeCollision (plate_tectonics_kernel.cu:794-836), including the as-compiled early-exit test
 * `packed >> 0 & 1 && packed >> 4 & 0x0F < cooldown` == `(packed & 1) && ((packed >> 4) &
 * (15 < cooldown))` (:813). */
static void write_collision(float hA, float hB, uint8_t A, uint8_t B, const uint8_t *bm,
                            pair_counts *counts, const tecto_kernel_settings *ks)
{
    const int cond = A < B;
    const uint8_t mn = cond ? A : B, mx = cond ? B : A;
    const float mnH = cond ? hA : hB, mxH = cond ? hB : hA;
    const uint32_t idx = tri_index(mn, mx);
    const uint8_t packed = bm[idx];
    if ((packed & 1u) && ((packed >> 4) & (uint32_t)(0x0F < ks->collisionTypeUpdateCooldown)))
        return;
    const int minCont = mnH >= ks->continentalCrustThreshold;
    const int maxCont = mxH >= ks->continentalCrustThreshold;
    if (minCont && maxCont) counts[idx].c[4]++;
    else if (minCont) counts[idx].c[2]++;
    else if (maxCont) counts[idx].c[0]++;
    else if (mnH <= mxH) counts[idx].c[1]++;
    else counts[idx].c[3]++;
}

/* determineCollisionType kernel (plate_tectonics_kernel.cu:838-888) and
 * createCollisionTypeMatrix (:890-972). */
void or_collision_types(int W, int H, const uint32_t *word, const float *h_old, const int32_t *off_x,
                        const int32_t *off_y, const tecto_kernel_settings *ks, uint8_t *bm)
{
    const size_t N = (size_t)W * (size_t)H;
    pair_counts *counts = (pair_counts *)calloc(TECTO_NUM_PAIRS, sizeof(pair_counts));
    for (size_t d = 0; d < N; ++d) {
        const uint32_t cp = word[d];
        if (cp <= 0xFFu) continue;
        const uint8_t A = (uint8_t)(255u - (cp & 0xFFu));
        const uint8_t B = (uint8_t)(255u - ((cp >> 8) & 0xFFu));
        const uint8_t C = (uint8_t)(255u - ((cp >> 16) & 0xFFu));
        const uint8_t D = (uint8_t)(255u - ((cp >> 24) & 0xFFu));
        const int x = (int)(d % (size_t)W), y = (int)(d / (size_t)W);
        /* determineCollisionHeight (:781-792): height at the arrival's source cell */
        const float hA = h_old[cidx(x - off_x[A], y - off_y[A], W, H)];
        const float hB = h_old[cidx(x - off_x[B], y - off_y[B], W, H)];
        if (D != NPLATE) {
            const float hC = h_old[cidx(x - off_x[C], y - off_y[C], W, H)];
            const float hD = h_old[cidx(x - off_x[D], y - off_y[D], W, H)];
            write_collision(hA, hB, A, B, bm, counts, ks);
            write_collision(hA, hC, A, C, bm, counts, ks);
            write_collision(hA, hD, A, D, bm, counts, ks);
            write_collision(hB, hC, B, C, bm, counts, ks);
            write_collision(hB, hD, B, D, bm, counts, ks);
            write_collision(hC, hD, C, D, bm, counts, ks);
        } else if (C != NPLATE) {
            const float hC = h_old[cidx(x - off_x[C], y - off_y[C], W, H)];
            write_collision(hA, hB, A, B, bm, counts, ks);
            write_collision(hA, hC, A, C, bm, counts, ks);
            write_collision(hB, hC, B, C, bm, counts, ks);
        } else {
            write_collision(hA, hB, A, B, bm, counts, ks);
        }
    }
    for (uint32_t idx = 0; idx < TECTO_NUM_PAIRS; ++idx) {
        const uint32_t packed = bm[idx];
        const int hasType = packed & 1u;
        const int count = (int)((packed >> 4) & 0x0Fu);
        const int32_t *c = counts[idx].c;
        const uint32_t total = (uint32_t)(c[0] + c[1] + c[2] + c[3] + c[4]);
        if (total == 0) continue;
        if (hasType && count < ks->collisionTypeUpdateCooldown) {
            bm[idx] = (uint8_t)((packed & 0x0Fu) | (((uint32_t)(count + 1) & 0x0Fu) << 4));
            continue;
        }
        if (total < (uint32_t)ks->minCollisionSize) continue;
        uint32_t out = packed & 0x0Fu;
        const int hasPol = (packed >> 2) & 1u;
        const int polA = (packed >> 3) & 1u;
        const int oppA = c[2] + c[4], oppB = c[0] + c[4];
        const int subA = c[0] + c[1] - oppA, subB = c[2] + c[3] - oppB;
        if (c[4] >= c[0] + c[1] && c[4] >= c[2] + c[3]) out |= 3u;
        else if (subA > 0 && subA > subB && (!hasPol || polA)) out = (out & ~2u) | 13u;
        else if (subB > 0 && subB > subA && (!hasPol || !polA)) out = (out & ~10u) | 5u;
        bm[idx] = (uint8_t)out;
    }
    free(counts);
}

/* determineCollisionType device function (plate_tectonics_kernel.cu:611-649) */
static uint32_t pair_type(const uint8_t *bm, uint8_t A, uint8_t B, float hA, float hB,
                          const tecto_kernel_settings *ks)
{
    const int cond = A < B;
    const uint8_t mn = cond ? A : B, mx = cond ? B : A;
    const float mnH = cond ? hA : hB, mxH = cond ? hB : hA;
    const uint8_t packed = bm[tri_index(mn, mx)];
    const int hasType = packed & 1u, type = (packed >> 1) & 1u, pol = (packed >> 3) & 1u;
    uint32_t out = 0;
    if (hasType && type == 0) {
        if (pol == 1) {
            if (mnH >= ks->continentalCrustThreshold) out = mn == A ? 3u : 4u;
            else out = mn == A ? 1u : 2u;
        }
        if (pol == 0) {
            if (mxH >= ks->continentalCrustThreshold) out = mx == A ? 3u : 4u;
            else out = mx == A ? 1u : 2u;
        }
    }
    return out;
}

/* ---- resolve ------------------------------------------------------------------------------ */

void or_gaussian_weights(float sigma, int radius, float *w_out)
{
    double tmp[17];
    double sum = 0.0;
    for (int k = -radius; k <= radius; ++k) {
        tmp[k + radius] = exp(-(double)(k * k) / (2.0 * (double)sigma * (double)sigma));
        sum += tmp[k + radius];
    }
    for (int k = 0; k <= 2 * radius; ++k) w_out[k] = (float)(tmp[k] / sum);
}

void or_resolve(int W, int H, const uint8_t *id_old, const float *h_old, const uint32_t *word,
                const int32_t *off_x, const int32_t *off_y, const uint8_t *bm, uint32_t *div_bitmap,
                const tecto_settings *st, uint32_t seed, uint32_t iteration, float *h_new,
                uint8_t *id_new, uint8_t *acc)
{
    or_resolve_ex(W, H, id_old, h_old, word, off_x, off_y, bm, div_bitmap, st, seed, iteration, h_new,
                  id_new, acc, NULL, NULL);
}

/* processCollisions plus the UpliftData record of every convergent cell (up_h = heightAddition,
 * up_t = typeByte, processConvergence :501-582); up_h / up_t may be NULL. */
void or_resolve_ex(int W, int H, const uint8_t *id_old, const float *h_old, const uint32_t *word,
                   const int32_t *off_x, const int32_t *off_y, const uint8_t *bm, uint32_t *div_bitmap,
                   const tecto_settings *st, uint32_t seed, uint32_t iteration, float *h_new,
                   uint8_t *id_new, uint8_t *acc, float *up_h, uint8_t *up_t)
{
    or_resolve_dyn(W, H, id_old, h_old, word, off_x, off_y, bm, div_bitmap, st, seed, iteration, h_new, id_new,
                   acc, up_h, up_t, NULL, NULL, NULL);
}

/* or_resolve_ex plus, when fric is not NULL, each plate's collision friction of the step: for every
 * arrival at a convergent cell, applyElasticVelocityChange's term (plate_tectonics_kernel.cu:371-394)
 * velocity x coefficient x (source height / plate mass), the coefficient chosen as
 * applyInelasticCollision does (:397-466: continental when a pair with this arrival has type 0,
 * accretion when one has type 3 or 4, else subduction), summed in fixed point (x 2^40) in fric[plate].
 * plates: the records the resolve sees (velocity); dyn: the step's plate masses. */
void or_resolve_dyn(int W, int H, const uint8_t *id_old, const float *h_old, const uint32_t *word,
                    const int32_t *off_x, const int32_t *off_y, const uint8_t *bm, uint32_t *div_bitmap,
                    const tecto_settings *st, uint32_t seed, uint32_t iteration, float *h_new,
                    uint8_t *id_new, uint8_t *acc, float *up_h, uint8_t *up_t, const tecto_plate *plates,
                    const tecto_plate_dynamics *dyn, int64_t *fric)
{
    const tecto_kernel_settings *ks = &st->kernel;
    const size_t N = (size_t)W * (size_t)H;
    uint32_t has_div[TECTO_NUM_DIV_WORDS];
    memset(has_div, 0, sizeof(has_div));
    memset(acc, 0, N);
    static const int PL[6][2] = {{0, 1}, {0, 2}, {1, 2}, {0, 3}, {1, 3}, {2, 3}};

    /* processCollisions (plate_tectonics_kernel.cu:677-745); cells in ascending order, so a later
     * accretion mark overwrites an earlier one exactly as a sequential launch would. */
    for (size_t d = 0; d < N; ++d) {
        const int x = (int)(d % (size_t)W), y = (int)(d / (size_t)W);
        const uint32_t cv = word[d];
        if (cv == 0) {
            /* processDivergence (:301-362) */
            const uint8_t prev = id_old[d];
            const uint32_t opp = cidx(x - off_x[prev], y - off_y[prev], W, H);
            const uint32_t cvo = word[opp];
            const uint8_t oppId = (uint8_t)((255u - cvo) & 0xFFu);
            uint8_t nid;
            if (cvo != 0 && cvo <= 0xFFu && oppId != prev) {
                const uint8_t mn = prev < oppId ? prev : oppId;
                const uint8_t mx = prev < oppId ? oppId : prev;
                const uint32_t bit = tri_index(mn, mx);
                nid = (div_bitmap[bit / 32u] & (1u << (bit % 32u))) ? mn : mx;
                has_div[bit / 32u] |= 1u << (bit % 32u);
            } else {
                nid = prev;
            }
            const float noise = or_simplex3((float)x, (float)y, (float)iteration, 0.01f, (int)seed);
            const float target = ks->divergence_height_target_min +
                                 noise * (ks->divergence_height_target_max -
                                          ks->divergence_height_target_min);
            h_new[d] = or_lerp(h_old[d], target, ks->divergence_interpolation_factor);
            id_new[d] = nid;
            continue;
        }
        uint8_t ids[4];
        for (int k = 0; k < 4; ++k) ids[k] = (uint8_t)(255u - ((cv >> (8 * k)) & 0xFFu));
        if (ids[1] == NPLATE) {
            /* processMovement (:586-609) */
            const uint8_t p = ids[0];
            id_new[d] = p;
            h_new[d] = h_old[cidx(x - off_x[p], y - off_y[p], W, H)];
            continue;
        }
        /* processConvergence (:469-584) */
        const int n = ids[3] != NPLATE ? 4 : ids[2] != NPLATE ? 3 : 2;
        const int pairLen = n == 4 ? 6 : n == 3 ? 3 : 1;
        float heights[4] = {0, 0, 0, 0};
        for (int k = 0; k < n; ++k)
            heights[k] = h_old[cidx(x - off_x[ids[k]], y - off_y[ids[k]], W, H)];
        uint32_t types[6];
        for (int a = 0; a < pairLen; ++a)
            types[a] = pair_type(bm, ids[PL[a][0]], ids[PL[a][1]], heights[PL[a][0]],
                                 heights[PL[a][1]], ks);
        int sub[4] = {0, 0, 0, 0};
        for (int a = 0; a < pairLen; ++a) {
            if (types[a] == 1 || types[a] == 3) sub[PL[a][0]] = 1;
            else if (types[a] == 2 || types[a] == 4) sub[PL[a][1]] = 1;
        }
        if (fric) {
            for (int k = 0; k < n; ++k) {
                int cont = 0, accr = 0;
                for (int a = 0; a < pairLen; ++a) {
                    if (PL[a][0] != k && PL[a][1] != k) continue;
                    if (types[a] == 0) cont = 1;
                    if (types[a] == 3 || types[a] == 4) accr = 1;
                }
                const float coef = cont ? ks->frictionCoefficientContinental
                                        : (accr ? ks->frictionCoefficientAccretion : ks->frictionCoefficientSubduction);
                const float massDiff = heights[k] / dyn[ids[k]].mass;
                const float f = (plates[ids[k]].velocity * coef) * massDiff;
                fric[ids[k]] += tecto_fix(f, OR_FRIC_SCALE, OR_FRIC_LIMIT);
            }
        }
        int owner = 0;
        for (int i = 0; i < n; ++i)
            if (!sub[i]) owner = i;
        const uint8_t ownerId = ids[owner];
        float writeH = heights[owner];
        float hadd = 0.0f;
        uint8_t tbyte = 0;
        for (int a = 0; a < pairLen; ++a) {
            const int ia = PL[a][0], ib = PL[a][1];
            float hh;
            if (ia == owner) hh = heights[ib];
            else if (ib == owner) hh = heights[ia];
            else continue;
            if (hh > writeH) { const float tmp = hh; hh = writeH; writeH = tmp; }
            hadd = hadd + hh;
            const uint32_t t = types[a];
            if (ia == owner)
                tbyte |= (uint8_t)(((t == 2 ? 0 : 1) & 1) | ((ia & 3) << 1) | ((ib & 3) << 3));
            else
                tbyte |= (uint8_t)(((t == 1 ? 0 : 1) & 1) | ((ib & 3) << 1) | ((ia & 3) << 3));
            int other = -1;
            if (ia == owner && t == 4) other = ib;
            else if (ib == owner && t == 3) other = ia;
            if (other >= 0) {
                const uint8_t po = ids[other];
                uint32_t target;
                if (off_x[po] != 0 || off_y[po] != 0)
                    target = cidx(x - off_x[po], y - off_y[po], W, H);
                else
                    target = cidx(x + off_x[ownerId], y + off_y[ownerId], W, H);
                acc[target] = (uint8_t)(255u - ownerId);
            }
        }
        h_new[d] = writeH;
        id_new[d] = ownerId;
        if (up_h) up_h[d] = hadd;
        if (up_t) up_t[d] = tbyte;
    }
    /* flipDivergedBitmap (:772-780) */
    for (int i = 0; i < TECTO_NUM_DIV_WORDS; ++i) div_bitmap[i] ^= has_div[i];

    /* Gaussian uplift: upliftAmount on convergent cells, separable blur (x then y), added. */
    if (st->step.upliftMode == TECTO_UPLIFT_GAUSSIAN) {
        const int r = st->step.upliftRadius;
        float wts[17];
        or_gaussian_weights(st->step.upliftSigma, r, wts);
        const float amount = st->step.upliftAmount;
        float *tmp = (float *)malloc(N * sizeof(float));
#pragma omp parallel for schedule(static)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                float a = 0.0f;
                for (int k = -r; k <= r; ++k) {
                    const float u = word[cidx(x + k, y, W, H)] > 0xFFu ? amount : 0.0f;
                    a = a + wts[k + r] * u;
                }
                tmp[(size_t)y * W + x] = a;
            }
#pragma omp parallel for schedule(static)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                float a = 0.0f;
                for (int k = -r; k <= r; ++k) a = a + wts[k + r] * tmp[cidx(x, y + k, W, H)];
                h_new[(size_t)y * W + x] = h_new[(size_t)y * W + x] + a;
            }
        free(tmp);
    }
}

/* ---- reference uplift: continental propagation, JFA distance field, applyUplift ------------- */

typedef struct {
    int x, y;
} iv2;

/* continentalPropagation (plate_tectonics_kernel.cu:975-1027): march from p against the plate's
 * motion (a DDA over cell edges) while the old height stays at or above continentalPropThreshold;
 * the returned coordinate is not wrapped (heights are read through the torus). */
static iv2 cont_prop(int W, int H, const float *h_old, iv2 p, const tecto_plate *pd, float start,
                     const tecto_kernel_settings *ks)
{
    if (start < ks->continentalPropThreshold) return p;
    const float posx = (float)p.x + pd->pixelCenter_x, posy = (float)p.y + pd->pixelCenter_y;
    const int stepX = -pd->direction_x > 0 ? 1 : -1;
    const int stepY = -pd->direction_y > 0 ? 1 : -1;
    const float tdx = fabsf(1.0f / -pd->direction_x), tdy = fabsf(1.0f / -pd->direction_y);
    const int nextX = stepX > 0 ? p.x + 1 : p.x, nextY = stepY > 0 ? p.y + 1 : p.y;
    float tmx = ((float)nextX - posx) / -pd->direction_x;
    float tmy = ((float)nextY - posy) / -pd->direction_y;
    iv2 prev = p;
    for (int i = 0; i < ks->continentalPropMaxIters; ++i) {
        if (tmx < tmy) {
            p.x += stepX;
            tmx = tmx + tdx;
        } else {
            p.y += stepY;
            tmy = tmy + tdy;
        }
        if (h_old[cidx(p.x, p.y, W, H)] < ks->continentalPropThreshold) return p;
        prev = p;
    }
    return prev;
}

/* atomicInsertPlatePair (:1029-1071) executed alone: both plates (as 255 - id bytes) go into free
 * bytes of the packed word, plates already present are skipped, nothing is written unless both fit. */
static int insert_pair(uint32_t *inv, int a, int b)
{
    uint32_t ins[2] = {255u - (uint32_t)a, 255u - (uint32_t)b};
    const uint32_t old = *inv;
    uint32_t nw = old;
    for (int i = 0; i < 4; ++i) {
        const uint32_t pl = (old >> (8 * i)) & 0xFFu;
        for (int j = 0; j < 2; ++j) {
            if (pl == 0 && ins[j] != 0) {
                nw |= ins[j] << (8 * i);
                ins[j] = 0;
                break;
            }
            if (pl == ins[j]) ins[j] = 0;
        }
    }
    if (ins[0] != 0 || ins[1] != 0) return 0;
    *inv = nw;
    return 1;
}

/* countCollision (:1073-1085) */
static void count_at(iv2 pos, iv2 *positions, int *counts, int *total, int inc)
{
    for (int i = 0; i < 6; ++i)
        if (counts[i] == 0 || (positions[i].x == pos.x && positions[i].y == pos.y)) {
            positions[i] = pos;
            counts[i] += inc;
            *total += inc;
            return;
        }
}

static float subduction_under(float x)
{
    const float v = tecto_log10f(1.0f + 8.0f * (x - 1.0f)) / 1.908485019f - 1.0f;
    return fminf(v, 0.0f);
}

static float continental_profile(float x)
{
    return tecto_expf(-0.02f * x * x) + tecto_expf(-0.2f * x * x) * (0.5f - fabsf(fmodf(fabsf(x), 1.0f) - 0.5f));
}

static int jfa_dist2(int cx, int cy, int seed, int W, int H)
{
    const int sx = seed % W, sy = seed / W;
    int dx = abs(cx - sx), dy = abs(cy - sy);
    dx = dx < W - dx ? dx : W - dx;
    dy = dy < H - dy ? dy : H - dy;
    return dx * dx + dy * dy;
}

/* The reference uplift of one step (plate_tectonic_sim.cu:270-317), every kernel run as one
 * sequential pass in ascending cell order - the canonical order of its atomic inserts and adds:
 * moveContinentalCollisions (:1087-1185), combinePropagatedCollisions (:1187-1218),
 * JFAInitialize / JFAPass / JFAComputeDistance (:1498-1600), applyUplift (:1662-1738).
 * word: this step's arrival words; up_h / up_t: processConvergence's records (valid where the word
 * holds two plates or more); h_old: heights before the step; plates: plate records before their
 * centre update; id_new / h_new: resolved ids and heights, h_new updated in place.  jfa_seed /
 * jfa_dist (optional outputs): the nearest propagated collision cell and its distance, -1 none. */
void or_uplift_ref(int W, int H, const uint32_t *word, const float *up_h, const uint8_t *up_t,
                   const float *h_old, const tecto_plate *plates, const uint8_t *id_new, float *h_new,
                   const tecto_kernel_settings *ks, int32_t *jfa_seed, int32_t *jfa_dist)
{
    const size_t N = (size_t)W * (size_t)H;
    float *ph = (float *)calloc(N, sizeof(float));
    uint32_t *pinv = (uint32_t *)calloc(N, sizeof(uint32_t));
    uint8_t *pt = (uint8_t *)calloc(N, 1);
    int32_t *ja = (int32_t *)malloc(N * sizeof(int32_t));
    int32_t *jb = (int32_t *)malloc(N * sizeof(int32_t));
    /* moveContinentalCollisions */
    for (size_t d = 0; d < N; ++d) {
        const uint32_t cp = word[d];
        if ((cp >> 8) == 0) continue;
        if ((up_t[d] & 1) != 1) continue;
        const int pidx = (up_t[d] >> 1) & 3;
        const int primary = 255 - (int)((cp >> (8 * pidx)) & 0xFFu);
        const iv2 pos = {(int)(d % (size_t)W), (int)(d / (size_t)W)};
        const float cur = h_old[d];
        const iv2 ppos = cont_prop(W, H, h_old, pos, &plates[primary], cur, ks);
        iv2 positions[6];
        int counts[6] = {0, 0, 0, 0, 0, 0}, total = 0;
        for (int k = 0; k < 4; ++k) {
            const int sec = 255 - (int)((cp >> (8 * k)) & 0xFFu);
            if (sec == 255 || sec == primary) continue;
            const iv2 spos = cont_prop(W, H, h_old, pos, &plates[sec], cur, ks);
            if (ppos.x == spos.x && ppos.y == spos.y) {
                if (insert_pair(&pinv[cidx(ppos.x, ppos.y, W, H)], primary, sec))
                    count_at(ppos, positions, counts, &total, 2);
            } else {
                if (insert_pair(&pinv[cidx(ppos.x, ppos.y, W, H)], primary, sec))
                    count_at(ppos, positions, counts, &total, 1);
                if (insert_pair(&pinv[cidx(spos.x, spos.y, W, H)], primary, sec))
                    count_at(spos, positions, counts, &total, 1);
            }
            count_at(ppos, positions, counts, &total, 1);
            count_at(spos, positions, counts, &total, 1);
        }
        for (int i = 0; i < 6; ++i) {
            if (counts[i] == 0) break;
            const uint32_t t = cidx(positions[i].x, positions[i].y, W, H);
            ph[t] = ph[t] + (up_h[d] / (float)total) * (float)counts[i];
        }
    }
    /* combinePropagatedCollisions (cells without two plates never become JFA seeds, so their
     * non-seed record is taken as is) */
    for (size_t d = 0; d < N; ++d) {
        if (pinv[d] != 0) {
            pt[d] = 1;
        } else if ((word[d] >> 8) != 0) {
            if ((up_t[d] & 1) == 0) {
                pt[d] = up_t[d];
                ph[d] = up_h[d];
                pinv[d] = word[d];
            } else {
                pinv[d] = 1;
            }
        } else {
            pinv[d] = word[d];
        }
    }
    /* JFAInitialize */
    for (size_t d = 0; d < N; ++d) ja[d] = (pinv[d] >> 8) != 0 ? (int32_t)d : -1;
    /* JFAPass, steps from the largest power of two below max(W, H) down to 1 */
    const int maxDim = W > H ? W : H;
    int step = 1;
    while (step < maxDim) step <<= 1;
    step >>= 1;
    while (step > 0) {
#pragma omp parallel for schedule(static)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const size_t d = (size_t)y * W + x;
                int best = ja[d], bestDist = 0x7FFFFFFF;
                if (best >= 0) bestDist = jfa_dist2(x, y, best, W, H);
                for (int oy = -1; oy <= 1; ++oy)
                    for (int ox = -1; ox <= 1; ++ox) {
                        if (ox == 0 && oy == 0) continue;
                        const int cand = ja[cidx(x + ox * step, y + oy * step, W, H)];
                        if (cand < 0) continue;
                        const int dist = jfa_dist2(x, y, cand, W, H);
                        if (dist < bestDist) {
                            bestDist = dist;
                            best = cand;
                        }
                    }
                jb[d] = best;
            }
        int32_t *tmp = ja;
        ja = jb;
        jb = tmp;
        step >>= 1;
    }
    /* JFAComputeDistance + applyUplift */
    for (size_t d = 0; d < N; ++d) {
        const int x = (int)(d % (size_t)W), y = (int)(d / (size_t)W);
        const int seed = ja[d];
        int dist = -1;
        uint32_t orig = 0;
        if (seed >= 0) {
            dist = (int)sqrtf((float)jfa_dist2(x, y, seed, W, H));
            orig = (uint32_t)seed;
        }
        if (jfa_seed) jfa_seed[d] = seed;
        if (jfa_dist) jfa_dist[d] = dist;
        if (dist <= -1) continue;
        const uint8_t ct = pt[orig];
        const uint32_t inv = pinv[orig];
        const int type = ct & 1, pi = (ct >> 1) & 3, si = (ct >> 3) & 3;
        const int prim = 255 - (int)((inv >> (8 * pi)) & 0xFFu);
        const int secp = 255 - (int)((inv >> (8 * si)) & 0xFFu);
        const int plate = id_new[d];
        if (type == 0 && secp == plate) {
            const float value = subduction_under((float)dist);
            const float mult = 1.0f + value * ks->subductionUnderUpliftMultiplier;
            h_new[d] = fmaxf(h_new[d] * mult, ks->minUpliftClamp);
        } else if (type == 0 && prim == plate) {
            const int ox = (int)(orig % (uint32_t)W), oy = (int)(orig / (uint32_t)W);
            const float sx = (float)W, sy = (float)H;
            const float ddx = fmodf((float)(x - ox) + sx * 0.5f, sx) - sx * 0.5f;
            const float ddy = fmodf((float)(y - oy) + sy * 0.5f, sy) - sy * 0.5f;
            float mag = sqrtf(ddx * ddx + ddy * ddy);
            mag = fmaxf(mag, 1e-20f);
            const float dirx = ddx / mag, diry = ddy / mag;
            /* plate 255 (an empty slot named by merged type bits) has no record: zero direction */
            const float odx = secp < 255 ? plates[secp].direction_x : 0.0f;
            const float ody = secp < 255 ? plates[secp].direction_y : 0.0f;
            const float dot = fmaxf(dirx * odx + diry * ody, 0.0f);
            const float value = continental_profile(((float)dist - (float)ks->subductionOverRange) - 10.0f);
            const float mult = 1.0f + (value * dot) * ks->subductionOverUpliftMultiplier;
            h_new[d] = fmaxf(h_new[d] * mult, ks->minUpliftClamp);
        } else if (type == 1) {
            const float height = ph[orig];
            const float value = continental_profile((float)dist);
            const float change = (value * height) * ks->continentalUpliftMultiplier;
            h_new[d] = fminf(h_new[d] + change, ks->maxUpliftClamp);
        }
    }
    free(ph);
    free(pinv);
    free(pt);
    free(ja);
    free(jb);
}

/* ---- thermal ------------------------------------------------------------------------------- */

static const int TH_DX[8] = {-1, 1, 0, 0, -1, -1, 1, 1};
static const int TH_DY[8] = {0, 0, -1, 1, -1, 1, -1, 1};

/* thermalErosionKernel (plate_tectonics_kernel.cu:2735-2786) in gather form. */
void or_thermal(int W, int H, float *h, int iters, const tecto_kernel_settings *ks)
{
    const size_t N = (size_t)W * (size_t)H;
    const float thr = ks->thermalThresholdAngle * ks->thermalCellSize;
    const float A = ks->thermalErosionAmplitude, S = ks->thermalErosionStrength;
    float *tot = (float *)malloc(N * sizeof(float));
    float *hn = (float *)malloc(N * sizeof(float));
    for (int it = 0; it < iters; ++it) {
#pragma omp parallel for schedule(static)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const float hc = h[(size_t)y * W + x];
                float t = 0.0f;
                for (int d = 0; d < 8; ++d) {
                    const float diff = hc - h[cidx(x + TH_DX[d], y + TH_DY[d], W, H)];
                    if (diff > thr) t = t + diff;
                }
                tot[(size_t)y * W + x] = t;
            }
#pragma omp parallel for schedule(static)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const size_t i = (size_t)y * W + x;
                const float hc = h[i];
                float v = hc;
                /* a flow that evaluates to exactly zero moves nothing and is skipped */
                if (tot[i] > 0.0f)
                    for (int d = 0; d < 8; ++d) {
                        const float diff = hc - h[cidx(x + TH_DX[d], y + TH_DY[d], W, H)];
                        if (diff > thr) {
                            const float f = (A * (diff / tot[i])) * S;
                            if (f != 0.0f) v = v - f;
                        }
                    }
                for (int d = 0; d < 8; ++d) {
                    const uint32_t nb = cidx(x + TH_DX[d], y + TH_DY[d], W, H);
                    const float diff = h[nb] - hc;
                    if (diff > thr && tot[nb] > 0.0f) {
                        const float f = (A * (diff / tot[nb])) * S;
                        if (f != 0.0f) v = v + f;
                    }
                }
                hn[i] = v;
            }
        memcpy(h, hn, N * sizeof(float));
    }
    free(tot);
    free(hn);
}

/* ---- hydraulic ----------------------------------------------------------------------------- */

/* applyHydraulicErosion (plate_tectonic_sim.cu:331-373): per sub-iteration rain, flux, flow,
 * sediment (slope from a copy of the height), transport, evaporate; kernels at
 * plate_tectonics_kernel.cu:2430-2593. */
void or_hydraulic(int W, int H, float *h, float *w, float *s, float *flux, int iters, float dt,
                  uint32_t rain_seed, const tecto_kernel_settings *ks)
{
    const size_t N = (size_t)W * (size_t)H;
    float *fl = (float *)malloc(N * 4 * sizeof(float));  /* new flux */
    float *vx = (float *)malloc(N * sizeof(float));
    float *vy = (float *)malloc(N * sizeof(float));
    float *hc = (float *)malloc(N * sizeof(float));       /* height copy */
    float *s2 = (float *)malloc(N * sizeof(float));
    const int seed = (int)rain_seed;
    const float A = ks->hydrationPipeCrossSection, L = ks->hydrationPipeLength, G = ks->gravity;
    for (int it = 0; it < iters; ++it) {
        /* rain (:2430-2437) */
#pragma omp parallel for schedule(static)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const size_t i = (size_t)y * W + x;
                w[i] = w[i] + (fmaxf(0.0f, or_rain_noise(x, y, seed)) * dt) * ks->hydrationRainfall;
            }
        /* flux (:2439-2485) */
#pragma omp parallel for schedule(static)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const size_t i = (size_t)y * W + x;
                const int nx[4] = {x - 1, x, x + 1, x};
                const int ny[4] = {y, y + 1, y, y - 1};
                float o[4];
                for (int k = 0; k < 4; ++k) {
                    const uint32_t n = cidx(nx[k], ny[k], W, H);
                    const float dh = ((h[i] + w[i]) - h[n]) - w[n];
                    o[k] = fmaxf(0.0f, flux[4 * i + k] + (dt * A) * ((G * dh) / L));
                }
                const float total = (((o[0] + o[1]) + o[2]) + o[3]) + 1e-6f;
                float K = fminf(1.0f, w[i] / (total * dt + 1e-6f));
                K = fmaxf(K, 0.01f);
                for (int k = 0; k < 4; ++k) fl[4 * i + k] = o[k] * K;
            }
        /* flow (:2487-2533); the flux texture is replaced by the new flux */
#pragma omp parallel for schedule(static)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const size_t i = (size_t)y * W + x;
                const float *fL = fl + 4 * (size_t)cidx(x - 1, y, W, H);
                const float *fU = fl + 4 * (size_t)cidx(x, y + 1, W, H);
                const float *fR = fl + 4 * (size_t)cidx(x + 1, y, W, H);
                const float *fD = fl + 4 * (size_t)cidx(x, y - 1, W, H);
                const float *fC = fl + 4 * i;
                float in = 0.0f;
                in = in + fL[2];
                in = in + fU[3];
                in = in + fR[0];
                in = in + fD[1];
                const float out = ((fC[0] + fC[1]) + fC[2]) + fC[3];
                const float dv = dt * (in - out);
                const float wn = fmaxf(0.0f, w[i] + dv);
                w[i] = wn;
                const float nfx = (((fL[2] - fC[0]) + fC[2]) - fR[0]) * 0.5f;
                const float nfy = (((fU[3] - fC[1]) + fC[1]) - fD[3]) * 0.5f;
                const float hh = fmaxf(wn, 0.01f);
                float ux = nfx / hh, uy = nfy / hh;
                const float mag = sqrtf(ux * ux + uy * uy);
                if (mag > 50.0f) {
                    const float sc = 50.0f / mag;
                    ux = ux * sc;
                    uy = uy * sc;
                }
                vx[i] = ux;
                vy[i] = uy;
            }
        memcpy(flux, fl, N * 4 * sizeof(float));
        memcpy(hc, h, N * sizeof(float));
        /* sediment (:2535-2570), slope of the height copy (cuda_texture.cuh:78-89) */
#pragma omp parallel for schedule(static)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const size_t i = (size_t)y * W + x;
                const float dzdx = (hc[cidx(x + 1, y, W, H)] - hc[cidx(x - 1, y, W, H)]) * 0.5f;
                const float dzdy = (hc[cidx(x, y + 1, W, H)] - hc[cidx(x, y - 1, W, H)]) * 0.5f;
                const float slope = sqrtf(dzdx * dzdx + dzdy * dzdy);
                const float mag = sqrtf(vx[i] * vx[i] + vy[i] * vy[i]);
                float C = (ks->sedimentCapacity * or_sinf(fmaxf(slope, 0.03f))) * mag;
                C = fminf(C, 5.0f);
                const float sd = s[i];
                if (C > sd) {
                    float e = (ks->sedimentErosionRate * (C - sd)) * dt;
                    e = fminf(e, hc[i]);
                    h[i] = hc[i] - e;
                    s[i] = sd + e;
                } else {
                    float dd = (ks->sedimentDepositionRate * (sd - C)) * dt;
                    dd = fminf(dd, sd);
                    s[i] = sd - dd;
                    h[i] = hc[i] + dd;
                }
            }
        /* transport (:2572-2585): bilinear sample with wrap (cuda_helper.cuh:48-65) */
#pragma omp parallel for schedule(static)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const size_t i = (size_t)y * W + x;
                const float px = (float)x - vx[i] * dt;
                const float py = (float)y - vy[i] * dt;
                const int x0 = (int)floorf(px), y0 = (int)floorf(py);
                const int x1 = x0 + 1, y1 = y0 + 1;
                const float wx = px - (float)x0, wy = py - (float)y0;
                const float I0 = (1.0f - wx) * s[cidx(x0, y0, W, H)] + wx * s[cidx(x1, y0, W, H)];
                const float I1 = (1.0f - wx) * s[cidx(x0, y1, W, H)] + wx * s[cidx(x1, y1, W, H)];
                s2[i] = (1.0f - wy) * I0 + wy * I1;
            }
        memcpy(s, s2, N * sizeof(float));
        /* evaporate (:2587-2593) */
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < N; ++i)
            w[i] = fmaxf(0.0f, w[i] - (fminf(w[i], 20.0f) * ks->hydrationEvaporation) * dt);
    }
    free(fl);
    free(vx);
    free(vy);
    free(hc);
    free(s2);
}

/* ---- accretion ------------------------------------------------------------------------------ */

/* applyAccretion (plate_tectonics_kernel.cu:747-770) */
void or_accretion(int W, int H, const float *h, const uint8_t *acc, uint8_t *id,
                  const tecto_kernel_settings *ks)
{
    const size_t N = (size_t)W * (size_t)H;
    for (size_t i = 0; i < N; ++i) {
        const uint8_t a = (uint8_t)(255u - acc[i]);
        if (a == NPLATE) continue;
        if (h[i] >= ks->continentalCrustThreshold) id[i] = a;
    }
}

/* ---- CCL ------------------------------------------------------------------------------------ */

static uint32_t uf_find(uint32_t *p, uint32_t a)
{
    while (p[a] != a) {
        p[a] = p[p[a]];
        a = p[a];
    }
    return a;
}

static void uf_union(uint32_t *p, uint32_t a, uint32_t b)
{
    a = uf_find(p, a);
    b = uf_find(p, b);
    if (a < b) p[b] = a;
    else if (b < a) p[a] = b;
}

/* Connected components of equal plate id on the torus (ccl.cu:35-177).  Modes 4 and 8 are the
 * true 4- and 8-neighbourhoods; TECTO_CCL_REF8 is the union set the reference's kernels build:
 * init's single link to the first equal of (tl, t, tr, l) (ccl.cu:107-116), reduce's l and tl
 * unions on every row and t and tr unions on row 0 (ccl.cu:157-176).  Labels = minimum index. */
void or_ccl(int W, int H, const uint8_t *id, uint32_t *labels, int mode)
{
    const size_t N = (size_t)W * (size_t)H;
    for (size_t i = 0; i < N; ++i) labels[i] = (uint32_t)i;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const uint32_t i = (uint32_t)((size_t)y * W + x);
            const uint8_t c = id[i];
            const uint32_t l = cidx(x - 1, y, W, H), t = cidx(x, y - 1, W, H);
            const uint32_t tl = cidx(x - 1, y - 1, W, H), tr = cidx(x + 1, y - 1, W, H);
            if (mode == TECTO_CCL_4) {
                if (id[l] == c) uf_union(labels, i, l);
                if (id[t] == c) uf_union(labels, i, t);
            } else if (mode == TECTO_CCL_8) {
                if (id[l] == c) uf_union(labels, i, l);
                if (id[t] == c) uf_union(labels, i, t);
                if (id[tl] == c) uf_union(labels, i, tl);
                if (id[tr] == c) uf_union(labels, i, tr);
            } else {
                if (id[tl] == c) uf_union(labels, i, tl);
                else if (id[t] == c) uf_union(labels, i, t);
                else if (id[tr] == c) uf_union(labels, i, tr);
                else if (id[l] == c) uf_union(labels, i, l);
                if (y == 0) {
                    if (id[t] == c) uf_union(labels, i, t);
                    if (id[tr] == c) uf_union(labels, i, tr);
                }
                if (id[tl] == c) uf_union(labels, i, tl);
                if (id[l] == c) uf_union(labels, i, l);
            }
        }
    for (size_t i = 0; i < N; ++i) labels[i] = uf_find(labels, (uint32_t)i);
}

/* ---- full step ---------------------------------------------------------------------------- */

/* PlateTectonicSim::executeIteration (plate_tectonic_sim.cu:54-131), hot-path phases. */
/* ---- plate dynamics ------------------------------------------------------------------------- */

/* The per-plate values a step starts from: mass (sum of heights) and size over all cells, as
 * mergeAndCountSizeMass leaves them without merges (plate_tectonics_kernel.cu:100-195), and the
 * geometric centre of accumulatePlateAngularCoords / calculatePlateCenters (:2154-2226): the cells
 * whose x and y are multiples of 10 contribute sin and cos of their angle around each axis, the
 * means go back to a cell coordinate through atan2.  The sums are exact fixed-point sums (mass x 2^16,
 * angular terms x 2^32).  Iteration 0 keeps the stored centre (the reference computes the first one
 * at the end of its first iteration). */
void or_plate_stats(int W, int H, const float *h, const uint8_t *id, uint32_t iteration,
                    tecto_plate_dynamics *dyn)
{
    int64_t mass[NPLATE], ang[NPLATE][4];
    int size[NPLATE], samples[NPLATE];
    memset(mass, 0, sizeof(mass));
    memset(ang, 0, sizeof(ang));
    memset(size, 0, sizeof(size));
    memset(samples, 0, sizeof(samples));
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t d = (size_t)y * (size_t)W + (size_t)x;
            const unsigned p = id[d];
            if (p >= NPLATE) continue;
            mass[p] += tecto_fix(h[d], OR_MASS_SCALE, OR_MASS_LIMIT);
            size[p] += 1;
            if (x % 10 == 0 && y % 10 == 0) {
                const float ax = (OR_TWO_PI_F * (float)x) / (float)W;
                const float ay = (OR_TWO_PI_F * (float)y) / (float)H;
                ang[p][0] += tecto_fix(tecto_sinf(ax), OR_ANG_SCALE, 1.0f);
                ang[p][1] += tecto_fix(tecto_cosf(ax), OR_ANG_SCALE, 1.0f);
                ang[p][2] += tecto_fix(tecto_sinf(ay), OR_ANG_SCALE, 1.0f);
                ang[p][3] += tecto_fix(tecto_cosf(ay), OR_ANG_SCALE, 1.0f);
                samples[p] += 1;
            }
        }
    for (unsigned p = 0; p < NPLATE; ++p) {
        dyn[p].mass = tecto_unfix(mass[p], 1.0 / (double)OR_MASS_SCALE);
        dyn[p].size = size[p];
        if (samples[p] > 0 && iteration > 0) {
            const float n = (float)samples[p];
            const float sx = tecto_unfix(ang[p][0], 1.0 / (double)OR_ANG_SCALE) / n;
            const float cx = tecto_unfix(ang[p][1], 1.0 / (double)OR_ANG_SCALE) / n;
            const float sy = tecto_unfix(ang[p][2], 1.0 / (double)OR_ANG_SCALE) / n;
            const float cy = tecto_unfix(ang[p][3], 1.0 / (double)OR_ANG_SCALE) / n;
            float gx = tecto_atan2f(sx, cx) * (float)W / OR_TWO_PI_F;
            float gy = tecto_atan2f(sy, cy) * (float)H / OR_TWO_PI_F;
            if (gx < 0.0f) gx += (float)W;
            if (gy < 0.0f) gy += (float)H;
            dyn[p].geometricCenter_x = gx;
            dyn[p].geometricCenter_y = gy;
        }
    }
}

static int wrap_i(int v, int n)
{
    const int r = v % n;
    return r < 0 ? r + n : r;
}

/* computeCurl (plate_tectonics_kernel.cu:2788-2822) at world cell (cx, cy): the pressure texture
 * (pw x ph) sampled nearest at (cx * pw / W, cy * ph / H), its central differences rotated. */
void or_curl_at(const float *pr, int pw, int ph, int W, int H, int cx, int cy, float *out_x, float *out_y)
{
    const double xs = (double)pw / (double)W, ys = (double)ph / (double)H;
    const int qx = (int)((double)cx * xs), qy = (int)((double)cy * ys);
    const float left = pr[(size_t)qy * pw + wrap_i(qx - 1, pw)];
    const float right = pr[(size_t)qy * pw + wrap_i(qx + 1, pw)];
    const float bottom = pr[(size_t)wrap_i(qy - 1, ph) * pw + qx];
    const float top = pr[(size_t)wrap_i(qy + 1, ph) * pw + qx];
    *out_y = (float)((double)(right - left) * 0.5);
    *out_x = (float)(-((double)(top - bottom) * 0.5));
}

/* applyPlateMovementChanges (plate_tectonics_kernel.cu:1863-1925) for velocity, direction,
 * smoothing and the merge wait (the sub-cell centre update is or_plate_offsets'): the velocity
 * loses the friction fric[k] (fixed point x 2^40), then drag pulls it towards the asthenosphere flow,
 * the curl of the pressure texture at the plate's geometric centre (zero without a texture),
 * offset by 0.2 away from zero and clamped to [-1, 1]. */
void or_plate_motion(int W, int H, tecto_plate *plates, tecto_plate_dynamics *dyn, const int64_t *fric,
                     const float *pressure, int pw, int ph, const tecto_kernel_settings *ks)
{
    for (unsigned k = 0; k < NPLATE; ++k) {
        tecto_plate *p = &plates[k];
        tecto_plate_dynamics *dd = &dyn[k];
        const float friction = tecto_unfix(fric[k], 1.0 / (double)OR_FRIC_SCALE);
        float sx = 0.0f, sy = 0.0f;
        if (pressure) {
            const float gx = fminf(fmaxf(dd->geometricCenter_x + 0.5f, -1073741824.0f), 1073741824.0f);
            const float gy = fminf(fmaxf(dd->geometricCenter_y + 0.5f, -1073741824.0f), 1073741824.0f);
            or_curl_at(pressure, pw, ph, W, H, wrap_i((int)gx, W), wrap_i((int)gy, H), &sx, &sy);
        }
        const float avx = fmaxf(fminf((float)((double)(sx * ks->curlNoiseMultiplier) + (sx < 0.0f ? -0.2 : 0.2)), 1.0f), -1.0f);
        const float avy = fmaxf(fminf((float)((double)(sy * ks->curlNoiseMultiplier) + (sy < 0.0f ? -0.2 : 0.2)), 1.0f), -1.0f);
        const float ox = p->direction_x * p->velocity, oy = p->direction_y * p->velocity;
        const float mag = fmaxf(sqrtf(ox * ox + oy * oy), 1e-20f);
        const float post = fmaxf(mag - friction, 0.0f);
        const float vx = p->direction_x * post, vy = p->direction_y * post;
        const float rx = avx - vx, ry = avy - vy;
        const float rmag = sqrtf(rx * rx + ry * ry);
        const float drag = ks->environmentalDragCoefficient * rmag * rmag;
        const float rn = fmaxf(sqrtf(rx * rx + ry * ry), 1e-20f);
        const float nx = vx + (rx / rn) * drag, ny = vy + (ry / rn) * drag;
        const float nm = fmaxf(sqrtf(nx * nx + ny * ny), 1e-20f);
        p->velocity = nm;
        p->direction_x = nx / nm;
        p->direction_y = ny / nm;
        const float vs = ks->velocitySmoothingFactor, ds = ks->directionSmoothingFactor;
        dd->velocitySmoothed = dd->velocitySmoothed * vs + p->velocity * (1.0f - vs);
        const float sdx = dd->directionSmoothed_x * ds + p->direction_x * (1.0f - ds);
        const float sdy = dd->directionSmoothed_y * ds + p->direction_y * (1.0f - ds);
        const float sm = fmaxf(sqrtf(sdx * sdx + sdy * sdy), 1e-20f);
        dd->directionSmoothed_x = sdx / sm;
        dd->directionSmoothed_y = sdy / sm;
        dd->mergeWaitTime = dd->mergeWaitTime > 0 ? dd->mergeWaitTime - 1 : 0;
        dd->frictionLoss = friction;
    }
}

void or_step(int W, int H, float *h, float *w, float *s, float *flux, uint8_t *id, uint32_t *labels,
             uint32_t *word, uint8_t *acc, uint8_t *bm, uint32_t *div_bitmap, tecto_plate *plates,
             const tecto_settings *st, uint32_t seed, uint32_t *iteration)
{
    or_step_dyn(W, H, h, w, s, flux, id, labels, word, acc, bm, div_bitmap, plates, NULL, NULL, 0, 0, st, seed,
                iteration);
}

/* or_step with plate dynamics when st->step.plateDynamics is TECTO_PLATE_DYNAMICS_REFERENCE: dyn
 * holds the plate dynamics records, pressure (pw x ph, or NULL) the asthenosphere texture. */
void or_step_dyn(int W, int H, float *h, float *w, float *s, float *flux, uint8_t *id, uint32_t *labels,
                 uint32_t *word, uint8_t *acc, uint8_t *bm, uint32_t *div_bitmap, tecto_plate *plates,
                 tecto_plate_dynamics *dyn, const float *pressure, int pw, int ph, const tecto_settings *st,
                 uint32_t seed, uint32_t *iteration)
{
    const size_t N = (size_t)W * (size_t)H;
    int32_t offx[NPLATE], offy[NPLATE];
    tecto_plate next[NPLATE];
    or_plate_offsets(plates, offx, offy, next);
    or_collision_words(W, H, id, offx, offy, NULL, word, NULL, NULL);
    or_collision_types(W, H, word, h, offx, offy, &st->kernel, bm);
    float *hn = (float *)malloc(N * sizeof(float));
    uint8_t *idn = (uint8_t *)malloc(N);
    const int dynamics = dyn && st->step.plateDynamics == TECTO_PLATE_DYNAMICS_REFERENCE;
    const int policy = dyn ? st->step.platePolicy & (TECTO_PLATE_RELABEL | TECTO_PLATE_MERGE) : 0;
    int64_t fric[NPLATE];
    memset(fric, 0, sizeof(fric));
    if (dynamics || policy) or_plate_stats(W, H, h, id, *iteration, dyn);
    float *uh = NULL;
    uint8_t *ut = NULL;
    if (st->step.upliftMode == TECTO_UPLIFT_REFERENCE) {
        uh = (float *)calloc(N, sizeof(float));
        ut = (uint8_t *)calloc(N, 1);
    }
    or_resolve_dyn(W, H, id, h, word, offx, offy, bm, div_bitmap, st, seed, *iteration, hn, idn, acc, uh, ut,
                   plates, dyn, dynamics ? fric : NULL);
    if (st->step.upliftMode == TECTO_UPLIFT_REFERENCE) {
        or_uplift_ref(W, H, word, uh, ut, h, plates, idn, hn, &st->kernel, NULL, NULL);
        free(uh);
        free(ut);
    }
    memcpy(h, hn, N * sizeof(float));
    memcpy(id, idn, N);
    free(hn);
    free(idn);
    or_thermal(W, H, h, st->step.thermalIterations, &st->kernel);
    or_hydraulic(W, H, h, w, s, flux, st->step.hydraulicIterations, st->step.hydraulicDt,
                 seed + *iteration, &st->kernel);
    memcpy(plates, next, sizeof(next));
    if (dynamics) or_plate_motion(W, H, plates, dyn, fric, pressure, pw, ph, &st->kernel);
    or_accretion(W, H, h, acc, id, &st->kernel);
    const int period = st->sim.iterationsForCCL > 0 ? st->sim.iterationsForCCL : 1;
    const int ccl_due = *iteration % (uint32_t)period == 0;
    if (ccl_due) or_ccl(W, H, id, labels, st->step.cclConnectivity);
    if (ccl_due && (policy & TECTO_PLATE_RELABEL))
        or_relabel(W, H, id, labels, plates, dyn, st->kernel.minPlateSize);
    if (policy & TECTO_PLATE_MERGE) or_merge(W, H, id, plates, dyn, bm, &st->kernel);
    *iteration += 1;
}

/* ---- image export ------------------------------------------------------------------------------ */

/* convertFloatToGray16Kernel, texture_save.cu:80-96. */
void or_gray16(size_t n, const float *h, float minv, float maxv, uint16_t *out)
{
    for (size_t i = 0; i < n; ++i) {
        float norm = (h[i] - minv) / (maxv - minv);
        norm = fminf(fmaxf(norm, 0.0f), 1.0f);
        out[i] = (uint16_t)(norm * 65535.0f);
    }
}

/* convertGrayscaleToRgbKernel, texture_save.cu:16-70: hue steps of 1/8 by id mod 8 plus a small
 * offset by id / 8, saturation and value oscillating with sin / cos of id * 0.1, the standard HSV
 * to RGB sectors (compared in double, as the reference's literals are), rounded to the nearest
 * byte; id 255 is the background (230, 235, 240). */
void or_plate_palette(uint8_t *rgb768)
{
    for (int val = 0; val < 256; ++val) {
        uint8_t *o = rgb768 + 3 * val;
        if (val == 255) {
            o[0] = 230;
            o[1] = 235;
            o[2] = 240;
            continue;
        }
        const float hue = 0.125f * (float)(val % 8) + (float)val / 8.0f / 256.0f;
        const float sat = 0.5f + 0.5f * sinf((float)val * 0.1f);
        const float v = 0.5f + 0.5f * cosf((float)val * 0.1f);
        const float c = v * sat;
        const float x = c * (1.0f - fabsf(fmodf(hue * 6.0f, 2.0f) - 1.0f));
        const float m = v - c;
        const double hd = hue;
        float r, g, b;
        if (hd < 1.0 / 6.0) { r = c; g = x; b = 0.0f; }
        else if (hd < 2.0 / 6.0) { r = x; g = c; b = 0.0f; }
        else if (hd < 3.0 / 6.0) { r = 0.0f; g = c; b = x; }
        else if (hd < 4.0 / 6.0) { r = 0.0f; g = x; b = c; }
        else if (hd < 5.0 / 6.0) { r = x; g = 0.0f; b = c; }
        else { r = c; g = 0.0f; b = x; }
        o[0] = (uint8_t)lroundf((r + m) * 255.0f);
        o[1] = (uint8_t)lroundf((g + m) * 255.0f);
        o[2] = (uint8_t)lroundf((b + m) * 255.0f);
    }
}

/* ---- the reference's world initialisation ---------------------------------------------------- */

/* std::default_random_engine as libstdc++ defines it (minstd_rand0: x <- 16807 x mod 2^31 - 1, a seed
 * that is 0 mod the modulus becomes 1) and std::uniform_real_distribution<float> on it: one draw of
 * generate_canonical<float, 24> (the engine spans 31 bits, so a single call: (x - 1) / (float)(2^31 - 2),
 * the divisor rounding to 2^31, results of 1 pulled below 1), scaled to [a, b) as u * (b - a) + a. */
typedef struct {
    uint64_t x;
} or_minstd;

static void minstd_seed(or_minstd *g, uint64_t s)
{
    const uint64_t r = s % 2147483647u;
    g->x = r == 0 ? 1u : r;
}

static float minstd_uniform(or_minstd *g, float a, float b)
{
    g->x = (g->x * 16807u) % 2147483647u;
    const float sum = (float)(g->x - 1u) * 1.0f;
    float u = sum / 2147483648.0f;
    if (u >= 1.0f) u = nextafterf(1.0f, 0.0f);
    return (u * (b - a)) + a;
}

/* PlateTectonicSim::initializeTectonics' host part (plate_tectonic_sim.cu:705-745):
 * generatePlateCenters (:873-890), the generations of generateVoronoiSeeds (:892-929) and
 * generatePlateData (:816-842).  Positions are drawn as {height range, width range}, as the
 * reference does.  Returns 0, or -1 for invalid arguments or too small a capacity. */
int or_reference_seeds(int W, int H, uint32_t seed, int numPlates, const int *gens, int ngens, float *seed_x,
                       float *seed_y, uint8_t *seed_id, int capacity, int *count, tecto_plate *plates,
                       tecto_plate_dynamics *dyn)
{
    if (numPlates < 1 || numPlates > (int)NPLATE || ngens < 0 || ngens > TECTO_MAX_VORONOI_GENS) return -1;
    int maxn = numPlates;
    for (int g = 0; g < ngens; ++g) {
        if (gens[g] < 0 || gens[g] > (1 << 20)) return -1;
        if (gens[g] > maxn) maxn = gens[g];
    }
    or_minstd rng;
    minstd_seed(&rng, seed);
    float *cx = (float *)malloc(sizeof(float) * (size_t)numPlates), *cy = (float *)malloc(sizeof(float) * (size_t)numPlates);
    float *px = (float *)malloc(sizeof(float) * (size_t)maxn), *py = (float *)malloc(sizeof(float) * (size_t)maxn);
    float *nx = (float *)malloc(sizeof(float) * (size_t)maxn), *ny = (float *)malloc(sizeof(float) * (size_t)maxn);
    int *pid = (int *)malloc(sizeof(int) * (size_t)maxn), *nid = (int *)malloc(sizeof(int) * (size_t)maxn);
    for (int i = 0; i < numPlates; ++i) {
        cx[i] = minstd_uniform(&rng, 0.0f, (float)H);
        cy[i] = minstd_uniform(&rng, 0.0f, (float)W);
        px[i] = cx[i];
        py[i] = cy[i];
        pid[i] = i;
    }
    int n = numPlates;
    for (int g = 0; g < ngens; ++g) {
        for (int i = 0; i < gens[g]; ++i) {
            const float sx = minstd_uniform(&rng, 0.0f, (float)H);
            const float sy = minstd_uniform(&rng, 0.0f, (float)W);
            float best = 3.40282347e38f;
            int id = 0;
            for (int c = 0; c < n; ++c) {
                const float dx = fabsf(sx - px[c]), dy = fabsf(sy - py[c]);
                const float wx = fminf(dx, (float)W - dx), wy = fminf(dy, (float)H - dy);
                const float d2 = wx * wx + wy * wy;
                if (d2 < best) {
                    id = pid[c];
                    best = d2;
                }
            }
            nx[i] = sx;
            ny[i] = sy;
            nid[i] = id;
        }
        n = gens[g];
        memcpy(px, nx, sizeof(float) * (size_t)n);
        memcpy(py, ny, sizeof(float) * (size_t)n);
        memcpy(pid, nid, sizeof(int) * (size_t)n);
    }
    if (n < numPlates) {
        n = numPlates;
        for (int i = 0; i < n; ++i) {
            px[i] = cx[i];
            py[i] = cy[i];
            pid[i] = i;
        }
    }
    int rc = 0;
    *count = n;
    if (seed_x || seed_y || seed_id) {
        if (capacity < n) rc = -1;
        else
            for (int i = 0; i < n; ++i) {
                if (seed_x) seed_x[i] = px[i];
                if (seed_y) seed_y[i] = py[i];
                if (seed_id) seed_id[i] = (uint8_t)pid[i];
            }
    }
    if (plates) memset(plates, 0, sizeof(tecto_plate) * NPLATE);
    if (dyn) memset(dyn, 0, sizeof(tecto_plate_dynamics) * NPLATE);
    for (int i = 0; i < numPlates; ++i) {
        const float v = (minstd_uniform(&rng, -1.0f, 1.0f) + 1.0f) / 2.0f;
        const float xd = minstd_uniform(&rng, -1.0f, 1.0f);
        const float yd = minstd_uniform(&rng, -1.0f, 1.0f);
        const float m = sqrtf(xd * xd + yd * yd);
        if (plates) {
            plates[i].pixelCenter_x = cx[i] - floorf(cx[i]);
            plates[i].pixelCenter_y = cy[i] - floorf(cy[i]);
            plates[i].velocity = v;
            plates[i].direction_x = xd / m;
            plates[i].direction_y = yd / m;
        }
        if (dyn) {
            dyn[i].velocitySmoothed = v;
            dyn[i].directionSmoothed_x = xd / m;
            dyn[i].directionSmoothed_y = yd / m;
        }
    }
    free(cx); free(cy); free(px); free(py); free(nx); free(ny); free(pid); free(nid);
    return rc;
}

/* initPlateIDs (plate_tectonics_kernel.cu:31-63): the first seed at the minimum wrapped squared
 * distance; initHeightmap (:65-99): four octaves of simplex noise at frequencies 0.01 x 10^k with
 * amplitudes 0.9 x 0.1^k, each remapped from [-1, 1] to [0, 1] after damping by 1 + |gradient|
 * (forward differences at 0.001 cells), scaled to 5000..15000. */
void or_init_reference(int W, int H, uint32_t seed, const float *sx, const float *sy, const uint8_t *sid, int S,
                       float *h, uint8_t *id)
{
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t i = (size_t)y * (size_t)W + (size_t)x;
            const float fx = (float)x, fy = (float)y;
            float best = 3.40282347e38f;
            int plate = 0;
            for (int k = 0; k < S; ++k) {
                const float dx = fabsf(fx - sx[k]), dy = fabsf(fy - sy[k]);
                const float wx = fminf(dx, (float)W - dx), wy = fminf(dy, (float)H - dy);
                const float d2 = wx * wx + wy * wy;
                if (d2 < best) {
                    plate = sid[k];
                    best = d2;
                }
            }
            id[i] = (uint8_t)plate;
            const float d = 0.001f;
            float value = 0.0f, amp = 0.9f, freq = 0.01f;
            for (int octave = 0; octave < 4; ++octave) {
                const int sd = (int)seed + octave;
                const float v = or_simplex3(fx, fy, 0.0f, freq, sd);
                const float vx = or_simplex3(fx + d, fy, 0.0f, freq, sd);
                const float vy = or_simplex3(fx, fy + d, 0.0f, freq, sd);
                const float gx = (vx - v) / d, gy = (vy - v) / d;
                const float mag = sqrtf(gx * gx + gy * gy);
                const float r = 0.0f + 1.0f * ((v / (1.0f + mag) - -1.0f) / (1.0f - -1.0f));
                value = value + r * amp;
                amp = amp * 0.1f;
                freq = freq * 10.0f;
            }
            h[i] = 5000.0f + value * (15000.0f - 5000.0f);
        }
}

/* ---- plate relabel and merges ------------------------------------------------------------------ */

static int cmp_u64_desc(const void *a, const void *b)
{
    const uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? 1 : (x > y ? -1 : 0);
}

/* applyCCL's relabel (plate_tectonic_sim.cu:391-467; createPlateIdLabelMap, getMaxSizeLabels,
 * createLabelIdLookup, postCClIdReassign, assignUnassignedIdsToNeighbor :1394-1405, :3114-3206,
 * :2052-2101).  Components (CCL labels: the minimum cell index of each) are ranked by cell count,
 * larger first, ties by the larger label (the reference's sort by label and then by count).  Of the
 * first min(255, components): a component as large as its plate's largest keeps the plate's id;
 * a smaller one of at least minPlateSize cells takes the next free id (ascending among the ids below
 * min(255, components) whose plate has no cells), with a copy of the plate's records; any other
 * component loses its id.  Cells without an id then take the most frequent id among their eight
 * neighbours (first in the order +x, -x, +y, -y, +x+y, +x-y, -x+y, -x-y on ties), in rounds that
 * each read the ids of the round before, until none is left or a round assigns nothing.  Returns
 * the number of cells left without an id. */
int or_relabel(int W, int H, uint8_t *id, const uint32_t *labels, tecto_plate *plates, tecto_plate_dynamics *dyn,
               int minPlateSize)
{
    const size_t N = (size_t)W * (size_t)H;
    uint32_t *count = (uint32_t *)calloc(N, sizeof(uint32_t));
    for (size_t i = 0; i < N; ++i) count[labels[i]] += 1;
    size_t M = 0;
    for (size_t i = 0; i < N; ++i)
        if (labels[i] == i) ++M;
    uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * (M ? M : 1));
    int max_count[256];
    memset(max_count, 0, sizeof(max_count));
    size_t m = 0;
    for (size_t i = 0; i < N; ++i)
        if (labels[i] == i) {
            keys[m++] = ((uint64_t)count[i] << 32) | (uint64_t)i;
            if ((int)count[i] > max_count[id[i]]) max_count[id[i]] = (int)count[i];
        }
    qsort(keys, M, sizeof(uint64_t), cmp_u64_desc);
    const int ntop = M < NPLATE ? (int)M : (int)NPLATE;
    int avail[NPLATE], navail = 0, next = 0;
    for (int k = 0; k < ntop; ++k)
        if (dyn[k].size == 0) avail[navail++] = k;
    uint8_t *lookup = (uint8_t *)malloc(N);  /* by root cell */
    for (size_t i = 0; i < N; ++i)
        if (labels[i] == i) lookup[i] = (uint8_t)NPLATE;
    for (int t = 0; t < ntop; ++t) {
        const uint32_t label = (uint32_t)(keys[t] & 0xFFFFFFFFu);
        const int c = (int)(keys[t] >> 32);
        const uint8_t plate = id[label];
        if (c == max_count[plate]) {
            lookup[label] = plate;
        } else if (c >= minPlateSize && next < navail) {
            const int nid = avail[next++];
            plates[nid] = plates[plate];
            dyn[nid] = dyn[plate];
            lookup[label] = (uint8_t)nid;
        }
    }
    size_t left = 0;
    for (size_t i = 0; i < N; ++i) {
        id[i] = lookup[labels[i]];
        if (id[i] == NPLATE) ++left;
    }
    static const int OX[8] = {1, -1, 0, 0, 1, 1, -1, -1}, OY[8] = {0, 0, 1, -1, 1, -1, 1, -1};
    uint8_t *pending = (uint8_t *)malloc(N);
    while (left > 0) {
        size_t assigned = 0;
        for (size_t i = 0; i < N; ++i) {
            pending[i] = (uint8_t)NPLATE;
            if (id[i] != NPLATE) continue;
            const int x = (int)(i % (size_t)W), y = (int)(i / (size_t)W);
            uint8_t nb[8];
            int n = 0;
            for (int k = 0; k < 8; ++k) {
                const uint8_t v = id[cidx(x + OX[k], y + OY[k], W, H)];
                if (v != NPLATE) nb[n++] = v;
            }
            int best = 0;
            uint8_t sel = (uint8_t)NPLATE;
            for (int a = 0; a < n; ++a) {
                int c = 1;
                for (int b = 0; b < n; ++b)
                    if (a != b && nb[b] == nb[a]) ++c;
                if (c > best) {
                    best = c;
                    sel = nb[a];
                }
            }
            pending[i] = sel;
        }
        for (size_t i = 0; i < N; ++i)
            if (pending[i] != NPLATE) {
                id[i] = pending[i];
                ++assigned;
            }
        left -= assigned;
        if (assigned == 0) break;
    }
    free(pending);
    free(lookup);
    free(keys);
    free(count);
    return (int)left;
}

/* mergePlates (plate_tectonic_sim.cu:470-494): getNeighboringPlates (:1283-1311) marks the plate
 * pairs that touch across a +x or +y cell edge; getPlateMerges (:1313-1379) takes the pairs in
 * ascending (max, min) order: two touching plates merge when both move no faster than
 * mergeMinVelocity, or when their smoothed directions agree (dot >= mergeDotDirectionThreshold) and
 * their smoothed speeds differ by at most mergeVelocityDiffThreshold; not while either waits
 * (mergeWaitTime) nor above targetMaximumPlateArea together; each plate merges at most once; the
 * heavier (ties: the lower id) is the parent.  Each merge clears the collision-type bitmap
 * entries clearCollisionTypes (:1381-1392) addresses: it indexes the 1-D triangle array with
 * (min(parent, k), max(parent, k)), which lands on entry min(parent, k), so entries 0..parent-1 and,
 * for a parent below 254, entry parent.  mergeAndCountSizeMass (:100-135) then gives each child's
 * cells the parent's id.  Returns the number of merges. */
int or_merge(int W, int H, uint8_t *id, const tecto_plate *plates, const tecto_plate_dynamics *dyn,
             uint8_t *type_bitmap, const tecto_kernel_settings *ks)
{
    static uint8_t nb[NPLATE * NPLATE];
    memset(nb, 0, sizeof(nb));
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const uint8_t c = id[(size_t)y * W + x];
            const uint8_t r = id[cidx(x + 1, y, W, H)], t = id[cidx(x, y + 1, W, H)];
            if (c != r && c != NPLATE && r != NPLATE)
                nb[(r < c ? c : r) * NPLATE + (r < c ? r : c)] = 1;
            if (c != t && c != NPLATE && t != NPLATE)
                nb[(t < c ? c : t) * NPLATE + (t < c ? t : c)] = 1;
        }
    int merge_ids[NPLATE];
    memset(merge_ids, 0, sizeof(merge_ids));
    int merges = 0;
    for (int idx = 0; idx < (int)(NPLATE * NPLATE); ++idx) {
        const int x = idx % (int)NPLATE, y = idx / (int)NPLATE;
        if (x >= y || !nb[idx]) continue;
        const float dot = dyn[x].directionSmoothed_x * dyn[y].directionSmoothed_x +
                          dyn[x].directionSmoothed_y * dyn[y].directionSmoothed_y;
        const float vdiff = fabsf(dyn[x].velocitySmoothed - dyn[y].velocitySmoothed);
        if (!(plates[x].velocity <= ks->mergeMinVelocity && plates[y].velocity <= ks->mergeMinVelocity) &&
            !(dot >= ks->mergeDotDirectionThreshold && vdiff <= ks->mergeVelocityDiffThreshold))
            continue;
        if (dyn[x].mergeWaitTime > 0 || dyn[y].mergeWaitTime > 0) continue;
        if (dyn[x].size + dyn[y].size > ks->targetMaximumPlateArea) continue;
        const int x_parent = dyn[y].mass <= dyn[x].mass;
        if (merge_ids[x] != 0) continue;
        merge_ids[x] = x_parent ? -1 : (int)NPLATE - y;
        if (merge_ids[y] != 0) {
            merge_ids[x] = 0;
            continue;
        }
        merge_ids[y] = x_parent ? (int)NPLATE - x : -1;
        const int parent = x_parent ? x : y;
        for (int k = 0; k < (int)NPLATE; ++k)
            if (k != parent) type_bitmap[k < parent ? k : parent] = 0;
        ++merges;
    }
    const size_t N = (size_t)W * (size_t)H;
    for (size_t i = 0; i < N; ++i)
        if (id[i] != NPLATE && merge_ids[id[i]] > 0) id[i] = (uint8_t)((int)NPLATE - merge_ids[id[i]]);
    return merges;
}

/* ---- settings and the synthetic world generator, restated for the CPU-only legs ----------------
 *
 * The reference arm and the CPU baseline of bench.py must not load the engine's library, so the
 * oracle carries its own copies of the two parameter sets and of the benchmark's world generator.
 * tests/test_oracle_units.py checks that both equal the engine's byte for byte. */

/* KernelSettings' initialisers (src/cuda_compute/kernel_settings.cuh:6-71), SimulationSettings'
 * (src/generation_settings.h:69-72) and the literal step constants of plate_tectonic_sim.cu:73,
 * :336-363. */
void or_settings_default(tecto_settings *out)
{
    memset(out, 0, sizeof(*out));
    tecto_kernel_settings *k = &out->kernel;
    k->inelasticCollisionMultiplierContinental = 1.f;
    k->inelasticCollisionMultiplierSubduction = 0.25f;
    k->inelasticCollisionMultiplierAccretion = 0.5f;
    k->frictionCoefficientContinental = 1.f;
    k->frictionCoefficientSubduction = 0.2f;
    k->frictionCoefficientAccretion = 0.5f;
    k->environmentalDragCoefficient = 0.25f;
    k->velocitySmoothingFactor = 0.9f;
    k->directionSmoothingFactor = 0.9f;
    k->breakScoreSmoothingFactor = 0.9f;
    k->mergeDotDirectionThreshold = .998f;
    k->mergeVelocityDiffThreshold = 0.01f;
    k->mergeMinVelocity = 0.05f;
    k->mergeWaitAfterSplit = 10;
    k->minPlateSize = 10;
    k->continentalCrustThreshold = 10000.f;
    k->divergence_height_target_min = 1000.f;
    k->divergence_height_target_max = 2000.f;
    k->divergence_interpolation_factor = 0.025f;
    k->collisionTypeUpdateCooldown = 4;
    k->minCollisionSize = 50;
    k->subductionOverUpliftMultiplier = 0.005f;
    k->subductionUnderUpliftMultiplier = 0.01f;
    k->continentalUpliftMultiplier = 0.01f;
    k->minUpliftClamp = 0.f;
    k->maxUpliftClamp = 20000.f;
    k->upliftRange = 50;
    k->subductionOverRange = 20;
    k->continentalPropMaxIters = 50;
    k->continentalPropThreshold = 13000;
    k->hydrationPipeCrossSection = 1000;
    k->hydrationPipeLength = 1000;
    k->hydrationRainfall = (float)0.101;
    k->hydrationEvaporation = (float)0.303;
    k->gravity = (float)9.81;
    k->sedimentCapacity = (float)0.9;
    k->sedimentErosionRate = (float)0.5;
    k->sedimentDepositionRate = (float)0.01;
    k->pressureAccumulation = 0.02f;
    k->pressureDecayRate = 0.8f;
    k->pressureBlurRange = 25;
    k->pressureMultiplier = 1.0f;
    k->curlNoiseMultiplier = 30.f;
    k->stressSplitThreshold = 30.0f;
    k->targetMinimumPlateArea = 100;
    k->targetMaximumPlateArea = 100000;
    k->thermalErosionStrength = 1.0f;
    k->thermalErosionAmplitude = 0.5f;
    k->thermalCellSize = 1000.0f;
    k->thermalThresholdAngle = 0.5f;
    out->sim.numStartingPlates = 16;
    out->sim.seed = 1000;
    out->sim.numVoronoiSeeds[0] = 200;
    out->sim.numVoronoiSeeds[1] = 500;
    out->sim.numVoronoiGenerations = 2;
    out->sim.iterationsForCCL = 10;
    out->step.hydraulicIterations = 10;
    out->step.hydraulicDt = 1.0f;
    out->step.thermalIterations = 1;
    out->step.upliftMode = TECTO_UPLIFT_GAUSSIAN;
    out->step.upliftAmount = 0.01f;
    out->step.upliftSigma = 1.5f;
    out->step.upliftRadius = 3;
    out->step.cclConnectivity = TECTO_CCL_REF8;
}

/* The benchmark physics mapped onto the reference's parameters: rain 0.01, evaporation 0.05,
 * Kc 0.1, Ks 0.3, Kd 0.1, 20 hydraulic sub-iterations of dt 0.02, 10 thermal iterations with talus
 * 0.01 and rate 0.5, continental above height 0, Gaussian uplift 0.01 (sigma 1.5, radius 3), 4-connected
 * CCL every 10 steps. */
void or_settings_baseline(tecto_settings *out)
{
    or_settings_default(out);
    tecto_kernel_settings *k = &out->kernel;
    k->hydrationRainfall = 0.01f;
    k->hydrationEvaporation = 0.05f;
    k->sedimentCapacity = 0.1f;
    k->sedimentErosionRate = 0.3f;
    k->sedimentDepositionRate = 0.1f;
    k->thermalThresholdAngle = 0.01f;
    k->thermalCellSize = 1.0f;
    k->thermalErosionAmplitude = 0.5f;
    k->thermalErosionStrength = 1.0f;
    k->continentalCrustThreshold = 0.0f;
    out->step.hydraulicIterations = 20;
    out->step.hydraulicDt = 0.02f;
    out->step.thermalIterations = 10;
    out->step.upliftMode = TECTO_UPLIFT_GAUSSIAN;
    out->step.upliftAmount = 0.01f;
    out->step.upliftSigma = 1.5f;
    out->step.upliftRadius = 3;
    out->step.cclConnectivity = TECTO_CCL_4;
    out->sim.iterationsForCCL = 10;
}

/* splitmix64 (G. L. Steele, D. Lea, C. H. Flood, "Fast splittable pseudorandom number generators",
 * OOPSLA 2014) and a 24-bit uniform in [0, 1). */
static uint64_t or_splitmix64(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static float or_u01(uint64_t r) { return (float)(r >> 40) * (1.0f / 16777216.0f); }

/* The synthetic world of the benchmark configurations: P seed points uniform on the grid, each a
 * plate with a velocity uniform in [-velRange, velRange]^2; every cell takes the plate of its
 * nearest seed on the torus (first on ties); even plates are continental, 0.5 + 0.05 N, odd ones
 * oceanic, -0.5 + 0.02 N, N the Irwin-Hall sum of 12 uniforms minus 6 from a per-cell stream. */
int or_generate_world(int W, int H, int P, float velRange, uint64_t genSeed, float *height_out, uint8_t *id_out,
                      tecto_plate *plates_out)
{
    if (W < 1 || H < 1 || P < 1 || P > TECTO_MAX_PLATES) return -1;
    float *sx = (float *)calloc((size_t)P, sizeof(float)), *sy = (float *)calloc((size_t)P, sizeof(float));
    if (!sx || !sy) {
        free(sx);
        free(sy);
        return -3;
    }
    uint64_t st = genSeed;
    if (plates_out) memset(plates_out, 0, sizeof(tecto_plate) * TECTO_MAX_PLATES);
    for (int k = 0; k < P; ++k) {
        sx[k] = or_u01(or_splitmix64(&st)) * (float)W;
        sy[k] = or_u01(or_splitmix64(&st)) * (float)H;
        const float vx = (2.0f * or_u01(or_splitmix64(&st)) - 1.0f) * velRange;
        const float vy = (2.0f * or_u01(or_splitmix64(&st)) - 1.0f) * velRange;
        const float v = sqrtf(vx * vx + vy * vy);
        if (plates_out) {
            plates_out[k].velocity = v;
            plates_out[k].direction_x = v > 0.0f ? vx / v : 1.0f;
            plates_out[k].direction_y = v > 0.0f ? vy / v : 0.0f;
            plates_out[k].pixelCenter_x = sx[k] - floorf(sx[k]);
            plates_out[k].pixelCenter_y = sy[k] - floorf(sy[k]);
        }
    }
    const float fW = (float)W, fH = (float)H;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            const size_t i = (size_t)y * (size_t)W + (size_t)x;
            float best = 3.4e38f;
            int bid = 0;
            for (int k = 0; k < P; ++k) {
                const float dx = fabsf((float)x - sx[k]), dy = fabsf((float)y - sy[k]);
                const float wx = fminf(dx, fW - dx), wy = fminf(dy, fH - dy);
                const float d2 = wx * wx + wy * wy;
                if (d2 < best) {
                    best = d2;
                    bid = k;
                }
            }
            if (id_out) id_out[i] = (uint8_t)bid;
            if (height_out) {
                uint64_t cs = genSeed ^ (0xD1B54A32D192ED03ull * (uint64_t)(i + 1));
                float sum = 0.0f;
                for (int r = 0; r < 12; ++r) sum = sum + or_u01(or_splitmix64(&cs));
                const float n = sum - 6.0f;
                height_out[i] = (bid % 2 == 0) ? 0.5f + 0.05f * n : -0.5f + 0.02f * n;
            }
        }
    }
    free(sx);
    free(sy);
    return 0;
}
