// tecto_init.cu - the reference's world initialisation with its per-cell work on the device:
// PlateTectonicSim::initializeTectonics (src/cuda_compute/plate_tectonic_sim.cu:705-773).
//
// Host (cheap: plates x seeds distance tests): the plate centres, the Voronoi seed generations and
// the plate kinematics, drawn from std::default_random_engine seeded with the world's seed through
// std::uniform_real_distribution<float>, in the reference's order of draws (generatePlateCenters
// :873-890, generateVoronoiSeeds :892-929, generatePlateData :816-842).  The reference draws a
// position as {height range, width range}: x from [0, H) and y from [0, W); that is kept.
// Device (per cell): the nearest seed on the torus (initPlateIDs, plate_tectonics_kernel.cu:31-63)
// and the four-octave simplex height map with its slope damping (initHeightmap, :65-99), in one
// kernel.  The reference's initPixelDependantPlateData and applyCCL follow: mass and size come from
// the plate-dynamics sums of the first step, and the CCL labels are computed here (the relabel of
// plate fragments is not part of this engine).
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "noise.cuh"
#include "tecto_internal.cuh"

namespace tecto {

namespace {

struct SeedPoint {
    float x, y;
    int id;
};

// initializeTectonics' host part.  Returns false on invalid settings.
bool reference_seeds(int W, int H, uint32_t seed, int numPlates, const int *gens, int ngens,
                     std::vector<SeedPoint> &seeds, std::vector<tecto_plate> &plates,
                     std::vector<tecto_plate_dynamics> &dyn)
{
    if (numPlates < 1 || numPlates > kPlates || ngens < 0 || ngens > TECTO_MAX_VORONOI_GENS) return false;
    for (int g = 0; g < ngens; ++g)
        if (gens[g] < 0 || gens[g] > (1 << 20)) return false;
    std::default_random_engine generator(seed);
    std::uniform_real_distribution<float> randomHeight(0, (float)H);
    std::uniform_real_distribution<float> randomWidth(0, (float)W);
    std::vector<SeedPoint> centres((size_t)numPlates);
    for (int i = 0; i < numPlates; ++i) {
        const float px = randomHeight(generator);
        const float py = randomWidth(generator);
        centres[(size_t)i] = SeedPoint{px, py, i};
    }
    seeds = centres;
    for (int g = 0; g < ngens; ++g) {
        std::vector<SeedPoint> next((size_t)gens[g]);
        for (int i = 0; i < gens[g]; ++i) {
            const float sx = randomHeight(generator);
            const float sy = randomWidth(generator);
            float best = 3.40282347e38f;
            int id = 0;
            for (const SeedPoint &c : seeds) {
                const float dx = fabsf(sx - c.x), dy = fabsf(sy - c.y);
                const float wx = std::min(dx, (float)W - dx), wy = std::min(dy, (float)H - dy);
                const float d2 = wx * wx + wy * wy;
                if (d2 < best) {
                    id = c.id;
                    best = d2;
                }
            }
            next[(size_t)i] = SeedPoint{sx, sy, id};
        }
        seeds.swap(next);
    }
    if (seeds.size() < centres.size()) seeds = centres;
    std::uniform_real_distribution<float> dist(-1, 1);
    plates.assign(kPlates, tecto_plate{});
    dyn.assign(kPlates, tecto_plate_dynamics{});
    for (int i = 0; i < numPlates; ++i) {
        tecto_plate &p = plates[(size_t)i];
        const SeedPoint &c = centres[(size_t)i];
        p.pixelCenter_x = c.x - std::floor(c.x);
        p.pixelCenter_y = c.y - std::floor(c.y);
        p.velocity = (dist(generator) + 1) / 2;
        const float xd = dist(generator);
        const float yd = dist(generator);
        const float m = std::sqrt(xd * xd + yd * yd);
        p.direction_x = xd / m;
        p.direction_y = yd / m;
        dyn[(size_t)i].velocitySmoothed = p.velocity;
        dyn[(size_t)i].directionSmoothed_x = p.direction_x;
        dyn[(size_t)i].directionSmoothed_y = p.direction_y;
    }
    return true;
}

constexpr int kSeedChunk = 2048;

// initPlateIDs + initHeightmap for one cell per thread.  Seeds go through shared memory in chunks,
// in index order, so the first seed at the minimum distance wins as in the reference's loop.
__global__ __launch_bounds__(256) void k_init_reference(float *h, uint8_t *id, int W, int H, const float *sx,
                                                        const float *sy, const int *sid, int nseeds, int seed)
{
    __shared__ float s_x[kSeedChunk], s_y[kSeedChunk];
    __shared__ int s_id[kSeedChunk];
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < (size_t)W * (size_t)H;
    const int y = live ? (int)(i / (size_t)W) : 0, x = live ? (int)(i - (size_t)y * W) : 0;
    const float fx = (float)x, fy = (float)y, fW = (float)W, fH = (float)H;
    float best = 3.40282347e38f;
    int plate = 0;
    for (int base = 0; base < nseeds; base += kSeedChunk) {
        const int n = min(kSeedChunk, nseeds - base);
        __syncthreads();
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            s_x[k] = sx[base + k];
            s_y[k] = sy[base + k];
            s_id[k] = sid[base + k];
        }
        __syncthreads();
        for (int k = 0; k < n; ++k) {
            const float dx = fabsf(fx - s_x[k]), dy = fabsf(fy - s_y[k]);
            const float wx = fminf(dx, fW - dx), wy = fminf(dy, fH - dy);
            const float d2 = wx * wx + wy * wy;
            if (d2 < best) {
                plate = s_id[k];
                best = d2;
            }
        }
    }
    if (!live) return;
    id[i] = (uint8_t)plate;
    const float d = 0.001f;
    float value = 0.0f, amp = 0.9f, freq = 0.01f;
    for (int octave = 0; octave < 4; ++octave) {
        const float v = simplex3(fx, fy, 0.0f, freq, seed + octave);
        const float vx = simplex3(fx + d, fy, 0.0f, freq, seed + octave);
        const float vy = simplex3(fx, fy + d, 0.0f, freq, seed + octave);
        const float gx = (vx - v) / d, gy = (vy - v) / d;
        const float mag = sqrtf(gx * gx + gy * gy);
        const float r = 0.0f + 1.0f * ((v / (1.0f + mag) - -1.0f) / (1.0f - -1.0f));
        value = value + r * amp;
        amp = amp * 0.1f;
        freq = freq * 10.0f;
    }
    h[i] = 5000.0f + value * (15000.0f - 5000.0f);
}

}  // namespace

}  // namespace tecto

using namespace tecto;

extern "C" {

int tecto_world_init(tecto_world *world, int numPlates, const int *numVoronoiSeeds, int generations,
                     tecto_stream_t stream)
{
    if (!world || numPlates < 1 || numPlates > kPlates || generations < 0 || generations > TECTO_MAX_VORONOI_GENS ||
        (generations > 0 && !numVoronoiSeeds)) {
        set_error("tecto_world_init: 1..255 plates, 0..8 Voronoi generations");
        return TECTO_ERR_INVALID;
    }
    tecto_settings s = world->settings;
    s.sim.numStartingPlates = numPlates;
    s.sim.numVoronoiGenerations = generations;
    for (int g = 0; g < generations; ++g) s.sim.numVoronoiSeeds[g] = numVoronoiSeeds[g];
    const int rc = tecto_world_set_settings(world, &s);
    if (rc != TECTO_OK) return rc;
    return tecto_world_init_reference(world, stream);
}

int tecto_reference_seeds(int width, int height, uint32_t seed, int numPlates, const int *numVoronoiSeeds,
                          int generations, float *seed_x, float *seed_y, uint8_t *seed_id, int capacity,
                          int *count, tecto_plate *plates, tecto_plate_dynamics *dynamics)
{
    if (width < 1 || height < 1 || (generations > 0 && !numVoronoiSeeds) || !count) return TECTO_ERR_INVALID;
    std::vector<SeedPoint> seeds;
    std::vector<tecto_plate> pl;
    std::vector<tecto_plate_dynamics> dy;
    if (!reference_seeds(width, height, seed, numPlates, numVoronoiSeeds, generations, seeds, pl, dy)) {
        set_error("tecto_reference_seeds: 1..255 plates, 0..8 generations of 0..2^20 seeds");
        return TECTO_ERR_INVALID;
    }
    *count = (int)seeds.size();
    if (plates) std::memcpy(plates, pl.data(), sizeof(tecto_plate) * kPlates);
    if (dynamics) std::memcpy(dynamics, dy.data(), sizeof(tecto_plate_dynamics) * kPlates);
    if (seed_x || seed_y || seed_id) {
        if (capacity < (int)seeds.size()) {
            set_error("tecto_reference_seeds: output capacity below the seed count");
            return TECTO_ERR_INVALID;
        }
        for (size_t k = 0; k < seeds.size(); ++k) {
            if (seed_x) seed_x[k] = seeds[k].x;
            if (seed_y) seed_y[k] = seeds[k].y;
            if (seed_id) seed_id[k] = (uint8_t)seeds[k].id;
        }
    }
    return TECTO_OK;
}

int tecto_world_init_reference(tecto_world *w, tecto_stream_t stream)
{
    if (!w) return TECTO_ERR_INVALID;
    const tecto_simulation_settings &sim = w->settings.sim;
    std::vector<SeedPoint> seeds;
    std::vector<tecto_plate> pl;
    std::vector<tecto_plate_dynamics> dy;
    if (!reference_seeds(w->W, w->H, w->seed, sim.numStartingPlates, sim.numVoronoiSeeds, sim.numVoronoiGenerations,
                         seeds, pl, dy)) {
        set_error("tecto_world_init_reference: numStartingPlates 1..255, numVoronoiGenerations 0..8, seeds 0..2^20");
        return TECTO_ERR_INVALID;
    }
    if (!w->arena) {
        set_error("null or destroyed world");
        return TECTO_ERR_INVALID;
    }
    TECTO_CUDA(cudaSetDevice(w->device));
    cudaStream_t st = (cudaStream_t)stream;
    // a fresh world: every field, bitmap and record zero, iteration 0
    w->iteration = 0;
    TECTO_CUDA(cudaMemsetAsync(w->arena, 0, w->arena_bytes, st));
    Control c{};
    c.seed = w->seed;
    TECTO_CUDA(cudaMemcpyAsync(w->dev.ctl, &c, sizeof(c), cudaMemcpyHostToDevice, st));
    const int S = (int)seeds.size();
    std::vector<float> hx((size_t)S), hy((size_t)S);
    std::vector<int> hid((size_t)S);
    for (int k = 0; k < S; ++k) {
        hx[(size_t)k] = seeds[(size_t)k].x;
        hy[(size_t)k] = seeds[(size_t)k].y;
        hid[(size_t)k] = seeds[(size_t)k].id;
    }
    void *tmp = nullptr;
    TECTO_CUDA(cudaMalloc(&tmp, (size_t)S * 12 + 16));
    float *dx = (float *)tmp, *dyp = dx + S;
    int *did = (int *)(dyp + S);
    cudaError_t e = cudaMemcpyAsync(dx, hx.data(), (size_t)S * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dyp, hy.data(), (size_t)S * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(did, hid.data(), (size_t)S * 4, cudaMemcpyHostToDevice, st);
    const WorldDev &d = w->dev;
    if (e == cudaSuccess) {
        k_init_reference<<<(unsigned)((w->N + 255) / 256), 256, 0, st>>>(d.h[w->cur_h], d.id[w->cur_id], w->W, w->H,
                                                                        dx, dyp, did, S, (int)w->seed);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.plates, pl.data(), sizeof(tecto_plate) * kPlates, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d.dyn, dy.data(), sizeof(tecto_plate_dynamics) * kPlates, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(tmp);
    if (e != cudaSuccess) return cuda_fail(e, "tecto_world_init_reference");
    w->launches += 1;
    return tecto_phase_ccl(w, w->settings.step.cclConnectivity, stream);
}

}  // extern "C"
