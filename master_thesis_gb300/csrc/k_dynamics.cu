// k_dynamics.cu - plate dynamics (TECTO_PLATE_DYNAMICS_REFERENCE): the per-plate sums a step starts
// from (mass, size, the angular centre sums) and applyPlateMovementChanges at the step's end.
// Reference: src/cuda_compute/plate_tectonics_kernel.cu - mergeAndCountSizeMass's mass and size
// (:100-195, without merges), accumulatePlateAngularCoords (:2154-2189), calculatePlateCenters
// (:2191-2226), applyPlateMovementChanges (:1863-1925), computeCurl (:2788-2822); the order of
// PlateTectonicSim::executeIteration (plate_tectonic_sim.cu:54-131).
//
// The reference adds these sums with float atomics in whatever order the threads arrive, so its
// results vary from run to run in the last bits.  Here every term is converted to 64-bit fixed point
// first (tecto_fix) and the integer sums are exact, so each run, the batch path and the CPU oracle
// give the same bits.  The collision friction is accumulated in the resolve kernel
// (k_resolve.cu) the same way.
#include "tecto_internal.cuh"

namespace tecto {

namespace {

// Per-plate mass and size over all cells, and the angular sums of every cell whose x and y are
// multiples of 10, over 256 x 16 tiles of the batch.  Each thread walks one column of its tile and
// keeps a run of equal plate ids in registers; runs and samples go to shared sums, the block's
// sums to the world's PlateAcc.
__global__ __launch_bounds__(256) void k_plate_stats(const WorldDev *worlds, const uint2 *tiles, int cur_h,
                                                     int cur_id)
{
    __shared__ unsigned long long s_mass[kPlates];
    __shared__ unsigned long long s_ang[4][kPlates];
    __shared__ int s_size[kPlates], s_samp[kPlates];
    int wi, tx, ty;
    tile_of(tiles[blockIdx.x], &wi, &tx, &ty);
    const WorldDev &wd = worlds[wi];
    for (int i = threadIdx.x; i < kPlates; i += blockDim.x) {
        s_mass[i] = 0ull;
        s_ang[0][i] = s_ang[1][i] = s_ang[2][i] = s_ang[3][i] = 0ull;
        s_size[i] = 0;
        s_samp[i] = 0;
    }
    __syncthreads();
    const int W = wd.W, H = wd.H;
    const int x = tx * kStatTileX + (int)threadIdx.x;
    if (x < W) {
        const float *h = wd.h[cur_h];
        const uint8_t *id = wd.id[cur_id];
        const int y0 = ty * kStatTileY;
        const int y1 = min(y0 + kStatTileY, H);
        int run = -1, run_n = 0;
        unsigned long long run_m = 0ull;
        const bool xs = x % 10 == 0;
        const float ax = (kTwoPiF * (float)x) / (float)W;
        const float sin_x = tecto_sinf(ax), cos_x = tecto_cosf(ax);
        for (int y = y0; y < y1; ++y) {
            const size_t d = (size_t)y * (size_t)W + (size_t)x;
            const int p = id[d];
            const float hv = h[d];
            if (p != run) {
                if (run >= 0 && run < kPlates) {
                    atomicAdd(s_mass + run, run_m);
                    atomicAdd(s_size + run, run_n);
                }
                run = p;
                run_m = 0ull;
                run_n = 0;
            }
            run_m += (unsigned long long)tecto_fix(hv, kMassScale, kMassLimit);
            ++run_n;
            if (xs && y % 10 == 0 && p < kPlates) {
                const float ay = (kTwoPiF * (float)y) / (float)H;
                atomicAdd(&s_ang[0][p], (unsigned long long)tecto_fix(sin_x, kAngScale, 1.0f));
                atomicAdd(&s_ang[1][p], (unsigned long long)tecto_fix(cos_x, kAngScale, 1.0f));
                atomicAdd(&s_ang[2][p], (unsigned long long)tecto_fix(tecto_sinf(ay), kAngScale, 1.0f));
                atomicAdd(&s_ang[3][p], (unsigned long long)tecto_fix(tecto_cosf(ay), kAngScale, 1.0f));
                atomicAdd(s_samp + p, 1);
            }
        }
        if (run >= 0 && run < kPlates) {
            atomicAdd(s_mass + run, run_m);
            atomicAdd(s_size + run, run_n);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kPlates; i += blockDim.x) {
        if (s_size[i] == 0) continue;
        PlateAcc &a = wd.pacc[i];
        atomicAdd(&a.mass, s_mass[i]);
        atomicAdd(&a.size, s_size[i]);
        if (s_samp[i] == 0) continue;
        atomicAdd(&a.ang[0], s_ang[0][i]);
        atomicAdd(&a.ang[1], s_ang[1][i]);
        atomicAdd(&a.ang[2], s_ang[2][i]);
        atomicAdd(&a.ang[3], s_ang[3][i]);
        atomicAdd(&a.samples, s_samp[i]);
    }
}

__device__ __forceinline__ int wrap_coord(int v, int n)
{
    const int r = v % n;
    return r < 0 ? r + n : r;
}

struct MotionParams {
    float curlMul, drag, velSmooth, dirSmooth;
};

// applyPlateMovementChanges (:1863-1925) for plate velocity and direction, one block per world.
// The sub-cell centre update of the same kernel ran at the step's start (k_plates), with the same
// velocity and direction.
__global__ void k_plate_motion(const WorldDev *worlds, MotionParams mp)
{
    const WorldDev &wd = worlds[blockIdx.x];
    const int k = threadIdx.x;
    if (k >= kPlates) return;
    tecto_plate p = wd.plates[k];
    tecto_plate_dynamics dd = wd.dyn[k];
    const float friction = tecto_unfix((long long)wd.pacc[k].fric, 1.0 / (double)kFricScale);
    wd.pacc[k].fric = 0ull;
    // asthenosphere flow at the geometric centre: the curl of the pressure texture, nearest-scaled
    // to the world (computeCurl at that one cell)
    float sx = 0.0f, sy = 0.0f;
    if (wd.pressure) {
        const float gx = fminf(fmaxf(dd.geometricCenter_x + 0.5f, -1073741824.0f), 1073741824.0f);
        const float gy = fminf(fmaxf(dd.geometricCenter_y + 0.5f, -1073741824.0f), 1073741824.0f);
        const int cx = wrap_coord((int)gx, wd.W), cy = wrap_coord((int)gy, wd.H);
        const double xs = (double)wd.pw / (double)wd.W, ys = (double)wd.ph / (double)wd.H;
        const int qx = (int)((double)cx * xs), qy = (int)((double)cy * ys);
        const float *pr = wd.pressure;
        const int pw = wd.pw, ph = wd.ph;
        const float left = pr[(size_t)qy * pw + wrap_coord(qx - 1, pw)];
        const float right = pr[(size_t)qy * pw + wrap_coord(qx + 1, pw)];
        const float bottom = pr[(size_t)wrap_coord(qy - 1, ph) * pw + qx];
        const float top = pr[(size_t)wrap_coord(qy + 1, ph) * pw + qx];
        sy = (float)((double)(right - left) * 0.5);
        sx = (float)(-((double)(top - bottom) * 0.5));
    }
    const float avx = fmaxf(fminf((float)((double)(sx * mp.curlMul) + (sx < 0.0f ? -0.2 : 0.2)), 1.0f), -1.0f);
    const float avy = fmaxf(fminf((float)((double)(sy * mp.curlMul) + (sy < 0.0f ? -0.2 : 0.2)), 1.0f), -1.0f);
    const float dx = p.direction_x, dy = p.direction_y;
    const float ovx = dx * p.velocity, ovy = dy * p.velocity;
    const float mag = fmaxf(sqrtf(ovx * ovx + ovy * ovy), 1e-20f);
    const float post = fmaxf(mag - friction, 0.0f);
    const float pvx = dx * post, pvy = dy * post;
    const float rx = avx - pvx, ry = avy - pvy;
    const float rmag = sqrtf(rx * rx + ry * ry);
    const float drag = mp.drag * rmag * rmag;
    const float rn = fmaxf(sqrtf(rx * rx + ry * ry), 1e-20f);
    const float nvx = pvx + (rx / rn) * drag, nvy = pvy + (ry / rn) * drag;
    const float nmag = fmaxf(sqrtf(nvx * nvx + nvy * nvy), 1e-20f);
    p.velocity = nmag;
    p.direction_x = nvx / nmag;
    p.direction_y = nvy / nmag;
    dd.velocitySmoothed = dd.velocitySmoothed * mp.velSmooth + p.velocity * (1.0f - mp.velSmooth);
    const float sdx = dd.directionSmoothed_x * mp.dirSmooth + p.direction_x * (1.0f - mp.dirSmooth);
    const float sdy = dd.directionSmoothed_y * mp.dirSmooth + p.direction_y * (1.0f - mp.dirSmooth);
    const float sm = fmaxf(sqrtf(sdx * sdx + sdy * sdy), 1e-20f);
    dd.directionSmoothed_x = sdx / sm;
    dd.directionSmoothed_y = sdy / sm;
    dd.mergeWaitTime = dd.mergeWaitTime > 0 ? dd.mergeWaitTime - 1 : 0;
    dd.frictionLoss = friction;
    wd.plates[k] = p;
    wd.dyn[k] = dd;
}

}  // namespace

int launch_plate_stats(Batch &b, cudaStream_t st)
{
    k_plate_stats<<<(unsigned)b.ntiles[TK_STATS], 256, 0, st>>>(b.d_worlds, b.d_tiles[TK_STATS], b.cur_h, b.cur_id);
    TECTO_CUDA(cudaGetLastError());
    b.launches += 1;
    return TECTO_OK;
}

int launch_plate_motion(Batch &b, cudaStream_t st)
{
    const tecto_kernel_settings &ks = b.settings.kernel;
    const MotionParams mp{ks.curlNoiseMultiplier, ks.environmentalDragCoefficient, ks.velocitySmoothingFactor,
                          ks.directionSmoothingFactor};
    k_plate_motion<<<(unsigned)b.members.size(), 256, 0, st>>>(b.d_worlds, mp);
    TECTO_CUDA(cudaGetLastError());
    b.launches += 1;
    return TECTO_OK;
}

}  // namespace tecto
