// k_resolve.cu - per-destination-cell resolve (divergence / movement / convergence), the
// Gaussian uplift fused into the same tile, the divergence-bitmap flip, and accretion.
// Reference: processCollisions and helpers, src/cuda_compute/plate_tectonics_kernel.cu:301-780.
#include "noise.cuh"
#include "tecto_internal.cuh"

namespace tecto {

namespace {

constexpr int RX = 64;   // resolve tile width (cells)
constexpr int RY = 16;   // resolve tile height
constexpr int kMaxBlurRadius = 8;

struct ResolveParams {
    const WorldDev *worlds;
    const uint2 *tiles;
    int cur_h, cur_id;
    float thr;
    float tmin, tmax, tfac;
    float amount;
    float wts[2 * kMaxBlurRadius + 1];
    float *upl_h;      // reference uplift: processConvergence's records by virtual cell, or null
    uint8_t *upl_t;
    float fricC, fricA, fricS;  // frictionCoefficientContinental / Accretion / Subduction
};

// Plate dynamics' view inside the resolve: velocity and mass per plate, and the block's friction
// sums (fixed point, see PlateAcc).
struct ResolveDyn {
    const float *vel;
    const float *mass;
    unsigned long long *fric;
};

// One world's view inside the resolve kernel.
struct ResolveWorld {
    int W, H;
    uint32_t vbase;
    const uint32_t *word;
    const uint8_t *id_old;
    const float *h_old;
    const uint8_t *bm;
    const uint32_t *div_bitmap;
    uint32_t *has_div;
    unsigned long long *acc;
    uint32_t *acc_list;
    uint32_t *acc_count;
};

// determineCollisionType device function (:611-649)
__device__ __forceinline__ uint32_t pair_type(const uint8_t *bm, uint8_t A, uint8_t B, float hA,
                                              float hB, float thr)
{
    const bool cond = A < B;
    const uint8_t mn = cond ? A : B, mx = cond ? B : A;
    const float mnH = cond ? hA : hB, mxH = cond ? hB : hA;
    const uint32_t packed = __ldg(bm + tri_index(mn, mx));
    const uint32_t hasType = packed & 1u, type = (packed >> 1) & 1u, pol = (packed >> 3) & 1u;
    uint32_t out = 0;
    if (hasType && type == 0) {
        if (pol == 1) out = (mnH >= thr) ? (mn == A ? 3u : 4u) : (mn == A ? 1u : 2u);
        if (pol == 0) out = (mxH >= thr) ? (mx == A ? 3u : 4u) : (mx == A ? 1u : 2u);
    }
    return out;
}

__device__ __forceinline__ void mark_accretion(const ResolveParams &p, const ResolveWorld &w,
                                               uint32_t target, uint32_t d, uint8_t owner)
{
    // last writer in cell order wins (the reference writes the byte plainly, :531-555)
    const unsigned long long v = ((unsigned long long)(d + 1u) << 8) | (unsigned long long)(255u - owner);
    const unsigned long long old = atomicMax(w.acc + target, v);
    if (old == 0ull) {
        const uint32_t slot = atomicAdd(w.acc_count, 1u);
        w.acc_list[slot] = target;
    }
}

// Resolve one destination cell d = (x, y); returns the new height (before uplift).
template <bool DYN>
__device__ __forceinline__ float resolve_cell(const ResolveParams &p, const ResolveWorld &w,
                                              const int2 *s_off, int x, int y, uint32_t d, uint32_t cv,
                                              uint32_t seed, uint32_t iteration, uint8_t *id_out,
                                              const ResolveDyn &dyn)
{
    // Convergent cells also leave processConvergence's UpliftData (:501-582) for the reference
    // uplift when it is on: heightAddition, the sum of each owner pair's lower height, and typeByte.
    const int W = w.W, H = w.H;
    if (cv == 0u) {
        // processDivergence (:301-362)
        const uint8_t prev = w.id_old[d];
        const int2 o = s_off[prev];
        const uint32_t cvo = w.word[cidx(x - o.x, y - o.y, W, H)];
        const uint8_t oppId = (uint8_t)((255u - cvo) & 0xFFu);
        uint8_t nid = prev;
        if (cvo != 0u && cvo <= 0xFFu && oppId != prev) {
            const uint8_t mn = prev < oppId ? prev : oppId;
            const uint8_t mx = prev < oppId ? oppId : prev;
            const uint32_t bit = tri_index(mn, mx);
            nid = (__ldg(w.div_bitmap + bit / 32u) & (1u << (bit % 32u))) ? mn : mx;
            atomicOr(w.has_div + bit / 32u, 1u << (bit % 32u));
        }
        const float noise = simplex3((float)x, (float)y, (float)iteration, 0.01f, (int)seed);
        const float target = p.tmin + noise * (p.tmax - p.tmin);
        *id_out = nid;
        return lerp_p0811(w.h_old[d], target, p.tfac);
    }
    uint8_t ids[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) ids[k] = (uint8_t)(255u - ((cv >> (8 * k)) & 0xFFu));
    if (ids[1] == 255) {
        // processMovement (:586-609)
        const int2 o = s_off[ids[0]];
        *id_out = ids[0];
        return w.h_old[cidx(x - o.x, y - o.y, W, H)];
    }
    // processConvergence (:469-584)
    const int n = ids[3] != 255 ? 4 : ids[2] != 255 ? 3 : 2;
    const int pairLen = n == 4 ? 6 : n == 3 ? 3 : 1;
    const int PA[6] = {0, 0, 1, 0, 1, 2};
    const int PB[6] = {1, 2, 2, 3, 3, 3};
    float heights[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int k = 0; k < n; ++k) {
        const int2 o = s_off[ids[k]];
        heights[k] = w.h_old[cidx(x - o.x, y - o.y, W, H)];
    }
    uint32_t types[6];
    bool sub[4] = {false, false, false, false};
    for (int a = 0; a < pairLen; ++a) {
        types[a] = pair_type(w.bm, ids[PA[a]], ids[PB[a]], heights[PA[a]], heights[PB[a]], p.thr);
        if (types[a] == 1u || types[a] == 3u) sub[PA[a]] = true;
        else if (types[a] == 2u || types[a] == 4u) sub[PB[a]] = true;
    }
    if (DYN) {
        // applyInelasticCollision's friction (:397-466 with applyElasticVelocityChange :371-394):
        // per arrival, velocity x coefficient x (source height / plate mass); the coefficient is the
        // continental one when a pair with this arrival has type 0, else the accretion one when a
        // pair has type 3 or 4, else the subduction one
        for (int k = 0; k < n; ++k) {
            bool cont = false, accr = false;
            for (int a = 0; a < pairLen; ++a) {
                if (PA[a] != k && PB[a] != k) continue;
                cont = cont || types[a] == 0u;
                accr = accr || types[a] == 3u || types[a] == 4u;
            }
            const float coef = cont ? p.fricC : (accr ? p.fricA : p.fricS);
            const float f = (dyn.vel[ids[k]] * coef) * (heights[k] / dyn.mass[ids[k]]);
            atomicAdd(dyn.fric + ids[k], (unsigned long long)tecto_fix(f, kFricScale, kFricLimit));
        }
    }
    int owner = 0;
    for (int i = 0; i < n; ++i)
        if (!sub[i]) owner = i;
    const uint8_t ownerId = ids[owner];
    float writeH = heights[owner];
    float hadd = 0.0f;
    uint32_t tbyte = 0;
    for (int a = 0; a < pairLen; ++a) {
        const int ia = PA[a], ib = PB[a];
        float hh;
        if (ia == owner) hh = heights[ib];
        else if (ib == owner) hh = heights[ia];
        else continue;
        if (hh > writeH) {  // writeHeight keeps the larger of the pair, the sum the smaller
            const float tmp = hh;
            hh = writeH;
            writeH = tmp;
        }
        hadd = hadd + hh;
        if (ia == owner)
            tbyte |= (types[a] == 2u ? 0u : 1u) | ((uint32_t)(ia & 3) << 1) | ((uint32_t)(ib & 3) << 3);
        else
            tbyte |= (types[a] == 1u ? 0u : 1u) | ((uint32_t)(ib & 3) << 1) | ((uint32_t)(ia & 3) << 3);
        int other = -1;
        if (ia == owner && types[a] == 4u) other = ib;
        else if (ib == owner && types[a] == 3u) other = ia;
        if (other >= 0) {
            const int2 oo = s_off[ids[other]];
            uint32_t target;
            if (oo.x != 0 || oo.y != 0) {
                target = cidx(x - oo.x, y - oo.y, W, H);
            } else {
                const int2 ow = s_off[ownerId];
                target = cidx(x + ow.x, y + ow.y, W, H);
            }
            mark_accretion(p, w, target, d, ownerId);
        }
    }
    if (p.upl_h) {
        p.upl_h[w.vbase + d] = hadd;
        p.upl_t[w.vbase + d] = (uint8_t)tbyte;
    }
    *id_out = ownerId;
    return writeH;
}

// Six blocks per SM (40 registers): the kernel waits mostly on its gathers from the arrival
// sources, and the extra resident warps hide them.
template <int R, bool DYN>
__global__ __launch_bounds__(256, 6) void k_resolve(ResolveParams p)
{
    constexpr int SX = RX + 2 * R, SY = RY + 2 * R;
    __shared__ uint32_t s_word[SY * SX];
    __shared__ float s_tmp[(R > 0) ? SY * RX : 1];
    __shared__ int2 s_off[kPlates + 1];
    __shared__ float s_vel[DYN ? kPlates : 1], s_mass[DYN ? kPlates : 1];
    __shared__ unsigned long long s_fric[DYN ? kPlates : 1];
    int wi, tx, ty;
    tile_of(p.tiles[blockIdx.x], &wi, &tx, &ty);
    const WorldDev &wd = p.worlds[wi];
    ResolveWorld w;
    w.W = wd.W;
    w.H = wd.H;
    w.vbase = wd.vbase;
    w.word = wd.word;
    w.id_old = wd.id[p.cur_id];
    w.h_old = wd.h[p.cur_h];
    w.bm = wd.type_bitmap;
    w.div_bitmap = wd.div_bitmap;
    w.has_div = wd.has_div;
    w.acc = wd.acc;
    w.acc_list = wd.acc_list;
    w.acc_count = &wd.ctl->acc_count;
    float *h_new = wd.h[p.cur_h ^ 1];
    uint8_t *id_new = wd.id[p.cur_id ^ 1];
    const int t = threadIdx.x;
    const int x0 = tx * RX, y0 = ty * RY;
    for (int i = t; i < kPlates + 1; i += 256) s_off[i] = wd.off[i];
    if (DYN) {
        for (int i = t; i < kPlates; i += 256) {
            s_vel[i] = wd.plates[i].velocity;
            s_mass[i] = wd.dyn[i].mass;
            s_fric[i] = 0ull;
        }
    }
    const ResolveDyn dyn{s_vel, s_mass, s_fric};
    for (int e = t; e < SY * SX; e += 256) {
        const int ly = e / SX, lx = e - ly * SX;
        const int gx = wrap_fast(x0 + lx - R, w.W), gy = wrap_fast(y0 + ly - R, w.H);
        s_word[e] = w.word[(size_t)gy * w.W + gx];
    }
    __syncthreads();
    if (R > 0) {
        // horizontal pass of the separable blur over the convergent-cell field
        for (int e = t; e < SY * RX; e += 256) {
            const int ly = e / RX, lx = e - ly * RX;
            float a = 0.0f;
#pragma unroll
            for (int k = -R; k <= R; ++k) {
                const float u = s_word[ly * SX + lx + R + k] > 0xFFu ? p.amount : 0.0f;
                a = a + p.wts[k + R] * u;
            }
            s_tmp[e] = a;
        }
        __syncthreads();
    }
    const uint32_t seed = wd.ctl->seed, iteration = wd.ctl->iteration;
    const int lx = t % RX;
#pragma unroll 1
    for (int ly = t / RX; ly < RY; ly += 256 / RX) {
        const int x = x0 + lx, y = y0 + ly;
        if (x >= w.W || y >= w.H) continue;
        const uint32_t d = (uint32_t)y * (uint32_t)w.W + (uint32_t)x;
        const uint32_t cv = s_word[(ly + R) * SX + lx + R];
        uint8_t nid;
        float hn = resolve_cell<DYN>(p, w, s_off, x, y, d, cv, seed, iteration, &nid, dyn);
        if (R > 0) {
            float a = 0.0f;
#pragma unroll
            for (int k = -R; k <= R; ++k) a = a + p.wts[k + R] * s_tmp[(ly + R + k) * RX + lx];
            hn = hn + a;
        }
        h_new[d] = hn;
        id_new[d] = nid;
    }
    if (DYN) {
        __syncthreads();
        for (int i = t; i < kPlates; i += 256)
            if (s_fric[i] != 0ull) atomicAdd(&wd.pacc[i].fric, s_fric[i]);
    }
}

// flipDivergedBitmap (:772-780) for every world; clears the per-step bits for the next step
__global__ void k_flip(const WorldDev *worlds)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kDivWords) {
        const WorldDev &wd = worlds[blockIdx.y];
        wd.div_bitmap[i] ^= wd.has_div[i];
        wd.has_div[i] = 0u;
    }
}

// applyAccretion (:747-770) over the cells that received a mark this step; clears the marks.
// Grid: (blocks, worlds).
__global__ void k_finish(const WorldDev *worlds, int cur_h, int cur_id, float thr)
{
    const WorldDev &wd = worlds[blockIdx.y];
    const uint32_t count = wd.ctl->acc_count;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t c = wd.acc_list[i];
        const unsigned long long m = wd.acc[c];
        wd.acc[c] = 0ull;
        const uint8_t value = (uint8_t)(m & 0xFFu);
        wd.acc_u8[c] = value;
        const uint8_t accId = (uint8_t)(255u - value);
        if (accId != 255 && wd.h[cur_h][c] >= thr) wd.id[cur_id][c] = accId;
    }
}

__global__ void k_bump_iteration(const WorldDev *worlds, int nworlds)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nworlds) worlds[i].ctl->iteration += 1u;
}

// Clears the previous step's decoded marks before this step's resolve.  Grid: (blocks, worlds).
__global__ void k_clear_acc_u8(const WorldDev *worlds)
{
    const WorldDev &wd = worlds[blockIdx.y];
    const uint32_t count = wd.ctl->acc_count;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        wd.acc_u8[wd.acc_list[i]] = 0;
}

}  // namespace

void gaussian_weights(float sigma, int radius, float *out)
{
    double tmp[2 * kMaxBlurRadius + 1];
    double sum = 0.0;
    for (int k = -radius; k <= radius; ++k) {
        tmp[k + radius] = exp(-(double)(k * k) / (2.0 * (double)sigma * (double)sigma));
        sum += tmp[k + radius];
    }
    for (int k = 0; k <= 2 * radius; ++k) out[k] = (float)(tmp[k] / sum);
}

int launch_resolve(Batch &b, cudaStream_t st)
{
    const tecto_settings &s = b.settings;
    ResolveParams p{};
    p.worlds = b.d_worlds;
    p.tiles = b.d_tiles[TK_RESOLVE];
    p.cur_h = b.cur_h;
    p.cur_id = b.cur_id;
    p.thr = s.kernel.continentalCrustThreshold;
    p.tmin = s.kernel.divergence_height_target_min;
    p.tmax = s.kernel.divergence_height_target_max;
    p.tfac = s.kernel.divergence_interpolation_factor;
    p.amount = s.step.upliftAmount;
    p.fricC = s.kernel.frictionCoefficientContinental;
    p.fricA = s.kernel.frictionCoefficientAccretion;
    p.fricS = s.kernel.frictionCoefficientSubduction;
    if (s.step.upliftMode == TECTO_UPLIFT_REFERENCE) {
        p.upl_h = b.upref.upl_h;
        p.upl_t = b.upref.upl_t;
        if (!p.upl_h) {
            set_error("reference uplift scratch not prepared");
            return TECTO_ERR_INVALID;
        }
    }
    int R = 0;
    if (s.step.upliftMode == TECTO_UPLIFT_GAUSSIAN) {
        R = s.step.upliftRadius;
        if (R < 0 || R > kMaxBlurRadius) {
            set_error("upliftRadius must be in 0..8");
            return TECTO_ERR_UNSUPPORTED;
        }
        gaussian_weights(s.step.upliftSigma, R, p.wts);
    }
    const unsigned grid = (unsigned)b.ntiles[TK_RESOLVE];
    if (s.step.plateDynamics == TECTO_PLATE_DYNAMICS_REFERENCE) {
        switch (R) {
            case 0: k_resolve<0, true><<<grid, 256, 0, st>>>(p); break;
            case 1: k_resolve<1, true><<<grid, 256, 0, st>>>(p); break;
            case 2: k_resolve<2, true><<<grid, 256, 0, st>>>(p); break;
            case 3: k_resolve<3, true><<<grid, 256, 0, st>>>(p); break;
            case 4: k_resolve<4, true><<<grid, 256, 0, st>>>(p); break;
            case 5: k_resolve<5, true><<<grid, 256, 0, st>>>(p); break;
            case 6: k_resolve<6, true><<<grid, 256, 0, st>>>(p); break;
            case 7: k_resolve<7, true><<<grid, 256, 0, st>>>(p); break;
            default: k_resolve<8, true><<<grid, 256, 0, st>>>(p); break;
        }
    } else switch (R) {
        case 0: k_resolve<0, false><<<grid, 256, 0, st>>>(p); break;
        case 1: k_resolve<1, false><<<grid, 256, 0, st>>>(p); break;
        case 2: k_resolve<2, false><<<grid, 256, 0, st>>>(p); break;
        case 3: k_resolve<3, false><<<grid, 256, 0, st>>>(p); break;
        case 4: k_resolve<4, false><<<grid, 256, 0, st>>>(p); break;
        case 5: k_resolve<5, false><<<grid, 256, 0, st>>>(p); break;
        case 6: k_resolve<6, false><<<grid, 256, 0, st>>>(p); break;
        case 7: k_resolve<7, false><<<grid, 256, 0, st>>>(p); break;
        default: k_resolve<8, false><<<grid, 256, 0, st>>>(p); break;
    }
    k_flip<<<dim3((kDivWords + 255) / 256, (unsigned)b.members.size()), 256, 0, st>>>(b.d_worlds);
    TECTO_CUDA(cudaGetLastError());
    b.launches += 2;
    b.cur_h ^= 1;
    b.cur_id ^= 1;
    return TECTO_OK;
}

int launch_finish(Batch &b, cudaStream_t st)
{
    if (b.settings.step.plateDynamics == TECTO_PLATE_DYNAMICS_REFERENCE) {
        const int rc = launch_plate_motion(b, st);  // executeIteration: before applyAccretion
        if (rc != TECTO_OK) return rc;
    }
    k_finish<<<dim3(4, (unsigned)b.members.size()), 256, 0, st>>>(b.d_worlds, b.cur_h, b.cur_id,
                                                                   b.settings.kernel.continentalCrustThreshold);
    TECTO_CUDA(cudaGetLastError());
    b.launches += 1;
    return TECTO_OK;
}

// Runs before launch_plates resets the list count: clears the previous step's decoded marks.
int launch_clear_marks(Batch &b, cudaStream_t st)
{
    k_clear_acc_u8<<<dim3(4, (unsigned)b.members.size()), 256, 0, st>>>(b.d_worlds);
    TECTO_CUDA(cudaGetLastError());
    b.launches += 1;
    return TECTO_OK;
}

int launch_bump_iteration(Batch &b, cudaStream_t st)
{
    const int n = (int)b.members.size();
    k_bump_iteration<<<(n + 255) / 256, 256, 0, st>>>(b.d_worlds, n);
    TECTO_CUDA(cudaGetLastError());
    b.launches += 1;
    return TECTO_OK;
}

}  // namespace tecto
