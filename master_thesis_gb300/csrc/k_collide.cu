// k_collide.cu - plate displacement, collision words from the sorted arrivals, collision-type
// evidence and the plate-pair type bitmap.  Reference: src/cuda_compute/plate_tectonics_kernel.cu.
#include "tecto_internal.cuh"

namespace tecto {

namespace {

// Per-plate integer displacement (getPixelMovements, :248-257) and the sub-cell centre update
// of applyPlateMovementChanges (:1871-1878), one block per world; the record before the update is
// kept in plates_prev for the kernels of the same step.  Also resets the world's per-step
// accretion list.  With plate dynamics it first turns the sums k_plate_stats left into each
// plate's mass, size and geometric centre (mergeAndCountSizeMass, calculatePlateCenters
// :2191-2226: the angular means back to cells through atan2), and clears them.  The reference
// computes no centre before its first iteration ends, so iteration 0 keeps the stored one.
__global__ void k_plates(const WorldDev *worlds, int dynamics)
{
    const WorldDev &wd = worlds[blockIdx.x];
    const int k = threadIdx.x;
    if (dynamics && k < kPlates) {
        PlateAcc &a = wd.pacc[k];
        tecto_plate_dynamics dd = wd.dyn[k];
        dd.mass = tecto_unfix((long long)a.mass, 1.0 / (double)kMassScale);
        dd.size = a.size;
        if (a.samples > 0 && wd.ctl->iteration > 0) {
            const float n = (float)a.samples;
            const float sx = tecto_unfix((long long)a.ang[0], 1.0 / (double)kAngScale) / n;
            const float cx = tecto_unfix((long long)a.ang[1], 1.0 / (double)kAngScale) / n;
            const float sy = tecto_unfix((long long)a.ang[2], 1.0 / (double)kAngScale) / n;
            const float cy = tecto_unfix((long long)a.ang[3], 1.0 / (double)kAngScale) / n;
            float gx = tecto_atan2f(sx, cx) * (float)wd.W / kTwoPiF;
            float gy = tecto_atan2f(sy, cy) * (float)wd.H / kTwoPiF;
            if (gx < 0.0f) gx += (float)wd.W;
            if (gy < 0.0f) gy += (float)wd.H;
            dd.geometricCenter_x = gx;
            dd.geometricCenter_y = gy;
        }
        wd.dyn[k] = dd;
        a.mass = 0ull;
        a.ang[0] = a.ang[1] = a.ang[2] = a.ang[3] = 0ull;
        a.size = 0;
        a.samples = 0;
    }
    if (k < kPlates) {
        tecto_plate p = wd.plates[k];
        wd.plates_prev[k] = p;  // the record the rest of the step sees in the reference
        const float mx = p.direction_x * p.velocity;
        const float my = p.direction_y * p.velocity;
        const float cx = p.pixelCenter_x + mx;
        const float cy = p.pixelCenter_y + my;
        const float fx = floorf(cx), fy = floorf(cy);
        wd.off[k] = make_int2((int)fx, (int)fy);
        p.pixelCenter_x = cx - fx;
        p.pixelCenter_y = cy - fy;
        wd.plates[k] = p;
    } else if (k == kPlates) {
        wd.off[k] = make_int2(0, 0);
    }
    if (k == 0) wd.ctl->acc_count = 0;
}

// writeCollision's classification (:794-836): returns category 0..4 or -1 to skip.  The early
// exit is the as-compiled `(packed & 1) && ((packed >> 4) & (15 < cooldown))` (:813).
__device__ __forceinline__ int evidence_category(const uint8_t *bm, uint8_t A, uint8_t B, float hA,
                                                 float hB, float thr, int cooldown, uint32_t *pair)
{
    const bool cond = A < B;
    const uint8_t mn = cond ? A : B, mx = cond ? B : A;
    const float mnH = cond ? hA : hB, mxH = cond ? hB : hA;
    const uint32_t idx = tri_index(mn, mx);
    *pair = idx;
    const uint32_t packed = __ldg(bm + idx);
    if ((packed & 1u) && ((packed >> 4) & (uint32_t)(0x0F < cooldown))) return -1;
    const bool minCont = mnH >= thr, maxCont = mxH >= thr;
    if (minCont && maxCont) return 4;
    if (minCont) return 2;
    if (maxCont) return 0;
    if (mnH <= mxH) return 1;
    return 3;
}

// Segmented winner pick over the sorted (destination, source) pairs of the whole batch: the
// first position of each destination's run builds the packed arrival word of
// registerPlateCollisions (:273-298) from its first four sources (ascending source order),
// writes zero words into the gap of destinations nobody moved into, and for convergent cells
// adds the collision-type evidence of the determineCollisionType kernel (:838-888) with
// warp-aggregated atomics.
__global__ __launch_bounds__(256) void k_words(const uint32_t *keys, const uint32_t *vals, uint32_t n,
                                               const WorldDev *worlds, const uint32_t *vbase, int nworlds,
                                               int cur_id, int cur_h, float thr, int cooldown)
{
    __shared__ uint32_t s_vbase[kMaxBatchWorlds + 1];
    for (int i = threadIdx.x; i <= nworlds; i += blockDim.x) s_vbase[i] = vbase[i];
    __syncthreads();
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned lane = threadIdx.x & 31u;
    const bool valid = j < n;
    bool leader = false;
    uint8_t ids[4] = {0, 0, 0, 0};
    float hs[4] = {0, 0, 0, 0};
    int cnt = 0;
    int wi = 0;
    if (valid) {
        const uint32_t key = keys[j];
        const uint32_t prev = j > 0 ? keys[j - 1] : 0xffffffffu;
        leader = j == 0 || prev != key;
        if (leader) {
            // gap of destinations without arrivals (they may belong to earlier worlds)
            const uint32_t gap0 = j == 0 ? 0u : prev + 1u;
            for (uint32_t c = gap0; c < key; ++c) {
                const WorldDev &gw = worlds[find_world(s_vbase, nworlds, c)];
                gw.word[c - gw.vbase] = 0u;
            }
            wi = find_world(s_vbase, nworlds, key);
            const WorldDev &wd = worlds[wi];
            uint32_t wv = 0;
            for (int k = 0; k < 4; ++k) {
                if (j + k >= n || keys[j + k] != key) break;
                const uint32_t src = vals[j + k] - wd.vbase;
                ids[k] = wd.id[cur_id][src];
                hs[k] = wd.h[cur_h][src];  // determineCollisionHeight: height at the arrival's source
                wv |= (uint32_t)(255u - ids[k]) << (8 * k);
                ++cnt;
            }
            wd.word[key - wd.vbase] = wv;
        }
        if (j == n - 1) {
            const uint32_t total = s_vbase[nworlds];  // vbase[n] holds the batch's cell count
            for (uint32_t c = key + 1u; c < total; ++c) {
                const WorldDev &gw = worlds[find_world(s_vbase, nworlds, c)];
                gw.word[c - gw.vbase] = 0u;
            }
        }
    }
    // pairs in determineCollisionType's order for 2, 3 and 4 arrivals (counts are sums, so the
    // order only has to cover the same pairs)
    const int npairs = cnt >= 4 ? 6 : cnt == 3 ? 3 : cnt == 2 ? 1 : 0;
    const uint8_t PA[6] = {0, 0, 0, 1, 1, 2};
    const uint8_t PB[6] = {1, 2, 3, 2, 3, 3};
    const uint8_t PA3[3] = {0, 0, 1};
    const uint8_t PB3[3] = {1, 2, 2};
    const uint8_t *bm = npairs ? worlds[wi].type_bitmap : nullptr;
#pragma unroll
    for (int slot = 0; slot < 6; ++slot) {
        uint32_t keyv = 0xffffffffu;
        uint32_t pair = 0;
        int cat = -1;
        if (slot < npairs) {
            const int a = cnt == 3 ? PA3[slot] : PA[slot];
            const int b = cnt == 3 ? PB3[slot] : PB[slot];
            cat = evidence_category(bm, ids[a], ids[b], hs[a], hs[b], thr, cooldown, &pair);
            // aggregation key: world, pair and category (worlds differ within a warp rarely)
            if (cat >= 0) keyv = ((uint32_t)wi * (uint32_t)kPairs + pair) * 5u + (uint32_t)cat;
        }
        const unsigned any = __ballot_sync(0xffffffffu, keyv != 0xffffffffu);
        if (any == 0) continue;
        const unsigned peers = __match_any_sync(0xffffffffu, keyv);
        if (keyv != 0xffffffffu && (peers & ((1u << lane) - 1u)) == 0)
            atomicAdd(&worlds[wi].counts[pair].c[cat], __popc(peers));
    }
}

// createCollisionTypeMatrix (:890-972) for every world of the batch; also clears the evidence.
__global__ void k_type_matrix(const WorldDev *worlds, int cooldown, int minSize)
{
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (uint32_t)kPairs) return;
    const WorldDev &wd = worlds[blockIdx.y];
    PairCounts *counts = wd.counts;
    uint8_t *bm = wd.type_bitmap;
    const PairCounts pc = counts[idx];
    const int *c = pc.c;
    const uint32_t total = (uint32_t)(c[0] + c[1] + c[2] + c[3] + c[4]);
    if (total == 0) return;  // no evidence: the counts are zero already
    int *cp = counts[idx].c;
    cp[0] = cp[1] = cp[2] = cp[3] = cp[4] = 0;
    const uint32_t packed = bm[idx];
    const bool hasType = packed & 1u;
    const int count = (int)((packed >> 4) & 0x0Fu);
    if (hasType && count < cooldown) {
        bm[idx] = (uint8_t)((packed & 0x0Fu) | (((uint32_t)(count + 1) & 0x0Fu) << 4));
        return;
    }
    if (total < (uint32_t)minSize) return;
    uint32_t out = packed & 0x0Fu;
    const bool hasPol = (packed >> 2) & 1u;
    const bool polA = (packed >> 3) & 1u;
    const int oppA = c[2] + c[4], oppB = c[0] + c[4];
    const int subA = c[0] + c[1] - oppA, subB = c[2] + c[3] - oppB;
    if (c[4] >= c[0] + c[1] && c[4] >= c[2] + c[3]) out |= 3u;
    else if (subA > 0 && subA > subB && (!hasPol || polA)) out = (out & ~2u) | 13u;
    else if (subB > 0 && subB > subA && (!hasPol || !polA)) out = (out & ~10u) | 5u;
    bm[idx] = (uint8_t)out;
}

}  // namespace

int launch_plates(Batch &b, cudaStream_t st)
{
    const int dyn = b.settings.step.plateDynamics;
    if (dyn != TECTO_PLATE_DYNAMICS_OFF && dyn != TECTO_PLATE_DYNAMICS_REFERENCE) {
        set_error("plateDynamics must be TECTO_PLATE_DYNAMICS_OFF or TECTO_PLATE_DYNAMICS_REFERENCE");
        return TECTO_ERR_UNSUPPORTED;
    }
    int rc = launch_clear_marks(b, st);  // must run before k_plates resets the list count
    if (rc != TECTO_OK) return rc;
    // plate dynamics and the plate policy read the per-plate mass, size and centre of the step
    const int stats = dyn != TECTO_PLATE_DYNAMICS_OFF || b.settings.step.platePolicy != 0;
    if (stats && (rc = launch_plate_stats(b, st)) != TECTO_OK) return rc;
    k_plates<<<(unsigned)b.members.size(), 256, 0, st>>>(b.d_worlds, stats);
    TECTO_CUDA(cudaGetLastError());
    b.launches += 1;
    return TECTO_OK;
}

int launch_sort_keys(Batch &b, cudaStream_t st)
{
    SortArgs a{};
    a.worlds = b.d_worlds;
    a.vbase = b.d_vbase;
    a.nworlds = (int)b.members.size();
    a.cur_id = b.cur_id;
    a.keys[0] = b.keys[0];
    a.keys[1] = b.keys[1];
    a.vals[0] = b.vals[0];
    a.vals[1] = b.vals[1];
    a.n = b.total;
    a.key_bits = key_bits_for(b.total);
    int half = 0;
    const int rc = run_sort(a, b.sort, st, &half);
    if (rc != TECTO_OK) return rc;
    b.sort_final = half;
    b.launches += 2 + (uint64_t)b.sort.passes;
    return TECTO_OK;
}

int launch_words(Batch &b, cudaStream_t st)
{
    const uint32_t n = (uint32_t)b.total;
    const tecto_kernel_settings &ks = b.settings.kernel;
    k_words<<<(n + 255) / 256, 256, 0, st>>>(b.keys[b.sort_final], b.vals[b.sort_final], n, b.d_worlds,
                                             b.d_vbase, (int)b.members.size(), b.cur_id, b.cur_h,
                                             ks.continentalCrustThreshold, ks.collisionTypeUpdateCooldown);
    TECTO_CUDA(cudaGetLastError());
    b.launches += 1;
    return TECTO_OK;
}

int launch_type_matrix(Batch &b, cudaStream_t st)
{
    const tecto_kernel_settings &ks = b.settings.kernel;
    const dim3 grid((kPairs + 255) / 256, (unsigned)b.members.size());
    k_type_matrix<<<grid, 256, 0, st>>>(b.d_worlds, ks.collisionTypeUpdateCooldown, ks.minCollisionSize);
    TECTO_CUDA(cudaGetLastError());
    b.launches += 1;
    return TECTO_OK;
}

}  // namespace tecto
