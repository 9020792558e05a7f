// k_policy.cu - plate policy after a step: the relabel of plate fragments after each CCL and the
// merges of touching plates that move alike.
// Reference: PlateTectonicSim::applyCCL (src/cuda_compute/plate_tectonic_sim.cu:374-467) and
// mergePlates (:470-494) with their kernels in src/cuda_compute/plate_tectonics_kernel.cu
// (createPlateIdLabelMap :1394-1405, getMaxSizeLabels :3114-3128, createLabelIdLookup :3130-3185,
// postCClIdReassign :3187-3206, assignUnassignedIdsToNeighbor :2052-2101, getNeighboringPlates
// :1283-1311, getPlateMerges :1313-1379, clearCollisionTypes :1381-1392, mergeAndCountSizeMass
// :100-135).
//
// The reference ranks the components with thrust sorts and assigns free plate ids and merge
// partners with atomics in thread order, so which fragment receives which id, and which of two
// competing merges wins, depends on scheduling; its neighbour fill writes in place while other
// threads read.  The engine fixes one order, the one a sequential run of the reference's kernels
// gives (components by size, then label, both descending; free ids ascending; merge pairs in
// ascending (larger id, smaller id) order), and fills unassigned cells in rounds that each read the
// previous round's ids.  The ranking is the engine's own: a radix select of the 255 largest
// (count, label) keys inside one block per world, no library sort.
//
// Scratch (free at the end of a step): the rain field holds the component sizes and then the
// unassigned list, s1 the per-label lookup and then the fill's pending ids, the split path's
// velocity field the component keys.
#include "tecto_internal.cuh"

namespace tecto {

namespace {

// The world of this block when its labelling ran this step (period 0: always).
__device__ __forceinline__ bool relabel_due(const WorldDev &wd, int period)
{
    return period == 0 || wd.ctl->iteration % (uint32_t)period == 0u;
}

// Component sizes: clear, then count the cells of each label; then the roots' keys; then the ids.
// Grid: TK_STATS tiles, one column of a tile per thread.
template <int PHASE>
__global__ __launch_bounds__(256) void k_rl_cells(const WorldDev *worlds, const uint2 *tiles, int cur_id,
                                                  int period)
{
    int wi, tx, ty;
    tile_of(tiles[blockIdx.x], &wi, &tx, &ty);
    const WorldDev &wd = worlds[wi];
    if (!relabel_due(wd, period)) return;
    const int x = tx * kStatTileX + (int)threadIdx.x;
    if (x >= wd.W) return;
    const int y0 = ty * kStatTileY, y1 = min(y0 + kStatTileY, wd.H);
    uint32_t *count = reinterpret_cast<uint32_t *>(wd.rain);
    uint32_t *lookup = reinterpret_cast<uint32_t *>(wd.s1);
    unsigned long long *keys = reinterpret_cast<unsigned long long *>(wd.vel);
    uint8_t *id = wd.id[cur_id];
    if (PHASE == 1) {
        // cells down a column mostly share a label: count runs in a register, one atomic per run
        uint32_t run = 0xffffffffu, n = 0u;
        for (int y = y0; y < y1; ++y) {
            const uint32_t lab = wd.labels[(uint32_t)y * (uint32_t)wd.W + (uint32_t)x];
            if (lab != run) {
                if (n) atomicAdd(count + run, n);
                run = lab;
                n = 0u;
            }
            ++n;
        }
        if (n) atomicAdd(count + run, n);
        return;
    }
    for (int y = y0; y < y1; ++y) {
        const uint32_t i = (uint32_t)y * (uint32_t)wd.W + (uint32_t)x;
        if (PHASE == 0) {
            count[i] = 0u;
        } else if (PHASE == 2) {
            // roots: one key per component, the plate's largest component, a cleared lookup entry
            if (wd.labels[i] == i) {
                const uint32_t c = count[i];
                const uint32_t slot = atomicAdd(&wd.ctl->comp_count, 1u);
                keys[slot] = ((unsigned long long)c << 32) | (unsigned long long)i;
                atomicMax(&wd.policy->max_count[id[i]], (int)c);
                lookup[i] = 255u;
            }
        } else {
            // postCClIdReassign: every cell takes its component's id; cells left without one are listed
            const uint8_t nid = (uint8_t)lookup[wd.labels[i]];
            id[i] = nid;
            if (nid == 255) {
                const uint32_t slot = atomicAdd(&wd.ctl->unassigned, 1u);
                count[slot] = i;  // the size counts are no longer needed: the list reuses them
            }
        }
    }
}

constexpr int kSelThreads = 1024;

// Ranking and id assignment, one block per world: radix select of the min(255, M) largest
// (count << 32 | label) keys, their order, then createLabelIdLookup's decisions in that order.
__global__ __launch_bounds__(kSelThreads) void k_rl_select(const WorldDev *worlds, int cur_id, int period,
                                                           int minPlateSize)
{
    const WorldDev &wd = worlds[blockIdx.x];
    if (!relabel_due(wd, period)) return;
    __shared__ unsigned int hist[256];
    __shared__ unsigned long long s_prefix, s_mask;
    __shared__ unsigned int s_need;
    __shared__ unsigned long long s_top[256];
    __shared__ unsigned int s_ntop;
    const unsigned long long *keys = reinterpret_cast<const unsigned long long *>(wd.vel);
    const uint32_t M = wd.ctl->comp_count;
    const uint32_t K = M < (uint32_t)kPlates ? M : (uint32_t)kPlates;
    const int t = threadIdx.x;
    if (t == 0) {
        s_prefix = 0ull;
        s_mask = 0ull;
        s_need = K;
        s_ntop = 0u;
    }
    __syncthreads();
    if (K > 0u && K < M) {
        // MSD radix select, 8 bits per pass: after the last pass s_prefix is the K-th largest key
        for (int shift = 56; shift >= 0; shift -= 8) {
            for (int b = t; b < 256; b += kSelThreads) hist[b] = 0u;
            __syncthreads();
            const unsigned long long pre = s_prefix, msk = s_mask;
            for (uint32_t j = t; j < M; j += kSelThreads) {
                const unsigned long long k = keys[j];
                if ((k & msk) == pre) atomicAdd(&hist[(k >> shift) & 255ull], 1u);
            }
            __syncthreads();
            if (t == 0) {
                unsigned int above = 0u, need = s_need;
                int d = 255;
                for (; d > 0; --d) {
                    if (above + hist[d] >= need) break;
                    above += hist[d];
                }
                s_need = need - above;
                s_prefix = pre | ((unsigned long long)d << shift);
                s_mask = msk | (255ull << shift);
            }
            __syncthreads();
        }
    }
    const unsigned long long thr = (K < M) ? s_prefix : 0ull;
    for (uint32_t j = t; j < M && K > 0u; j += kSelThreads) {
        const unsigned long long k = keys[j];
        if (k >= thr) {
            const unsigned int slot = atomicAdd(&s_ntop, 1u);
            if (slot < 256u) s_top[slot] = k;
        }
    }
    __syncthreads();
    // order: rank of each selected key among the selected (keys are distinct), descending
    const uint32_t n = min(s_ntop, K);
    unsigned long long mine = 0ull;
    uint32_t rank = 0u;
    if ((uint32_t)t < n) {
        mine = s_top[t];
        for (uint32_t j = 0; j < n; ++j) rank += s_top[j] > mine ? 1u : 0u;
    }
    __syncthreads();
    if ((uint32_t)t < n) wd.policy->top[rank] = mine;
    __syncthreads();
    if (t == 0) {
        // createLabelIdLookup: free ids are those below min(255, components) whose plate has no cells
        uint8_t avail[kPlates];
        int navail = 0, next = 0;
        for (uint32_t k = 0; k < n; ++k)
            if (wd.dyn[k].size == 0) avail[navail++] = (uint8_t)k;
        uint32_t *lookup = reinterpret_cast<uint32_t *>(wd.s1);
        const uint8_t *id = wd.id[cur_id];
        for (uint32_t r = 0; r < n; ++r) {
            const unsigned long long k = wd.policy->top[r];
            const uint32_t label = (uint32_t)(k & 0xFFFFFFFFull);
            const int c = (int)(k >> 32);
            const uint8_t plate = id[label];
            if (c == wd.policy->max_count[plate]) {
                lookup[label] = plate;
            } else if (c >= minPlateSize && next < navail) {
                const uint8_t nid = avail[next++];
                wd.plates[nid] = wd.plates[plate];
                wd.dyn[nid] = wd.dyn[plate];
                lookup[label] = nid;
            }
        }
        for (int p = 0; p < 256; ++p) wd.policy->max_count[p] = 0;
        wd.ctl->comp_count = 0u;
    }
}

// assignUnassignedIdsToNeighbor in rounds, one block per world: each listed cell still without an id
// takes the most frequent id among its eight neighbours (first on ties) as they stood at the start
// of the round; stops when none is left or a round assigns nothing.
__global__ __launch_bounds__(1024) void k_rl_fill(const WorldDev *worlds, int cur_id, int period)
{
    const WorldDev &wd = worlds[blockIdx.x];
    if (!relabel_due(wd, period)) return;
    __shared__ unsigned int s_assigned, s_left;
    const uint32_t n = wd.ctl->unassigned;
    const uint32_t *list = reinterpret_cast<const uint32_t *>(wd.rain);
    uint32_t *pending = reinterpret_cast<uint32_t *>(wd.s1);
    uint8_t *id = wd.id[cur_id];
    const int W = wd.W, H = wd.H;
    const int OX[8] = {1, -1, 0, 0, 1, 1, -1, -1}, OY[8] = {0, 0, 1, -1, 1, -1, 1, -1};
    if (threadIdx.x == 0) {
        s_left = n;
        s_assigned = 0u;
    }
    __syncthreads();
    for (uint32_t round = 0; round <= n && n > 0u; ++round) {
        for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
            const uint32_t c = list[j];
            uint32_t sel = 255u;
            if (id[c] == 255) {
                const int x = (int)(c % (uint32_t)W), y = (int)(c / (uint32_t)W);
                uint8_t nb[8];
                int m = 0;
                for (int k = 0; k < 8; ++k) {
                    const uint8_t v = id[cidx(x + OX[k], y + OY[k], W, H)];
                    if (v != 255) nb[m++] = v;
                }
                int best = 0;
                for (int a = 0; a < m; ++a) {
                    int cnt = 1;
                    for (int b = 0; b < m; ++b) cnt += (a != b && nb[b] == nb[a]) ? 1 : 0;
                    if (cnt > best) {
                        best = cnt;
                        sel = nb[a];
                    }
                }
            }
            pending[j] = sel;
        }
        __syncthreads();
        for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
            if (pending[j] != 255u) {
                id[list[j]] = (uint8_t)pending[j];
                atomicAdd(&s_assigned, 1u);
            }
        }
        __syncthreads();
        const unsigned int assigned = s_assigned;
        __syncthreads();  // every thread has read the count before it is reset
        if (threadIdx.x == 0) {
            s_left -= assigned;
            s_assigned = 0u;
        }
        __syncthreads();
        if (assigned == 0u || s_left == 0u) break;
    }
    if (threadIdx.x == 0) {
        wd.ctl->unresolved = s_left;
        wd.ctl->unassigned = 0u;
    }
}

// getNeighboringPlates: plate pairs that touch across a +x or +y edge (wrapped), as triangle bits.
__global__ __launch_bounds__(256) void k_mg_neighbors(const WorldDev *worlds, const uint2 *tiles, int cur_id)
{
    int wi, tx, ty;
    tile_of(tiles[blockIdx.x], &wi, &tx, &ty);
    const WorldDev &wd = worlds[wi];
    const int x = tx * kStatTileX + (int)threadIdx.x;
    if (x >= wd.W) return;
    const int y0 = ty * kStatTileY, y1 = min(y0 + kStatTileY, wd.H);
    const uint8_t *id = wd.id[cur_id];
    const int xr = x + 1 == wd.W ? 0 : x + 1;
    uint32_t *bits = wd.policy->neighbors;
    for (int y = y0; y < y1; ++y) {
        const size_t row = (size_t)y * (size_t)wd.W;
        const uint8_t c = id[row + x], r = id[row + xr];
        const uint8_t t = id[(size_t)(y + 1 == wd.H ? 0 : y + 1) * (size_t)wd.W + x];
        if (c != r && c != 255 && r != 255) {
            const uint32_t b = tri_index(min(c, r), max(c, r));
            atomicOr(bits + b / 32u, 1u << (b % 32u));
        }
        if (c != t && c != 255 && t != 255) {
            const uint32_t b = tri_index(min(c, t), max(c, t));
            atomicOr(bits + b / 32u, 1u << (b % 32u));
        }
    }
}

struct MergeParams {
    float minVel, dotThr, velDiffThr;
    int maxArea;
};

constexpr int kMaxCand = 2048;

// getPlateMerges' test for touching plates x < y (:1331-1350).
__device__ __forceinline__ bool merge_test(const WorldDev &wd, int x, int y, const MergeParams &mp)
{
    const tecto_plate_dynamics dx = wd.dyn[x], dy = wd.dyn[y];
    const float dot = dx.directionSmoothed_x * dy.directionSmoothed_x + dx.directionSmoothed_y * dy.directionSmoothed_y;
    const float vdiff = fabsf(dx.velocitySmoothed - dy.velocitySmoothed);
    const bool slow = wd.plates[x].velocity <= mp.minVel && wd.plates[y].velocity <= mp.minVel;
    const bool alike = dot >= mp.dotThr && vdiff <= mp.velDiffThr;
    if (!slow && !alike) return false;
    if (dx.mergeWaitTime > 0 || dy.mergeWaitTime > 0) return false;
    return dx.size + dy.size <= mp.maxArea;
}

// getPlateMerges, one block per world: the pairs that touch and pass the merge test are collected,
// put in ascending (larger id, smaller id) order and decided one after another as a sequential run
// of the reference's atomics would; each merge clears the bitmap entries clearCollisionTypes
// addresses; the neighbour bits are cleared for the next step.
__global__ __launch_bounds__(1024) void k_mg_decide(const WorldDev *worlds, MergeParams mp)
{
    const WorldDev &wd = worlds[blockIdx.x];
    __shared__ unsigned int s_cand[kMaxCand];
    __shared__ unsigned int s_n;
    __shared__ int s_merge[256];
    const int t = threadIdx.x;
    if (t == 0) s_n = 0u;
    for (int p = t; p < 256; p += blockDim.x) s_merge[p] = 0;
    __syncthreads();
    PolicyState &ps = *wd.policy;
    for (uint32_t b = t; b < (uint32_t)kPairs; b += blockDim.x) {
        if (!(ps.neighbors[b / 32u] & (1u << (b % 32u)))) continue;
        // pair (x, y), x < y, of triangle index b
        int x = 0;
        uint32_t base = 0u;
        while (base + (uint32_t)(kPlates - 1 - x) <= b) {
            base += (uint32_t)(kPlates - 1 - x);
            ++x;
        }
        const int y = x + 1 + (int)(b - base);
        if (!merge_test(wd, x, y, mp)) continue;
        const unsigned int slot = atomicAdd(&s_n, 1u);
        if (slot < (unsigned int)kMaxCand) s_cand[slot] = (unsigned int)y * (unsigned int)kPlates + (unsigned int)x;
    }
    __syncthreads();
    const unsigned int n = min(s_n, (unsigned int)kMaxCand);
    // ascending order of the candidates (distinct): rank sort
    unsigned int mine[2] = {0u, 0u}, rank[2] = {0u, 0u};
    for (int r = 0; r < 2; ++r) {
        const unsigned int j = (unsigned int)t + (unsigned int)r * blockDim.x;
        if (j < n) {
            mine[r] = s_cand[j];
            for (unsigned int q = 0; q < n; ++q) rank[r] += s_cand[q] < mine[r] ? 1u : 0u;
        }
    }
    __syncthreads();
    for (int r = 0; r < 2; ++r) {
        const unsigned int j = (unsigned int)t + (unsigned int)r * blockDim.x;
        if (j < n) s_cand[rank[r]] = mine[r];
    }
    __syncthreads();
    if (t == 0) {
        int merges = 0;
        const bool all = s_n > (unsigned int)kMaxCand;  // too many candidates to list: scan every pair
        const unsigned int count = all ? (unsigned int)(kPlates * kPlates) : n;
        for (unsigned int q = 0; q < count; ++q) {
            const unsigned int pi = all ? q : s_cand[q];
            const int x = (int)(pi % (unsigned int)kPlates), y = (int)(pi / (unsigned int)kPlates);
            if (all) {
                if (x >= y) continue;
                const uint32_t b = tri_index((uint32_t)x, (uint32_t)y);
                if (!(ps.neighbors[b / 32u] & (1u << (b % 32u)))) continue;
                if (!merge_test(wd, x, y, mp)) continue;
            }
            const bool x_parent = wd.dyn[y].mass <= wd.dyn[x].mass;
            if (s_merge[x] != 0) continue;
            s_merge[x] = x_parent ? -1 : kPlates - y;
            if (s_merge[y] != 0) {
                s_merge[x] = 0;
                continue;
            }
            s_merge[y] = x_parent ? kPlates - x : -1;
            const int parent = x_parent ? x : y;
            for (int k = 0; k < kPlates; ++k)
                if (k != parent) wd.type_bitmap[k < parent ? k : parent] = 0;
            ++merges;
        }
        ps.any_merge = merges;
        wd.ctl->merges = (uint32_t)merges;
    }
    __syncthreads();
    for (int p = t; p < 256; p += blockDim.x) ps.merge_ids[p] = s_merge[p];
    for (uint32_t w = t; w < (uint32_t)kDivWords; w += blockDim.x) ps.neighbors[w] = 0u;
}

// mergeAndCountSizeMass's remap: a child's cells take the parent's id.
__global__ __launch_bounds__(256) void k_mg_apply(const WorldDev *worlds, const uint2 *tiles, int cur_id)
{
    int wi, tx, ty;
    tile_of(tiles[blockIdx.x], &wi, &tx, &ty);
    const WorldDev &wd = worlds[wi];
    if (wd.policy->any_merge == 0) return;
    __shared__ int s_merge[256];
    for (int p = threadIdx.x; p < 256; p += blockDim.x) s_merge[p] = wd.policy->merge_ids[p];
    __syncthreads();
    const int x = tx * kStatTileX + (int)threadIdx.x;
    if (x >= wd.W) return;
    const int y0 = ty * kStatTileY, y1 = min(y0 + kStatTileY, wd.H);
    uint8_t *id = wd.id[cur_id];
    for (int y = y0; y < y1; ++y) {
        const size_t i = (size_t)y * (size_t)wd.W + (size_t)x;
        const int m = s_merge[id[i]];
        if (m > 0) id[i] = (uint8_t)(kPlates - m);
    }
}

}  // namespace

int launch_plate_policy(Batch &b, int ccl, cudaStream_t st)
{
    const tecto_settings &s = b.settings;
    const int pol = s.step.platePolicy;
    if (pol & ~(TECTO_PLATE_RELABEL | TECTO_PLATE_MERGE)) {
        set_error("platePolicy: only TECTO_PLATE_RELABEL and TECTO_PLATE_MERGE bits");
        return TECTO_ERR_UNSUPPORTED;
    }
    const unsigned grid = (unsigned)b.ntiles[TK_STATS];
    const uint2 *tiles = b.d_tiles[TK_STATS];
    const unsigned nw = (unsigned)b.members.size();
    if ((pol & TECTO_PLATE_RELABEL) && ccl) {
        const int period = ccl == 2 ? (s.sim.iterationsForCCL > 0 ? s.sim.iterationsForCCL : 1) : 0;
        k_rl_cells<0><<<grid, 256, 0, st>>>(b.d_worlds, tiles, b.cur_id, period);
        k_rl_cells<1><<<grid, 256, 0, st>>>(b.d_worlds, tiles, b.cur_id, period);
        k_rl_cells<2><<<grid, 256, 0, st>>>(b.d_worlds, tiles, b.cur_id, period);
        k_rl_select<<<nw, kSelThreads, 0, st>>>(b.d_worlds, b.cur_id, period, s.kernel.minPlateSize);
        k_rl_cells<3><<<grid, 256, 0, st>>>(b.d_worlds, tiles, b.cur_id, period);
        k_rl_fill<<<nw, 1024, 0, st>>>(b.d_worlds, b.cur_id, period);
        TECTO_CUDA(cudaGetLastError());
        b.launches += 6;
    }
    if (pol & TECTO_PLATE_MERGE) {
        const MergeParams mp{s.kernel.mergeMinVelocity, s.kernel.mergeDotDirectionThreshold,
                             s.kernel.mergeVelocityDiffThreshold, s.kernel.targetMaximumPlateArea};
        k_mg_neighbors<<<grid, 256, 0, st>>>(b.d_worlds, tiles, b.cur_id);
        k_mg_decide<<<nw, 1024, 0, st>>>(b.d_worlds, mp);
        k_mg_apply<<<grid, 256, 0, st>>>(b.d_worlds, tiles, b.cur_id);
        TECTO_CUDA(cudaGetLastError());
        b.launches += 3;
    }
    return TECTO_OK;
}

}  // namespace tecto
