// k_uplift.cu - the reference's uplift (TECTO_UPLIFT_REFERENCE) over a batch of worlds.
//
// Reference: plate_tectonic_sim.cu:270-317 with moveContinentalCollisions and
// combinePropagatedCollisions (src/cuda_compute/plate_tectonics_kernel.cu:975-1218), the JFA
// kernels (:1498-1600) and applyUplift (:1646-1738).
//
// moveContinentalCollisions lets every continental collision cell march against each involved
// plate's motion and insert the plate pair into the cells it reaches with a compare-and-swap loop
// that fails once four plates are registered, then spread its height sum over the cells it
// reached with float atomicAdd.  Both results depend on the order in which threads arrive.  The
// engine fixes that order to ascending source cell (the order of a one-thread-at-a-time run, which
// the CPU oracle and the reference kernels run in sequence also follow):
//   1. every source cell emits its insert events (source, slot, plate pair) into per-target
//      buckets (count, exclusive scan, fill);
//   2. one thread per target sorts its bucket by (source, slot) and applies the inserts in that
//      order, marking which events succeeded;
//   3. every source replays its counts from the success bits and emits its height contributions
//      into a second set of buckets, which one thread per target sums in (source, position) order.
// Then combine + JFA initialisation, the JFA passes (each world with its own step sequence inside
// one launch per step), and the distance and applyUplift per cell.
#include <algorithm>

#include "tecto_internal.cuh"

namespace tecto {

namespace {

constexpr int kUpThreads = 256;
constexpr int kScanItems = 4;                          // per thread in the block scan
constexpr int kScanBlock = 1024 * kScanItems;          // cells per scan block

struct UpArgs {
    const WorldDev *worlds;
    const uint32_t *vbase;
    int nworlds;
    uint32_t total;
    int cur_h, cur_id;       // halves written by resolve; heights before the step at cur_h ^ 1
    UpliftRefScratch u;
    float prop_thr;          // continentalPropThreshold
    int prop_iters;          // continentalPropMaxIters
    float under_mult, over_mult, cont_mult, min_clamp, max_clamp;
    int over_range;
};

__device__ __forceinline__ void load_vbase(const UpArgs &a, uint32_t *s)
{
    for (int i = threadIdx.x; i <= a.nworlds; i += blockDim.x) s[i] = a.vbase[i];
    __syncthreads();
}

// continentalPropagation (:975-1027); the returned coordinate is not wrapped (comparisons in the
// reference use the unwrapped value, accesses wrap)
__device__ int2 cont_prop(const float *h_old, int W, int H, int2 p, const tecto_plate &pd, float start,
                          float thr, int iters)
{
    if (start < thr) return p;
    const float posx = (float)p.x + pd.pixelCenter_x, posy = (float)p.y + pd.pixelCenter_y;
    const float ndx = -pd.direction_x, ndy = -pd.direction_y;
    const int stepX = ndx > 0 ? 1 : -1, stepY = ndy > 0 ? 1 : -1;
    const float tdx = fabsf(1.0f / ndx), tdy = fabsf(1.0f / ndy);
    const int nextX = stepX > 0 ? p.x + 1 : p.x, nextY = stepY > 0 ? p.y + 1 : p.y;
    float tmx = ((float)nextX - posx) / ndx;
    float tmy = ((float)nextY - posy) / ndy;
    int2 prev = p;
    for (int i = 0; i < iters; ++i) {
        if (tmx < tmy) {
            p.x += stepX;
            tmx = tmx + tdx;
        } else {
            p.y += stepY;
            tmy = tmy + tdy;
        }
        if (h_old[cidx(p.x, p.y, W, H)] < thr) return p;
        prev = p;
    }
    return prev;
}

// One continental collision source: the cell its primary plate reaches and, per arrival slot k,
// the secondary plate (-1 none) and the cell it reaches.
struct Source {
    int primary;
    int2 pp;
    int sec[4];
    int2 sp[4];
};

__device__ __forceinline__ bool source_of(const UpArgs &a, const WorldDev &wd, uint32_t v, uint32_t local,
                                          Source &s)
{
    const uint32_t cp = wd.word[local];
    if ((cp >> 8) == 0u) return false;
    const uint32_t ut = a.u.upl_t[v];
    if ((ut & 1u) != 1u) return false;
    const int pidx = (int)((ut >> 1) & 3u);
    s.primary = 255 - (int)((cp >> (8 * pidx)) & 0xFFu);
    if (s.primary >= kPlates) return false;  // the owner's slot always holds a plate
    const int W = wd.W, H = wd.H;
    const int2 pos = make_int2((int)(local % (uint32_t)W), (int)(local / (uint32_t)W));
    const float *h_old = wd.h[a.cur_h ^ 1];
    const float cur = h_old[local];
    s.pp = cont_prop(h_old, W, H, pos, wd.plates_prev[s.primary], cur, a.prop_thr, a.prop_iters);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int sec = 255 - (int)((cp >> (8 * k)) & 0xFFu);
        s.sec[k] = (sec == 255 || sec == s.primary) ? -1 : sec;
        s.sp[k] = s.pp;
        if (s.sec[k] >= 0)
            s.sp[k] = cont_prop(h_old, W, H, pos, wd.plates_prev[sec], cur, a.prop_thr, a.prop_iters);
    }
    return true;
}

__device__ __forceinline__ bool same(int2 a, int2 b) { return a.x == b.x && a.y == b.y; }

// Append one bucket entry (FILL) or count it.
template <bool FILL>
__device__ __forceinline__ void emit(const UpArgs &a, const WorldDev &wd, uint32_t target, uint32_t key,
                                     uint32_t val)
{
    if (!FILL) {
        atomicAdd(a.u.cnt + target, 1u);
        return;
    }
    const size_t pos = (size_t)a.u.off[target] + atomicAdd(a.u.cnt + target, 1u);
    if (pos >= a.u.ecap) {
        atomicOr(&wd.ctl->error, kErrUpliftCapacity);
        return;
    }
    a.u.ent_key[pos] = key;
    a.u.ent_val[pos] = val;
}

// Clears this step's propagation state.
__global__ void k_up_clear(UpArgs a)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.total; v += gridDim.x * blockDim.x) {
        a.u.cnt[v] = 0u;
        a.u.succ[v] = 0u;
        a.u.prop_h[v] = 0.0f;
        a.u.prop_inv[v] = 0u;
        a.u.prop_t[v] = 0u;
    }
}

// Step 1: insert events of every source, slot 2k (primary's cell) and 2k + 1 (secondary's cell
// when it differs), payload primary | secondary << 8.
template <bool FILL>
__global__ __launch_bounds__(kUpThreads) void k_up_inserts(UpArgs a)
{
    __shared__ uint32_t s_vbase[kMaxBatchWorlds + 1];
    load_vbase(a, s_vbase);
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.total; v += gridDim.x * blockDim.x) {
        const WorldDev &wd = a.worlds[find_world(s_vbase, a.nworlds, v)];
        Source s;
        if (!source_of(a, wd, v, v - wd.vbase, s)) continue;
        for (int k = 0; k < 4; ++k) {
            if (s.sec[k] < 0) continue;
            const uint32_t pair = (uint32_t)s.primary | ((uint32_t)s.sec[k] << 8);
            emit<FILL>(a, wd, wd.vbase + cidx(s.pp.x, s.pp.y, wd.W, wd.H), (v << 3) | (uint32_t)(2 * k), pair);
            if (!same(s.pp, s.sp[k]))
                emit<FILL>(a, wd, wd.vbase + cidx(s.sp[k].x, s.sp[k].y, wd.W, wd.H), (v << 3) | (uint32_t)(2 * k + 1),
                           pair);
        }
    }
}

// Bucket of target v holding n entries, sorted by key in place (insertion sort; buckets are
// short).  Returns the entry count that fits the scratch.
__device__ __forceinline__ uint32_t sorted_bucket(const UpArgs &a, uint32_t v, uint32_t n, size_t *base)
{
    const size_t b = a.u.off[v];
    *base = b;
    if (n == 0u || b >= a.u.ecap) return 0u;
    if (b + n > a.u.ecap) n = (uint32_t)(a.u.ecap - b);
    for (uint32_t i = 1; i < n; ++i) {
        const uint32_t k = a.u.ent_key[b + i], val = a.u.ent_val[b + i];
        uint32_t j = i;
        while (j > 0 && a.u.ent_key[b + j - 1] > k) {
            a.u.ent_key[b + j] = a.u.ent_key[b + j - 1];
            a.u.ent_val[b + j] = a.u.ent_val[b + j - 1];
            --j;
        }
        a.u.ent_key[b + j] = k;
        a.u.ent_val[b + j] = val;
    }
    return n;
}

// atomicInsertPlatePair (:1029-1071) executed alone
__device__ __forceinline__ bool insert_pair(uint32_t &inv, uint32_t a, uint32_t b)
{
    uint32_t ins[2] = {255u - a, 255u - b};
    const uint32_t old = inv;
    uint32_t nw = old;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const uint32_t pl = (old >> (8 * i)) & 0xFFu;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            if (pl == 0u && ins[j] != 0u) {
                nw |= ins[j] << (8 * i);
                ins[j] = 0u;
                break;
            }
            if (pl == ins[j]) ins[j] = 0u;
        }
    }
    if (ins[0] != 0u || ins[1] != 0u) return false;
    inv = nw;
    return true;
}

// Step 2: per target, the inserts in (source, slot) order.
__global__ __launch_bounds__(kUpThreads) void k_up_apply_inserts(UpArgs a)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.total; v += gridDim.x * blockDim.x) {
        size_t b;
        const uint32_t raw = a.u.cnt[v];
        a.u.cnt[v] = 0u;  // the contribution pass counts into the same array
        const uint32_t n = sorted_bucket(a, v, raw, &b);
        if (n == 0u) continue;
        uint32_t inv = 0u;
        for (uint32_t i = 0; i < n; ++i) {
            const uint32_t key = a.u.ent_key[b + i], val = a.u.ent_val[b + i];
            if (insert_pair(inv, val & 0xFFu, (val >> 8) & 0xFFu)) atomicOr(a.u.succ + (key >> 3), 1u << (key & 7u));
        }
        a.u.prop_inv[v] = inv;
    }
}

// countCollision (:1073-1085)
__device__ __forceinline__ void count_at(int2 pos, int2 *positions, int *counts, int &total, int inc)
{
    for (int i = 0; i < 6; ++i)
        if (counts[i] == 0 || same(positions[i], pos)) {
            positions[i] = pos;
            counts[i] += inc;
            total += inc;
            return;
        }
}

// Step 3a: each source's height contributions (the tail of moveContinentalCollisions,
// :1131-1184), keyed (source, position index), payload the float's bits.
template <bool FILL>
__global__ __launch_bounds__(kUpThreads) void k_up_contrib(UpArgs a)
{
    __shared__ uint32_t s_vbase[kMaxBatchWorlds + 1];
    load_vbase(a, s_vbase);
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.total; v += gridDim.x * blockDim.x) {
        const WorldDev &wd = a.worlds[find_world(s_vbase, a.nworlds, v)];
        Source s;
        if (!source_of(a, wd, v, v - wd.vbase, s)) continue;
        const uint32_t ok = a.u.succ[v];
        int2 positions[6];
        int counts[6] = {0, 0, 0, 0, 0, 0};
        int total = 0;
        for (int k = 0; k < 4; ++k) {
            if (s.sec[k] < 0) continue;
            if (same(s.pp, s.sp[k])) {
                if ((ok >> (2 * k)) & 1u) count_at(s.pp, positions, counts, total, 2);
            } else {
                if ((ok >> (2 * k)) & 1u) count_at(s.pp, positions, counts, total, 1);
                if ((ok >> (2 * k + 1)) & 1u) count_at(s.sp[k], positions, counts, total, 1);
            }
            count_at(s.pp, positions, counts, total, 1);
            count_at(s.sp[k], positions, counts, total, 1);
        }
        const float uh = a.u.upl_h[v];
        for (int i = 0; i < 6; ++i) {
            if (counts[i] == 0) break;
            const float value = (uh / (float)total) * (float)counts[i];
            emit<FILL>(a, wd, wd.vbase + cidx(positions[i].x, positions[i].y, wd.W, wd.H), (v << 3) | (uint32_t)i,
                       __float_as_uint(value));
        }
    }
}

// Step 3b: per target, the contributions summed in (source, position) order onto 0.
__global__ __launch_bounds__(kUpThreads) void k_up_sum(UpArgs a)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.total; v += gridDim.x * blockDim.x) {
        size_t b;
        const uint32_t n = sorted_bucket(a, v, a.u.cnt[v], &b);
        if (n == 0u) continue;
        float acc = 0.0f;
        for (uint32_t i = 0; i < n; ++i) acc = acc + __uint_as_float(a.u.ent_val[b + i]);
        a.u.prop_h[v] = acc;
    }
}

// combinePropagatedCollisions (:1187-1218) and JFAInitialize (:1498-1510).  Cells with fewer than
// two arrivals never become seeds, so the engine does not keep UpliftData from earlier steps there
// (the reference's buffer persists; its stale values only reach non-seed cells).
__global__ __launch_bounds__(kUpThreads) void k_up_combine(UpArgs a)
{
    __shared__ uint32_t s_vbase[kMaxBatchWorlds + 1];
    load_vbase(a, s_vbase);
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.total; v += gridDim.x * blockDim.x) {
        const WorldDev &wd = a.worlds[find_world(s_vbase, a.nworlds, v)];
        const uint32_t local = v - wd.vbase;
        uint32_t inv = a.u.prop_inv[v];
        const uint32_t word = wd.word[local];
        if (inv != 0u) {
            a.u.prop_t[v] = 1u;
        } else if ((word >> 8) != 0u) {
            const uint8_t ut = a.u.upl_t[v];
            if ((ut & 1u) == 0u) {
                a.u.prop_t[v] = ut;
                a.u.prop_h[v] = a.u.upl_h[v];
                inv = word;
            } else {
                inv = 1u;
            }
        } else {
            inv = word;
        }
        a.u.prop_inv[v] = inv;
        a.u.jfa[0][v] = (inv >> 8) != 0u ? (int32_t)local : -1;
    }
}

__device__ __forceinline__ int jfa_top(int W, int H)
{
    const int m = W > H ? W : H;
    int s = 1;
    while (s < m) s <<= 1;
    return s >> 1;
}

__device__ __forceinline__ int jfa_dist2(int cx, int cy, int seed, int W, int H)
{
    const int sx = seed % W, sy = seed / W;
    int dx = abs(cx - sx), dy = abs(cy - sy);
    dx = min(dx, W - dx);
    dy = min(dy, H - dy);
    return dx * dx + dy * dy;
}

// JFAPass (:1512-1570) with step `step`; a world whose own sequence starts below `step` copies.
__global__ __launch_bounds__(kUpThreads) void k_jfa_pass(UpArgs a, const int32_t *in, int32_t *out, int step)
{
    __shared__ uint32_t s_vbase[kMaxBatchWorlds + 1];
    load_vbase(a, s_vbase);
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.total; v += gridDim.x * blockDim.x) {
        const WorldDev &wd = a.worlds[find_world(s_vbase, a.nworlds, v)];
        const int W = wd.W, H = wd.H;
        int best = in[v];
        if (step > jfa_top(W, H)) {
            out[v] = best;
            continue;
        }
        const uint32_t local = v - wd.vbase;
        const int x = (int)(local % (uint32_t)W), y = (int)(local / (uint32_t)W);
        const int32_t *win = in + wd.vbase;
        int bestDist = 0x7FFFFFFF;
        if (best >= 0) bestDist = jfa_dist2(x, y, best, W, H);
        for (int oy = -1; oy <= 1; ++oy)
            for (int ox = -1; ox <= 1; ++ox) {
                if (ox == 0 && oy == 0) continue;
                const int cand = win[cidx(x + ox * step, y + oy * step, W, H)];
                if (cand < 0) continue;
                const int dist = jfa_dist2(x, y, cand, W, H);
                if (dist < bestDist) {
                    bestDist = dist;
                    best = cand;
                }
            }
        out[v] = best;
    }
}

__device__ __forceinline__ float subduction_under(float x)
{
    const float v = tecto_log10f(1.0f + 8.0f * (x - 1.0f)) / 1.908485019f - 1.0f;
    return fminf(v, 0.0f);
}

__device__ __forceinline__ float continental_profile(float x)
{
    return tecto_expf(-0.02f * x * x) + tecto_expf(-0.2f * x * x) * (0.5f - fabsf(fmodf(fabsf(x), 1.0f) - 0.5f));
}

// JFAComputeDistance (:1572-1600) and applyUplift (:1662-1738) on the resolved heights, in place.
__global__ __launch_bounds__(kUpThreads) void k_up_apply(UpArgs a, const int32_t *seeds)
{
    __shared__ uint32_t s_vbase[kMaxBatchWorlds + 1];
    load_vbase(a, s_vbase);
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.total; v += gridDim.x * blockDim.x) {
        const WorldDev &wd = a.worlds[find_world(s_vbase, a.nworlds, v)];
        const int W = wd.W, H = wd.H;
        const uint32_t local = v - wd.vbase;
        const int x = (int)(local % (uint32_t)W), y = (int)(local / (uint32_t)W);
        const int seed = seeds[v];
        int dist = -1;
        if (seed >= 0) dist = (int)sqrtf((float)jfa_dist2(x, y, seed, W, H));
        a.u.dist[v] = dist;
        if (dist <= -1) continue;
        const uint32_t o = wd.vbase + (uint32_t)seed;
        const uint32_t ct = a.u.prop_t[o], inv = a.u.prop_inv[o];
        const int type = (int)(ct & 1u), pi = (int)((ct >> 1) & 3u), si = (int)((ct >> 3) & 3u);
        const int prim = 255 - (int)((inv >> (8 * pi)) & 0xFFu);
        const int secp = 255 - (int)((inv >> (8 * si)) & 0xFFu);
        const int plate = wd.id[a.cur_id][local];
        float *h = wd.h[a.cur_h] + local;
        if (type == 0 && secp == plate) {
            const float value = subduction_under((float)dist);
            const float mult = 1.0f + value * a.under_mult;
            *h = fmaxf(*h * mult, a.min_clamp);
        } else if (type == 0 && prim == plate) {
            const int ox = seed % W, oy = seed / W;
            const float sx = (float)W, sy = (float)H;
            const float ddx = fmodf((float)(x - ox) + sx * 0.5f, sx) - sx * 0.5f;
            const float ddy = fmodf((float)(y - oy) + sy * 0.5f, sy) - sy * 0.5f;
            float mag = sqrtf(ddx * ddx + ddy * ddy);
            mag = fmaxf(mag, 1e-20f);
            const float dirx = ddx / mag, diry = ddy / mag;
            // plate 255 (an empty slot named by merged type bits) has no record: zero direction
            float odx = 0.0f, ody = 0.0f;
            if (secp < kPlates) {
                odx = wd.plates_prev[secp].direction_x;
                ody = wd.plates_prev[secp].direction_y;
            }
            const float dot = fmaxf(dirx * odx + diry * ody, 0.0f);
            const float value = continental_profile(((float)dist - (float)a.over_range) - 10.0f);
            const float mult = 1.0f + (value * dot) * a.over_mult;
            *h = fmaxf(*h * mult, a.min_clamp);
        } else if (type == 1) {
            const float value = continental_profile((float)dist);
            const float change = (value * a.u.prop_h[o]) * a.cont_mult;
            *h = fminf(*h + change, a.max_clamp);
        }
    }
}

// ---- exclusive scan of the bucket counts: block scans, a scan of the block totals, the add ----

__global__ __launch_bounds__(1024) void k_scan_local(const uint32_t *cnt, uint32_t *off, uint32_t *blk, uint32_t n)
{
    __shared__ uint32_t s_w[32];
    const uint32_t base = blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
    uint32_t x[kScanItems], sum = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        x[i] = base + i < n ? cnt[base + i] : 0u;
        sum += x[i];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) s_w[warp] = inc;
    __syncthreads();
    uint32_t wb = 0;
    for (int k = 0; k < warp; ++k) wb += s_w[k];
    uint32_t run = wb + inc - sum;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) off[base + i] = run;
        run += x[i];
    }
    if (threadIdx.x == 1023) blk[blockIdx.x] = run;
}

__global__ __launch_bounds__(1024) void k_scan_blocks(uint32_t *blk, uint32_t nblk)
{
    __shared__ uint32_t s_w[32];
    const uint32_t per = (nblk + 1023) / 1024;
    const uint32_t b0 = threadIdx.x * per;
    uint32_t sum = 0;
    for (uint32_t i = 0; i < per; ++i)
        if (b0 + i < nblk) sum += blk[b0 + i];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) s_w[warp] = inc;
    __syncthreads();
    uint32_t run = inc - sum;
    for (int k = 0; k < warp; ++k) run += s_w[k];
    for (uint32_t i = 0; i < per; ++i)
        if (b0 + i < nblk) {
            const uint32_t t = blk[b0 + i];
            blk[b0 + i] = run;
            run += t;
        }
}

__global__ void k_scan_add(uint32_t *cnt, uint32_t *off, const uint32_t *blk, uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        off[i] += blk[i / kScanBlock];
        cnt[i] = 0u;  // the fill pass counts again as its cursor
    }
}

unsigned grid_for(size_t n)
{
    size_t g = (n + kUpThreads - 1) / kUpThreads;
    return (unsigned)std::max<size_t>(1, std::min<size_t>(g, 152 * 8));
}

int scan_buckets(Batch &b, cudaStream_t st)
{
    const uint32_t n = (uint32_t)b.total;
    const uint32_t nblk = (n + kScanBlock - 1) / kScanBlock;
    UpliftRefScratch &u = b.upref;
    k_scan_local<<<nblk, 1024, 0, st>>>(u.cnt, u.off, u.blk, n);
    k_scan_blocks<<<1, 1024, 0, st>>>(u.blk, nblk);
    k_scan_add<<<grid_for(n), kUpThreads, 0, st>>>(u.cnt, u.off, u.blk, n);
    b.launches += 3;
    return TECTO_OK;
}

size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

void uplift_ref_release(Batch &b)
{
    if (b.upref.arena) cudaFree(b.upref.arena);
    b.upref = UpliftRefScratch{};
}

int uplift_ref_prepare(Batch &b, cudaStream_t st)
{
    if (b.settings.step.upliftMode != TECTO_UPLIFT_REFERENCE) return TECTO_OK;
    const size_t n = b.total;
    if (n >= ((size_t)1 << 29)) {
        set_error("reference uplift: a batch holds at most 2^29 cells");
        return TECTO_ERR_UNSUPPORTED;
    }
    if (b.upref.arena && b.upref.cells >= n) return TECTO_OK;
    uplift_ref_release(b);
    const size_t ecap = std::max<size_t>(2 * n, 4096);
    const size_t nblk = (n + kScanBlock - 1) / kScanBlock;
    const size_t bytes = a256(n * 4) + a256(n) + 4 * a256(n * 4) + a256(nblk * 4 + 4) + a256(n * 4) +
                         a256(n * 4) + a256(n) + 2 * a256(n * 4) + 2 * a256(ecap * 4);
    void *arena = nullptr;
    TECTO_CUDA(cudaMalloc(&arena, bytes));
    TECTO_CUDA(cudaMemsetAsync(arena, 0, bytes, st));
    UpliftRefScratch &u = b.upref;
    u.arena = arena;
    u.cells = n;
    u.ecap = ecap;
    char *p = (char *)arena;
    auto take = [&](size_t sz) {
        char *q = p;
        p += a256(sz);
        return q;
    };
    u.upl_h = (float *)take(n * 4);
    u.upl_t = (uint8_t *)take(n);
    u.cnt = (uint32_t *)take(n * 4);
    u.off = (uint32_t *)take(n * 4);
    u.succ = (uint32_t *)take(n * 4);
    u.prop_inv = (uint32_t *)take(n * 4);
    u.blk = (uint32_t *)take(nblk * 4 + 4);
    u.prop_h = (float *)take(n * 4);
    u.dist = (int32_t *)take(n * 4);
    u.prop_t = (uint8_t *)take(n);
    u.jfa[0] = (int32_t *)take(n * 4);
    u.jfa[1] = (int32_t *)take(n * 4);
    u.ent_key = (uint32_t *)take(ecap * 4);
    u.ent_val = (uint32_t *)take(ecap * 4);
    return TECTO_OK;
}

int launch_uplift_ref(Batch &b, cudaStream_t st)
{
    if (!b.upref.arena || b.upref.cells < b.total) {
        set_error("reference uplift scratch not prepared");
        return TECTO_ERR_INVALID;
    }
    const tecto_kernel_settings &ks = b.settings.kernel;
    UpArgs a{};
    a.worlds = b.d_worlds;
    a.vbase = b.d_vbase;
    a.nworlds = (int)b.members.size();
    a.total = (uint32_t)b.total;
    a.cur_h = b.cur_h;
    a.cur_id = b.cur_id;
    a.u = b.upref;
    a.prop_thr = ks.continentalPropThreshold;
    a.prop_iters = ks.continentalPropMaxIters;
    a.under_mult = ks.subductionUnderUpliftMultiplier;
    a.over_mult = ks.subductionOverUpliftMultiplier;
    a.cont_mult = ks.continentalUpliftMultiplier;
    a.min_clamp = ks.minUpliftClamp;
    a.max_clamp = ks.maxUpliftClamp;
    a.over_range = ks.subductionOverRange;
    const unsigned g = grid_for(b.total);
    int rc;
    k_up_clear<<<g, kUpThreads, 0, st>>>(a);
    k_up_inserts<false><<<g, kUpThreads, 0, st>>>(a);
    b.launches += 2;
    if ((rc = scan_buckets(b, st)) != TECTO_OK) return rc;
    k_up_inserts<true><<<g, kUpThreads, 0, st>>>(a);
    k_up_apply_inserts<<<g, kUpThreads, 0, st>>>(a);
    k_up_contrib<false><<<g, kUpThreads, 0, st>>>(a);
    b.launches += 3;
    if ((rc = scan_buckets(b, st)) != TECTO_OK) return rc;
    k_up_contrib<true><<<g, kUpThreads, 0, st>>>(a);
    k_up_sum<<<g, kUpThreads, 0, st>>>(a);
    k_up_combine<<<g, kUpThreads, 0, st>>>(a);
    b.launches += 3;
    int top = 0;
    for (const tecto_world *w : b.members) {
        const int m = std::max(w->W, w->H);
        int s = 1;
        while (s < m) s <<= 1;
        top = std::max(top, s >> 1);
    }
    int cur = 0;
    for (int step = top; step > 0; step >>= 1) {
        k_jfa_pass<<<g, kUpThreads, 0, st>>>(a, b.upref.jfa[cur], b.upref.jfa[cur ^ 1], step);
        cur ^= 1;
        b.launches += 1;
    }
    b.upref_final = cur;
    k_up_apply<<<g, kUpThreads, 0, st>>>(a, b.upref.jfa[cur]);
    b.launches += 1;
    TECTO_CUDA(cudaGetLastError());
    return TECTO_OK;
}

}  // namespace tecto
