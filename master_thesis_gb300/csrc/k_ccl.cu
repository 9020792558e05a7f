// k_ccl.cu - connected-component labelling of equal plate ids on the torus.
//
// Replaces the reference's union-find CCL (src/cuda_compute/ccl.cu:35-177, driver
// plate_tectonic_sim.cu:375-389).  Labels converge to the minimum linear index of each
// component, as the reference's roots do.  Three edge sets:
//   TECTO_CCL_4    left, top;
//   TECTO_CCL_8    left, top, top-left, top-right;
//   TECTO_CCL_REF8 the reference kernels' union set: every cell links left and top-left when
//                  equal, plus init's single link to the first equal of (tl, t, tr, l)
//                  (ccl.cu:107-116), plus top and top-right on row 0 (ccl.cu:161-170).
// (Edges are undirected; each is generated once, from the lower-right cell.)
//
// Three kernels: union-find inside a 32x32 tile in shared memory (roots = smallest index),
// unions across tile borders with global atomicMin linking, and a flatten pass.
#include "tecto_internal.cuh"

namespace tecto {

namespace {

constexpr int CX = kCclTileX, CY = kCclTileY;

// Edge mask of a cell on row y from its id c and its neighbours' ids: bit 0 l, bit 1 t, bit 2 tl,
// bit 3 tr.
__device__ __forceinline__ unsigned mask_of(unsigned c, unsigned l, unsigned t, unsigned tl, unsigned tr, int y,
                                            int mode)
{
    const bool el = l == c, et = t == c, etl = tl == c, etr = tr == c;
    if (mode == TECTO_CCL_4) return (el ? 1u : 0u) | (et ? 2u : 0u);
    if (mode == TECTO_CCL_8) return (el ? 1u : 0u) | (et ? 2u : 0u) | (etl ? 4u : 0u) | (etr ? 8u : 0u);
    unsigned m = (el ? 1u : 0u) | (etl ? 4u : 0u);
    if (y == 0) {
        m |= (et ? 2u : 0u) | (etr ? 8u : 0u);
    } else if (!etl) {
        if (et) m |= 2u;
        else if (etr) m |= 8u;
    }
    return m;
}

__device__ __forceinline__ unsigned edge_mask(const uint8_t *id, int x, int y, int W, int H, int mode)
{
    return mask_of(id[(size_t)y * W + x], id[cidx(x - 1, y, W, H)], id[cidx(x, y - 1, W, H)],
                   id[cidx(x - 1, y - 1, W, H)], id[cidx(x + 1, y - 1, W, H)], y, mode);
}

__device__ __forceinline__ int smem_find(const int *par, int a)
{
    while (par[a] != a) a = par[a];
    return a;
}

__device__ __forceinline__ void smem_union(int *par, int a, int b)
{
    while (true) {
        a = smem_find(par, a);
        b = smem_find(par, b);
        if (a == b) return;
        if (a > b) {
            const int tmp = a;
            a = b;
            b = tmp;
        }
        const int old = atomicMin(par + b, a);
        if (old == b) return;
        b = old;
    }
}

__device__ __forceinline__ uint32_t g_find(const uint32_t *L, uint32_t a)
{
    uint32_t p = L[a];
    while (p != a) {
        a = p;
        p = L[a];
    }
    return a;
}

__device__ __forceinline__ void g_union(uint32_t *L, uint32_t a, uint32_t b)
{
    while (true) {
        a = g_find(L, a);
        b = g_find(L, b);
        if (a == b) return;
        if (a > b) {
            const uint32_t tmp = a;
            a = b;
            b = tmp;
        }
        const uint32_t old = atomicMin(L + b, a);
        if (old == b) return;
        b = old;
    }
}

// The world of this block's tile, or nullptr when the world's labelling is not due this step.
__device__ __forceinline__ const WorldDev *ccl_tile(const WorldDev *worlds, const uint2 *tiles, int period,
                                                    int *x0, int *y0)
{
    int wi, tx, ty;
    tile_of(tiles[blockIdx.x], &wi, &tx, &ty);
    const WorldDev *wd = worlds + wi;
    if (period > 0 && wd->ctl->iteration % (uint32_t)period != 0u) return nullptr;
    *x0 = tx * CX;
    *y0 = ty * CY;
    return wd;
}

// One warp per tile row (CX is the warp width).  A row's left edges make runs: every cell's
// parent starts as the first cell of its run, found with one ballot, without atomics.  Up edges
// then join runs; an up edge is skipped when an edge already kept joins the same two runs:
//   t(x)  when x is joined to x - 1 and x - 1 has t or tr (same target, or the target's left
//         neighbour, joined to it by the left edge all modes include);
//   tl(x) when x is joined to x - 1 and x - 1 has t or tl;
//   tr(x) when x has t, or x is joined to x - 1 and x - 1 has tr.
// A skip depends only on edges strictly earlier in (column, t before tr) order, so every skipped
// edge's runs are already joined by kept ones: the components, and their minimum-index roots, are
// those of the full edge set.  Edges whose neighbour lies in the tile only through the torus wrap
// (a tile spanning the whole world) take the plain union.
// eight blocks per SM (32 registers, no spill): the pass waits on loads and shared atomics
__global__ __launch_bounds__(256, 8) void k_ccl_local(const WorldDev *worlds, const uint2 *tiles, int cur_id,
                                                   int mode, int period)
{
    static_assert(CX == 32 && CY % 8 == 0, "one warp per tile row, eight warps");
    __shared__ int par[CX * CY];
    int x0, y0;
    const WorldDev *wd = ccl_tile(worlds, tiles, period, &x0, &y0);
    if (!wd) return;
    const uint8_t *id = wd->id[cur_id];
    uint32_t *labels = wd->labels;
    const int W = wd->W, H = wd->H;
    const int tw = min(CX, W - x0), th = min(CY, H - y0);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int kRowsPerWarp = CY / 8;
    const int dxs[4] = {-1, 0, -1, 1}, dys[4] = {0, -1, -1, -1};
    unsigned keep[kRowsPerWarp], wrapped[kRowsPerWarp];
#pragma unroll
    for (int r = 0; r < kRowsPerWarp; ++r) {
        const int ly = warp + 8 * r;
        const int x = x0 + lane, y = y0 + ly;
        const bool valid = lane < tw && ly < th;
        // the row and the row above, one byte per lane; the left and right neighbours come from
        // the adjacent lanes, the row ends load theirs (wrapped)
        const int yu = y == 0 ? H - 1 : y - 1;
        const unsigned c = valid ? id[(size_t)y * W + x] : 0u;
        const unsigned t = valid ? id[(size_t)yu * W + x] : 0u;
        unsigned l = __shfl_up_sync(0xffffffffu, c, 1), tl = __shfl_up_sync(0xffffffffu, t, 1);
        unsigned tr = __shfl_down_sync(0xffffffffu, t, 1);
        if (valid && lane == 0) {
            const int xl = x == 0 ? W - 1 : x - 1;
            l = id[(size_t)y * W + xl];
            tl = id[(size_t)yu * W + xl];
        }
        if (valid && lane == tw - 1) tr = id[(size_t)yu * W + (x + 1 == W ? 0 : x + 1)];
        unsigned m = valid ? mask_of(c, l, t, tl, tr, y, mode) : 0u;
        // natural: the neighbour is the adjacent cell of the tile, no wrap; wrapped: inside the
        // tile only through the wrap; edges leaving the tile belong to k_ccl_border
        unsigned nat = 0, wrp = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (!(m & (1u << k))) continue;
            const int ax = lane + dxs[k], ay = ly + dys[k];
            if (ax >= 0 && ax < tw && ay >= 0) {
                nat |= 1u << k;
            } else {
                const int nlx = wrap_fast(x + dxs[k], W) - x0, nly = wrap_fast(y + dys[k], H) - y0;
                if (nlx >= 0 && nlx < tw && nly >= 0 && nly < th) wrp |= 1u << k;
            }
        }
        // runs of the row: a cell without a natural left edge starts one
        const unsigned starts = __ballot_sync(0xffffffffu, !(nat & 1u));
        par[ly * CX + lane] = ly * CX + (31 - __clz(starts & (0xffffffffu >> (31 - lane))));
        const unsigned prev = __shfl_up_sync(0xffffffffu, nat, 1);
        unsigned up = nat & 14u;
        if (nat & 1u) {  // joined to x - 1 (lane > 0)
            if (prev & (2u | 8u)) up &= ~2u;
            if (prev & (2u | 4u)) up &= ~4u;
            if (prev & 8u) up &= ~8u;
        }
        if (nat & 2u) up &= ~8u;
        keep[r] = up;
        wrapped[r] = wrp;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRowsPerWarp; ++r) {
        const int ly = warp + 8 * r;
        const int e = ly * CX + lane;
        const unsigned up = keep[r], wrp = wrapped[r];
        if (up & 2u) smem_union(par, e, e - CX);
        if (up & 4u) smem_union(par, e, e - CX - 1);
        if (up & 8u) smem_union(par, e, e - CX + 1);
        if (wrp) {
            const int x = x0 + lane, y = y0 + ly;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (!(wrp & (1u << k))) continue;
                const int nlx = wrap_fast(x + dxs[k], W) - x0, nly = wrap_fast(y + dys[k], H) - y0;
                smem_union(par, e, nly * CX + nlx);
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRowsPerWarp; ++r) {
        const int ly = warp + 8 * r;
        if (lane >= tw || ly >= th) continue;
        const int root = smem_find(par, ly * CX + lane);
        const int ry = root / CX, rx = root - ry * CX;
        labels[(size_t)(y0 + ly) * W + x0 + lane] = (uint32_t)((y0 + ry) * W + x0 + rx);
    }
}

// Unions across tile borders: only cells on a tile's top row or left/right column have edges
// leaving the tile.
__global__ __launch_bounds__(128) void k_ccl_border(const WorldDev *worlds, const uint2 *tiles, int cur_id,
                                                    int mode, int period)
{
    int x0, y0;
    const WorldDev *wd = ccl_tile(worlds, tiles, period, &x0, &y0);
    if (!wd) return;
    const uint8_t *id = wd->id[cur_id];
    uint32_t *labels = wd->labels;
    const int W = wd->W, H = wd->H;
    const int tw = min(CX, W - x0), th = min(CY, H - y0);
    const int nb = tw + 2 * th;  // top row, left column, right column (corners repeat harmlessly)
    const int dxs[4] = {-1, 0, -1, 1}, dys[4] = {0, -1, -1, -1};
    for (int e = threadIdx.x; e < nb; e += blockDim.x) {
        int lx, ly;
        if (e < tw) { lx = e; ly = 0; }
        else if (e < tw + th) { lx = 0; ly = e - tw; }
        else { lx = tw - 1; ly = e - tw - th; }
        const int x = x0 + lx, y = y0 + ly;
        const unsigned m = edge_mask(id, x, y, W, H, mode);
        for (int k = 0; k < 4; ++k) {
            if (!(m & (1u << k))) continue;
            const int nx = wrap_fast(x + dxs[k], W), ny = wrap_fast(y + dys[k], H);
            const int nlx = nx - x0, nly = ny - y0;
            if (nlx >= 0 && nlx < tw && nly >= 0 && nly < th) continue;  // handled locally
            g_union(labels, (uint32_t)((size_t)y * W + x), (uint32_t)((size_t)ny * W + nx));
        }
    }
}

__global__ void k_ccl_flatten(const WorldDev *worlds, const uint2 *tiles, int period)
{
    int x0, y0;
    const WorldDev *wd = ccl_tile(worlds, tiles, period, &x0, &y0);
    if (!wd) return;
    uint32_t *labels = wd->labels;
    const int W = wd->W, H = wd->H;
    for (int e = threadIdx.x; e < CX * CY; e += blockDim.x) {
        const int ly = e / CX, lx = e - ly * CX;
        const int x = x0 + lx, y = y0 + ly;
        if (x < W && y < H) {
            const uint32_t i = (uint32_t)y * (uint32_t)W + (uint32_t)x;
            labels[i] = g_find(labels, i);
        }
    }
}

}  // namespace

int launch_ccl(Batch &b, int connectivity, bool due_only, cudaStream_t st)
{
    if (connectivity != TECTO_CCL_4 && connectivity != TECTO_CCL_8 && connectivity != TECTO_CCL_REF8) {
        set_error("cclConnectivity must be 4, 8 or 9 (ref8)");
        return TECTO_ERR_INVALID;
    }
    const int period = due_only ? (b.settings.sim.iterationsForCCL > 0 ? b.settings.sim.iterationsForCCL : 1) : 0;
    const unsigned grid = (unsigned)b.ntiles[TK_CCL];
    const uint2 *tiles = b.d_tiles[TK_CCL];
    k_ccl_local<<<grid, 256, 0, st>>>(b.d_worlds, tiles, b.cur_id, connectivity, period);
    k_ccl_border<<<grid, 128, 0, st>>>(b.d_worlds, tiles, b.cur_id, connectivity, period);
    k_ccl_flatten<<<grid, 256, 0, st>>>(b.d_worlds, tiles, period);
    TECTO_CUDA(cudaGetLastError());
    b.launches += 3;
    return TECTO_OK;
}

}  // namespace tecto
