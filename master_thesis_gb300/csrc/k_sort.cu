// k_sort.cu - stable LSD radix sort of (destination cell, source cell) pairs.
//
// Replaces registerPlateCollisions' atomic slotting (src/cuda_compute/plate_tectonics_kernel.cu:
// 273-298): arrivals are grouped by sorting on the destination key; the sort is stable, so
// within one destination the sources stay in ascending order, which is the engine's canonical
// arrival-slot order.
//
// Onesweep structure: one kernel builds the digit histograms of every pass in a single read;
// then each pass is one kernel that ranks a tile of 4096 keys with warp ballots, publishes the
// tile's digit counts, walks back over earlier tiles (decoupled look-back, bounded spin) and
// scatters through shared memory so that runs of equal digits leave as contiguous stores.
// The keys can be generated from plate ids (advection fused into the sort: the key of cell i is
// getPixelMovements' wrapped destination, plate_tectonics_kernel.cu:248-265): the histogram
// kernel generates them once, counts them and stores them for the first pass, whose values are
// then the cell indices themselves.
//
// The digit width RB is a template parameter (8..11 bits): wider digits mean fewer passes over
// the keys but larger per-tile histograms and look-back tables; the autotuner picks per size.
#include "tecto_internal.cuh"

namespace tecto {

namespace {

constexpr int kWarps = kSortThreads / 32;
constexpr int kLookAhead = 8;  // predecessor tiles read per look-back round
// From this many tiles (16 M keys) a pass runs three blocks per SM: measured faster at 67 M keys
// (8192^2) and slower at 4 M (2048^2)
constexpr size_t kSortWideTiles = 4096;

template <int RB>
struct Digits {
    static constexpr int R = 1 << RB;               // digit values per pass
    static constexpr int DPT = R / kSortThreads;     // digits owned by each thread of a pass
    static constexpr uint32_t MASK = (uint32_t)R - 1u;
    static constexpr int MAX_PASSES = (32 + RB - 1) / RB;
    static_assert(RB >= 8 && RB <= kMaxRadixBits, "digit width out of range");
};

// Dynamic shared memory of one pass: per-warp digit counts, per-digit tile start and global
// base, the staged keys and values.
template <int RB>
constexpr size_t pass_smem()
{
    return ((size_t)kWarps * Digits<RB>::R + 2 * (size_t)Digits<RB>::R + 2 * (size_t)kSortTile) *
           sizeof(uint32_t);
}

// Batch-virtual destination of virtual cell i: the owning world's getPixelMovements destination
// (plate_tectonics_kernel.cu:248-265) offset by the world's virtual base.
struct GenArgs {
    const WorldDev *worlds;
    const uint32_t *vbase;
    int nworlds;
    int cur_id;
};

__device__ __forceinline__ uint32_t gen_key(size_t i, const GenArgs &g, const uint32_t *s_vbase)
{
    const uint32_t v = (uint32_t)i;  // n < 2^30
    const WorldDev &wd = g.worlds[find_world(s_vbase, g.nworlds, v)];
    const uint32_t local = v - wd.vbase;
    const int W = wd.W;
    const int y = (int)(local / (uint32_t)W);
    const int x = (int)(local - (uint32_t)y * (uint32_t)W);
    const int2 o = wd.off[wd.id[g.cur_id][local]];
    return wd.vbase + cidx(x + o.x, y + o.y, W, wd.H);
}

__device__ __forceinline__ void load_vbase(const GenArgs &g, uint32_t *s_vbase)
{
    for (int i = threadIdx.x; i < g.nworlds; i += blockDim.x) s_vbase[i] = g.vbase[i];
}

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p)
{
    return *(const volatile uint32_t *)p;
}

__device__ __forceinline__ void st_volatile(uint32_t *p, uint32_t v)
{
    *(volatile uint32_t *)p = v;
}

// Digit histograms of all passes in one read of the keys; generated keys are stored to keys_gen.
template <bool GEN, int RB>
__global__ __launch_bounds__(256) void k_sort_hist(GenArgs g, const uint32_t *keys_in, size_t n,
                                                   int passes, uint32_t *hist, uint32_t *keys_gen)
{
    using D = Digits<RB>;
    __shared__ uint32_t s_hist[D::MAX_PASSES][D::R];
    __shared__ uint32_t s_vbase[GEN ? kMaxBatchWorlds : 1];
    for (int i = threadIdx.x; i < D::MAX_PASSES * D::R; i += blockDim.x) (&s_hist[0][0])[i] = 0;
    if (GEN) load_vbase(g, s_vbase);
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    // every lane runs the same number of rounds so that the warp-wide match stays converged
    const size_t rounds = (n + stride - 1) / stride;
    for (size_t r = 0; r < rounds; ++r) {
        const size_t i = r * stride + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
        const bool valid = i < n;
        uint32_t key = 0;
        if (valid) {
            if (GEN) {
                key = gen_key(i, g, s_vbase);
                keys_gen[i] = key;
            } else {
                key = keys_in[i];
            }
        }
        for (int p = 0; p < passes; ++p) {
            const uint32_t d = valid ? ((key >> (RB * p)) & D::MASK) : (uint32_t)D::R;
            const unsigned peers = __match_any_sync(0xffffffffu, d);
            if (valid && (peers & ((1u << lane) - 1u)) == 0)
                atomicAdd(&s_hist[p][d], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * D::R; i += blockDim.x) {
        const uint32_t v = (&s_hist[0][0])[i];
        if (v) atomicAdd(&hist[i], v);
    }
}

// Block-wide exclusive scan of one value per thread (256 threads); returns the exclusive prefix
// and the block total.  s_w holds kWarps words; the call ends with a barrier.
__device__ __forceinline__ uint32_t block_scan(uint32_t v, uint32_t *s_w, uint32_t *total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) s_w[warp] = inc;
    __syncthreads();
    uint32_t wb = 0, all = 0;
#pragma unroll
    for (int k = 0; k < kWarps; ++k) {
        const uint32_t x = s_w[k];
        wb += k < warp ? x : 0u;
        all += x;
    }
    __syncthreads();
    *total = all;
    return wb + inc - v;
}

// Exclusive scan of each pass's digit counts, in place.  One block of 256 threads; thread t owns
// digits t, t + 256, ... and the chunks of 256 digits are scanned in order.
template <int RB>
__global__ void k_sort_scan(uint32_t *hist, int passes)
{
    using D = Digits<RB>;
    __shared__ uint32_t s_w[kWarps];
    const int t = threadIdx.x;
    for (int p = 0; p < passes; ++p) {
        uint32_t carry = 0;
        for (int c = 0; c < D::DPT; ++c) {
            uint32_t *h = hist + (size_t)p * D::R + c * kSortThreads + t;
            const uint32_t v = *h;
            uint32_t tot = 0;
            const uint32_t ex = block_scan(v, s_w, &tot);
            *h = carry + ex;
            carry += tot;
        }
    }
}

// One onesweep pass.  vals_in == nullptr: the value of position i is i.  Two kernels share the
// body: k_sort_pass (the compiler takes 128 registers: two blocks per SM) for small sorts, and
// k_sort_pass_wide (three blocks per SM: 80 registers, a few more bytes of spill) once there are
// enough tiles to fill the extra residency.
template <int RB>
__device__ __forceinline__ void sort_pass_body(
    const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_out, uint32_t *vals_out, size_t n,
    int shift, const uint32_t *digit_start, uint32_t *status, uint32_t *tile_counter, uint32_t *error)
{
    using D = Digits<RB>;
    constexpr int R = D::R, DPT = D::DPT;
    extern __shared__ __align__(16) uint32_t sm_sort[];
    uint32_t *s_cnt = sm_sort;                   // [kWarps][R] per-warp counts, then warp offsets
    uint32_t *s_start = s_cnt + kWarps * R;      // tile-local exclusive start per digit
    uint32_t *s_base = s_start + R;              // global output position of the digit's run
    uint32_t *s_keys = s_base + R;
    uint32_t *s_vals = s_keys + kSortTile;
    __shared__ uint32_t s_w[kWarps];
    __shared__ uint32_t s_tile;

    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (t == 0) s_tile = atomicAdd(tile_counter, 1u);
    for (int i = t; i < kWarps * R; i += kSortThreads) s_cnt[i] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const size_t base = (size_t)tile * kSortTile;

    uint32_t k[kSortItems], v[kSortItems], rank[kSortItems];
    const size_t wbase = base + (size_t)warp * (32 * kSortItems);
#pragma unroll
    for (int it = 0; it < kSortItems; ++it) {
        const size_t idx = wbase + (size_t)it * 32 + lane;
        if (idx < n) {
            k[it] = keys_in[idx];
            v[it] = vals_in ? vals_in[idx] : (uint32_t)idx;
        } else {
            k[it] = 0;
            v[it] = 0;
        }
    }

    // Warp-level ranking: items are visited in element order (item, lane), so the rank of an
    // item among equal digits of its warp preserves input order (stability).
    const unsigned lt = (1u << lane) - 1u;
    uint32_t *my_cnt = s_cnt + warp * R;
#pragma unroll
    for (int it = 0; it < kSortItems; ++it) {
        const bool valid = wbase + (size_t)it * 32 + lane < n;
        const uint32_t d = (k[it] >> shift) & D::MASK;
        unsigned peers = __ballot_sync(0xffffffffu, valid);
#pragma unroll
        for (int b = 0; b < RB; ++b) {
            const bool bit = (d >> b) & 1u;
            const unsigned bb = __ballot_sync(0xffffffffu, bit);
            peers &= bit ? bb : ~bb;
        }
        uint32_t before = 0;
        if (valid) before = my_cnt[d];
        __syncwarp();
        if (valid && (peers & lt) == 0) my_cnt[d] = before + (uint32_t)__popc(peers);
        __syncwarp();
        rank[it] = before + (uint32_t)__popc(peers & lt);
    }
    __syncthreads();

    // Per owned digit d = t + 256 c: warp offsets and the tile's count of that digit, published
    // at once so that later tiles can start their look-back.
    uint32_t run[DPT];
    uint32_t *my_status = status + (size_t)tile * R;
#pragma unroll
    for (int c = 0; c < DPT; ++c) {
        const int d = t + c * kSortThreads;
        uint32_t r = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const uint32_t x = s_cnt[w * R + d];
            s_cnt[w * R + d] = r;
            r += x;
        }
        run[c] = r;
        st_volatile(my_status + d, (tile == 0 ? kFlagPrefix : kFlagAggregate) | r);
    }
    // Tile-local exclusive start of every digit (chunks of 256 digits in order).
    uint32_t carry = 0;
#pragma unroll
    for (int c = 0; c < DPT; ++c) {
        uint32_t tot = 0;
        const uint32_t ex = block_scan(run[c], s_w, &tot);
        s_start[t + c * kSortThreads] = carry + ex;
        carry += tot;
    }

    // Decoupled look-back for the owned digits, walked side by side.  Each round reads the status
    // words of up to kLookAhead predecessors at once (independent loads in flight together) and
    // consumes them newest first until one is not yet published or carries an inclusive prefix.
    uint32_t prefix[DPT];
#pragma unroll
    for (int c = 0; c < DPT; ++c) prefix[c] = 0;
    if (tile > 0) {
        int j[DPT];
#pragma unroll
        for (int c = 0; c < DPT; ++c) j[c] = (int)tile - 1;
        uint32_t spins = 0;
        bool pending = true;
        while (pending) {
            pending = false;
            bool progressed = false;
#pragma unroll
            for (int c = 0; c < DPT; ++c) {
                if (j[c] < 0) continue;
                const uint32_t *col = status + t + c * kSortThreads;
                const int j0 = j[c];
                uint32_t sv[kLookAhead];
#pragma unroll
                for (int q = 0; q < kLookAhead; ++q) sv[q] = j0 - q >= 0 ? ld_volatile(col + (size_t)(j0 - q) * R) : 0u;
                int used = 0;
                bool done = false;
#pragma unroll
                for (int q = 0; q < kLookAhead; ++q) {
                    if (done || used < q || j0 - q < 0) continue;
                    const uint32_t st = sv[q];
                    if ((st & ~kValueMask) == 0) continue;  // not yet published: read it again next round
                    progressed = true;
                    prefix[c] += st & kValueMask;
                    used = q + 1;
                    done = (st & kFlagPrefix) != 0;
                }
                j[c] = done ? -1 : j0 - used;
                if (j[c] >= 0) pending = true;
            }
            if (pending && !progressed && ++spins > kSpinLimit) {  // a predecessor never published
                atomicOr(error, kErrLookbackTimeout);
                break;
            }
        }
#pragma unroll
        for (int c = 0; c < DPT; ++c)
            st_volatile(my_status + t + c * kSortThreads, kFlagPrefix | ((prefix[c] + run[c]) & kValueMask));
    }
#pragma unroll
    for (int c = 0; c < DPT; ++c) {
        const int d = t + c * kSortThreads;
        s_base[d] = digit_start[d] + prefix[c];
    }
    __syncthreads();

    // Scatter into shared memory in digit order.
#pragma unroll
    for (int it = 0; it < kSortItems; ++it) {
        if (wbase + (size_t)it * 32 + lane < n) {
            const uint32_t d = (k[it] >> shift) & D::MASK;
            const uint32_t pos = s_start[d] + my_cnt[d] + rank[it];
            s_keys[pos] = k[it];
            s_vals[pos] = v[it];
        }
    }
    __syncthreads();
    const size_t rem = n - base;
    const uint32_t tile_n = rem < (size_t)kSortTile ? (uint32_t)rem : (uint32_t)kSortTile;
    for (uint32_t jj = t; jj < tile_n; jj += kSortThreads) {
        const uint32_t key = s_keys[jj];
        const uint32_t d = (key >> shift) & D::MASK;
        const uint32_t out = s_base[d] + (jj - s_start[d]);
        keys_out[out] = key;
        vals_out[out] = s_vals[jj];
    }
}

template <int RB>
__global__ __launch_bounds__(kSortThreads) void k_sort_pass(
    const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_out, uint32_t *vals_out, size_t n,
    int shift, const uint32_t *digit_start, uint32_t *status, uint32_t *tile_counter, uint32_t *error)
{
    sort_pass_body<RB>(keys_in, vals_in, keys_out, vals_out, n, shift, digit_start, status, tile_counter, error);
}

template <int RB>
__global__ __launch_bounds__(kSortThreads, 3) void k_sort_pass_wide(
    const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_out, uint32_t *vals_out, size_t n,
    int shift, const uint32_t *digit_start, uint32_t *status, uint32_t *tile_counter, uint32_t *error)
{
    sort_pass_body<RB>(keys_in, vals_in, keys_out, vals_out, n, shift, digit_start, status, tile_counter, error);
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

template <int RB>
int set_sort_attributes()
{
    TECTO_CUDA(cudaFuncSetAttribute(k_sort_pass<RB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)pass_smem<RB>()));
    TECTO_CUDA(cudaFuncSetAttribute(k_sort_pass_wide<RB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)pass_smem<RB>()));
    return TECTO_OK;
}

bool g_sort_attr_done = false;

template <int RB>
int run_sort_rb(const SortArgs &a, const SortScratch &scr, cudaStream_t st, int *result_half)
{
    const int passes = scr.passes;
    const size_t tiles = (a.n + kSortTile - 1) / kSortTile;
    constexpr int R = Digits<RB>::R;
    // one memset covers hist, status and counters (contiguous in the scratch layout)
    const size_t clear = align256((size_t)passes * R * 4) + align256((size_t)passes * tiles * R * 4) +
                         align256(kMaxSortPasses * 4);
    TECTO_CUDA(cudaMemsetAsync(scr.hist, 0, clear, st));
    const bool gen = a.worlds != nullptr;
    const GenArgs g{a.worlds, a.vbase, a.nworlds, a.cur_id};
    int hist_blocks = (int)((a.n + 255) / 256);
    if (hist_blocks > 152 * 8) hist_blocks = 152 * 8;
    // generated keys go to the second key half, which the first pass reads and does not write
    const uint32_t *kin = a.keys_in, *vin = a.vals_in;
    if (gen) {
        k_sort_hist<true, RB><<<hist_blocks, 256, 0, st>>>(g, nullptr, a.n, passes, scr.hist, a.keys[1]);
        kin = a.keys[1];
        vin = nullptr;
    } else {
        k_sort_hist<false, RB><<<hist_blocks, 256, 0, st>>>(g, a.keys_in, a.n, passes, scr.hist, nullptr);
    }
    k_sort_scan<RB><<<1, kSortThreads, 0, st>>>(scr.hist, passes);
    int half = 0;
    for (int p = 0; p < passes; ++p) {
        uint32_t *kout = a.keys[half], *vout = a.vals[half];
        uint32_t *status = scr.status + (size_t)p * tiles * R;
        auto pass = tiles >= kSortWideTiles ? k_sort_pass_wide<RB> : k_sort_pass<RB>;
        pass<<<(unsigned)tiles, kSortThreads, pass_smem<RB>(), st>>>(
            kin, vin, kout, vout, a.n, RB * p, scr.hist + (size_t)p * R, status, scr.counters + p, scr.error);
        kin = kout;
        vin = vout;
        half ^= 1;
    }
    TECTO_CUDA(cudaGetLastError());
    *result_half = half ^ 1;
    return TECTO_OK;
}

}  // namespace

int sort_kernel_attributes()
{
    if (g_sort_attr_done) return TECTO_OK;
    int rc;
    if ((rc = set_sort_attributes<8>()) != TECTO_OK || (rc = set_sort_attributes<9>()) != TECTO_OK ||
        (rc = set_sort_attributes<10>()) != TECTO_OK || (rc = set_sort_attributes<11>()) != TECTO_OK)
        return rc;
    g_sort_attr_done = true;
    return TECTO_OK;
}

int key_bits_for(size_t n)
{
    int b = 1;
    while (b < 32 && ((size_t)1 << b) < n) ++b;
    return b;
}

bool valid_radix_bits(int rb) { return rb >= 8 && rb <= kMaxRadixBits; }

int sort_passes_for(int key_bits, int rb) { return (key_bits + rb - 1) / rb; }

size_t sort_scratch_bytes(size_t n, int key_bits, int rb)
{
    const size_t passes = (size_t)sort_passes_for(key_bits, rb);
    const size_t tiles = (n + kSortTile - 1) / kSortTile;
    const size_t R = (size_t)1 << rb;
    return align256(passes * R * 4) + align256(passes * tiles * R * 4) + align256(kMaxSortPasses * 4) +
           align256(4);
}

void sort_scratch_carve(void *base, size_t n, int key_bits, int rb, SortScratch *out)
{
    const int passes = sort_passes_for(key_bits, rb);
    const size_t tiles = (n + kSortTile - 1) / kSortTile;
    const size_t R = (size_t)1 << rb;
    char *p = (char *)base;
    out->passes = passes;
    out->tiles = (int)tiles;
    out->radix_bits = rb;
    out->hist = (uint32_t *)p;
    p += align256((size_t)passes * R * 4);
    out->status = (uint32_t *)p;
    p += align256((size_t)passes * tiles * R * 4);
    out->counters = (uint32_t *)p;
    p += align256(kMaxSortPasses * 4);
    out->error = (uint32_t *)p;
}

int run_sort(const SortArgs &a, const SortScratch &scr, cudaStream_t st, int *result_half)
{
    const int rb = scr.radix_bits;
    if (!valid_radix_bits(rb) || sort_passes_for(a.key_bits, rb) != scr.passes || a.n == 0 ||
        a.n > (size_t)kValueMask || (a.n + kSortTile - 1) / kSortTile > (size_t)scr.tiles) {
        set_error("run_sort: scratch does not match the problem size");
        return TECTO_ERR_INVALID;
    }
    if (a.worlds != nullptr && (a.nworlds < 1 || a.nworlds > kMaxBatchWorlds)) {
        set_error("run_sort: batch world count out of range");
        return TECTO_ERR_INVALID;
    }
    if (rb > 8 && !g_sort_attr_done) {  // wide digits need the opt-in shared memory size
        set_error("run_sort: sort kernel attributes not set");
        return TECTO_ERR_INVALID;
    }
    switch (rb) {
        case 8: return run_sort_rb<8>(a, scr, st, result_half);
        case 9: return run_sort_rb<9>(a, scr, st, result_half);
        case 10: return run_sort_rb<10>(a, scr, st, result_half);
        default: return run_sort_rb<11>(a, scr, st, result_half);
    }
}

}  // namespace tecto

// ---- C ABI: standalone sort -------------------------------------------------------------------

extern "C" size_t tecto_sort_scratch_bytes_radix(size_t n, int key_bits, int radix_bits)
{
    if (key_bits < 1 || key_bits > 32) return 0;
    if (radix_bits == 0) radix_bits = 8;
    if (!tecto::valid_radix_bits(radix_bits)) return 0;
    // two ping-pong halves for keys and values are carved after the sort's own scratch
    return tecto::sort_scratch_bytes(n, key_bits, radix_bits) + 4 * tecto::align256(n * sizeof(uint32_t));
}

extern "C" size_t tecto_sort_scratch_bytes(size_t n, int key_bits)
{
    return tecto_sort_scratch_bytes_radix(n, key_bits, 8);
}

extern "C" int tecto_sort_wide_pass(size_t n)
{
    return (n + tecto::kSortTile - 1) / tecto::kSortTile >= (size_t)tecto::kSortWideTiles ? 1 : 0;
}

extern "C" int tecto_sort_pairs_radix(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_out,
                                      uint32_t *vals_out, size_t n, int key_bits, int radix_bits, void *scratch,
                                      size_t scratch_bytes, tecto_stream_t stream)
{
    using namespace tecto;
    if (n == 0) return TECTO_OK;
    if (radix_bits == 0) radix_bits = 8;
    if (!keys_in || !vals_in || !keys_out || !vals_out || !scratch || key_bits < 1 ||
        key_bits > 32 || n > (size_t)kValueMask || !valid_radix_bits(radix_bits)) {
        set_error("tecto_sort_pairs: invalid argument");
        return TECTO_ERR_INVALID;
    }
    if (scratch_bytes < tecto_sort_scratch_bytes_radix(n, key_bits, radix_bits)) {
        set_error("tecto_sort_pairs: scratch too small");
        return TECTO_ERR_INVALID;
    }
    int rc;
    if (radix_bits > 8 && (rc = sort_kernel_attributes()) != TECTO_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    SortScratch scr{};
    sort_scratch_carve(scratch, n, key_bits, radix_bits, &scr);
    char *p = (char *)scratch + sort_scratch_bytes(n, key_bits, radix_bits);
    const size_t arr = align256(n * sizeof(uint32_t));
    SortArgs a{};
    a.keys_in = keys_in;
    a.vals_in = vals_in;
    a.keys[0] = (uint32_t *)p;
    a.vals[0] = (uint32_t *)(p + arr);
    a.keys[1] = (uint32_t *)(p + 2 * arr);
    a.vals[1] = (uint32_t *)(p + 3 * arr);
    a.n = n;
    a.key_bits = key_bits;
    TECTO_CUDA(cudaMemsetAsync(scr.error, 0, 4, st));
    int half = 0;
    rc = run_sort(a, scr, st, &half);
    if (rc != TECTO_OK) return rc;
    TECTO_CUDA(cudaMemcpyAsync(keys_out, a.keys[half], n * 4, cudaMemcpyDeviceToDevice, st));
    TECTO_CUDA(cudaMemcpyAsync(vals_out, a.vals[half], n * 4, cudaMemcpyDeviceToDevice, st));
    uint32_t err = 0;
    TECTO_CUDA(cudaMemcpyAsync(&err, scr.error, 4, cudaMemcpyDeviceToHost, st));
    TECTO_CUDA(cudaStreamSynchronize(st));
    if (err) {
        set_error("tecto_sort_pairs: look-back wait gave up");
        return TECTO_ERR_DEVICE_TIMEOUT;
    }
    return TECTO_OK;
}

extern "C" int tecto_sort_pairs(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_out,
                                uint32_t *vals_out, size_t n, int key_bits, void *scratch,
                                size_t scratch_bytes, tecto_stream_t stream)
{
    return tecto_sort_pairs_radix(keys_in, vals_in, keys_out, vals_out, n, key_bits, 8, scratch, scratch_bytes,
                                  stream);
}
