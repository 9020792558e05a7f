// tecto_internal.cuh - world and batch layout in HBM, launch parameters and device helpers shared
// by the engine's kernels.  Reference paths are relative to MarWo22/master_thesis.
//
// Every phase runs over a batch: a table of world descriptors plus, per phase, one work list of
// (world, tile) items, so many uneven worlds advance in one launch per phase.  A world stepped on
// its own is a batch of one.
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tecto.h"
#include "../../include/tecto_math.h"

namespace tecto {

constexpr int kPlates = TECTO_MAX_PLATES;       // plate ids 0..254; byte 0 in a word = no plate
constexpr int kPairs = TECTO_NUM_PAIRS;
constexpr int kDivWords = TECTO_NUM_DIV_WORDS;
constexpr int kSortTile = 4096;                 // keys per onesweep tile (256 threads x 16)
constexpr int kSortThreads = 256;
constexpr int kSortItems = kSortTile / kSortThreads;
constexpr int kMaxSortPasses = 4;               // 32-bit keys, 8-bit digits
constexpr int kMaxRadixBits = 11;              // widest sort digit
constexpr int kMaxBatchWorlds = 1024;           // worlds per batch (world lookup table in smem)

// Status word of the decoupled look-back: 2 flag bits + 30 value bits.
constexpr uint32_t kFlagAggregate = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1u;
constexpr uint32_t kSpinLimit = 1u << 24;       // bounded waits: give up, flag, carry on

// Device error flag bits.
constexpr uint32_t kErrLookbackTimeout = 1u;
constexpr uint32_t kErrUpliftCapacity = 2u;    // reference uplift: more bucket entries than its scratch holds

// Per-pair collision evidence, CollisionTypeCounts field order
// (src/cuda_compute/plate_tectonics_kernel.cuh:47-54).
struct PairCounts {
    int c[5];  // subductionsAContinental, subductionsAOceanic, subductionsBContinental,
               // subductionsBOceanic, continental
};

// Per-world device control block; kernels read the step counter from here so that a captured
// graph replays correctly step after step.
struct Control {
    uint32_t iteration;     // PlateTectonicSim::m_iterations
    uint32_t seed;          // PlateTectonicSim::m_seed
    uint32_t error;         // kErr* bits
    uint32_t acc_count;     // entries in this world's accretion list for the current step
    uint32_t comp_count;    // plate relabel: components listed this step
    uint32_t unassigned;    // plate relabel: cells without an id after the lookup
    uint32_t unresolved;    // plate relabel: cells the neighbour fill could not reach (last relabel)
    uint32_t merges;        // plate merges of the last step
    uint32_t pad[8];
};

// Per-batch device control block.
struct BatchCtl {
    uint32_t error;
    uint32_t pad[15];
};

// Scratch of the radix sort (histograms, look-back status).  Sizes in tecto_sort_scratch_bytes.
struct SortScratch {
    uint32_t *hist;      // [passes][2^radix_bits] digit counts -> exclusive digit starts
    uint32_t *status;    // [passes][tiles][2^radix_bits] look-back words
    uint32_t *counters;  // [passes] dynamic tile counters
    uint32_t *error;     // error flag word
    int passes;
    int tiles;
    int radix_bits;      // digit width, 8..kMaxRadixBits
};

// Per-plate sums of plate dynamics, in 64-bit fixed point so that the order of the atomic adds
// does not change the bits: mass (heights x 2^16), the angular centre sums (sin / cos x 2^32) and the
// collision friction (x 2^40).  Consumed and cleared within each step.
struct PlateAcc {
    unsigned long long mass;
    unsigned long long ang[4];  // sin x, cos x, sin y, cos y of the sampled cells
    unsigned long long fric;
    int size;
    int samples;
};

constexpr float kMassScale = 65536.0f;             // 2^16
constexpr float kMassLimit = 1099511627776.0f;     // |h| clamp before scaling, 2^40
constexpr float kAngScale = 4294967296.0f;         // 2^32
constexpr float kFricScale = 1099511627776.0f;     // 2^40
constexpr float kFricLimit = 4194304.0f;           // |friction term| clamp, 2^22
constexpr int kStatTileX = 256, kStatTileY = 16;   // TK_STATS tile
constexpr float kTwoPiF = 6.28318548202514648f;    // CURAND_2PI as a float

// Per-world state of the plate policy (relabel and merges).
struct PolicyState {
    int max_count[256];                // per plate: cells of its largest component
    int merge_ids[256];                // getPlateMerges' table: 0, -1 parent, 255 - parent for a child
    uint32_t neighbors[kDivWords];     // plate pairs that touch (triangle bits)
    unsigned long long top[256];       // ranked components (count << 32 | label)
    int any_merge;
    int pad[63];
};

// Device descriptor of one world (one cudaMalloc'd arena per world, structure of arrays).
struct WorldDev {
    int W, H;
    uint32_t N;
    uint32_t vbase;         // first virtual cell index of this world in its batch
    float *h[2];            // height, ping-pong
    float *w[2];            // water
    float *s[2];            // sediment
    float4 *flux[2];        // outflow flux (left, +y, right, -y)
    uint8_t *id[2];         // plate ids
    uint32_t *word;         // packed arrivals per destination cell
    uint32_t *labels;       // CCL labels
    float *rain;            // this step's rain increment per cell (constant over sub-iterations)
    float2 *vel;            // water velocity, split hydraulic path only
    float *s1;              // sediment before transport, split hydraulic path only
    unsigned long long *acc;  // accretion marks: ((dest + 1) << 8) | (255 - owner), atomicMax
    uint32_t *acc_list;     // cells holding a mark this step (count in ctl->acc_count)
    uint8_t *acc_u8;        // decoded marks of the last step (download only)
    uint8_t *type_bitmap;   // [kPairs]
    uint32_t *div_bitmap;   // [kDivWords]
    uint32_t *has_div;      // [kDivWords]
    PairCounts *counts;     // [kPairs]
    tecto_plate *plates;    // [kPlates]
    tecto_plate *plates_prev;  // [kPlates] plate records before this step's centre update
    int2 *off;              // [kPlates + 1] this step's integer displacement per plate
    tecto_plate_dynamics *dyn;  // [kPlates] plate dynamics records
    PlateAcc *pacc;         // [kPlates] plate dynamics sums of the current step
    PolicyState *policy;    // plate relabel and merges
    const float *pressure;  // asthenosphere pressure texture (pw x ph), or null
    int pw, ph;
    Control *ctl;
};

// Batch-level scratch of the reference uplift (TECTO_UPLIFT_REFERENCE), indexed by virtual cell.
struct UpliftRefScratch {
    size_t cells = 0;       // capacity in cells
    size_t ecap = 0;        // capacity in bucket entries
    void *arena = nullptr;
    float *upl_h = nullptr;       // processConvergence's heightAddition (convergent cells)
    uint8_t *upl_t = nullptr;     // processConvergence's typeByte
    uint32_t *cnt = nullptr;      // entries per target cell, then fill cursor
    uint32_t *off = nullptr;      // first entry of each target cell
    uint32_t *blk = nullptr;      // scan block totals
    uint32_t *succ = nullptr;     // per source: bit (2k + j) set when its insert event succeeded
    float *prop_h = nullptr;      // PropagatedUpliftData, structure of arrays
    uint32_t *prop_inv = nullptr;
    uint8_t *prop_t = nullptr;
    int32_t *jfa[2] = {};         // nearest seed (world-local cell index) or -1
    int32_t *dist = nullptr;      // JFAComputeDistance: distance to the seed, -1 none
    uint32_t *ent_key = nullptr;  // bucket entries: (source virtual cell << 3) | slot
    uint32_t *ent_val = nullptr;  // payload: plate pair, or a contribution's bits
};

// Phase work lists.
enum TileKind { TK_RESOLVE = 0, TK_THERMAL, TK_HYDRO, TK_CCL, TK_STATS, TK_COUNT };
// CCL tiles: one warp per row of kCclTileX cells, kCclTileY rows per block
constexpr int kCclTileX = 32, kCclTileY = 32;

// One batch: members, their device table, work lists and the batch-level buffers.
struct Batch {
    std::vector<tecto_world *> members;
    tecto_settings settings{};
    bool has_settings = false;
    int device = 0;
    int cur_h = 0, cur_wsf = 0, cur_id = 0;  // aligned ping-pong halves of every member
    int sort_final = 0;
    size_t total = 0;                        // sum of member cells
    int hydro_variant = 0;                   // tile variant the TK_HYDRO list was built for
    int thermal_variant = 0;                 // tile variant the TK_THERMAL list was built for
    int tuned_thermal = 0;
    int tuned_hydro = 0, tuned_rb = 0;       // autotuner's choices (0 = none), used when the
                                             // settings leave hydraulicTile / sortRadixBits at 0
    uint64_t launches = 0;
    bool dirty = true;                       // tables must be rebuilt before the next launch
    // device tables
    WorldDev *d_worlds = nullptr;
    uint32_t *d_vbase = nullptr;             // [n + 1] ascending virtual bases, last = total
    uint2 *d_tiles[TK_COUNT] = {};           // (world, ty << 16 | tx)
    int ntiles[TK_COUNT] = {};
    // column strips of the marching hydraulic kernel (hydraulic variant kHydroStripVariant):
    // {world, first column, interior width, first strip-row}, strip-rows counted over all strips
    uint4 *d_strips = nullptr;
    int nstrips = 0;
    unsigned long long strip_rows = 0;
    void *table_arena = nullptr;
    size_t table_bytes = 0;
    // batch-level buffers, sized for `capacity` cells
    size_t capacity = 0;
    void *arena = nullptr;
    uint32_t *keys[2] = {};
    uint32_t *vals[2] = {};
    size_t arena_bytes = 0;
    BatchCtl *bctl = nullptr;
    SortScratch sort{};
    UpliftRefScratch upref{};
    int upref_final = 0;                     // jfa[] half holding the last step's seeds
    void *stage = nullptr;                   // packed host transfers: one field of every member
    size_t stage_bytes = 0;
    // pipelined packed transfers: per field two upload and two download staging buffers, used in
    // turn, the events that order the copy streams against the compute stream, and how many stages,
    // commits, gathers and fetches each field has seen (a stage may run up to two commits ahead)
    void *up_stage[6][2] = {}, *down_stage[6][2] = {};
    size_t up_bytes[6] = {}, down_bytes[6] = {};
    cudaEvent_t ev_up_ready[6][2] = {}, ev_up_free[6][2] = {}, ev_down_ready[6][2] = {}, ev_down_free[6][2] = {};
    uint64_t n_staged[6] = {}, n_committed[6] = {}, n_gathered[6] = {}, n_fetched[6] = {};
    // graphs of one step keyed by (cur_h, cur_wsf, cur_id, ccl)
    cudaGraphExec_t graphs[16] = {};
    bool graph_valid[16] = {};
    int graph_end[16][4] = {};
    uint64_t graph_launches[16] = {};
};

}  // namespace tecto

struct tecto_world {
    int W = 0, H = 0;
    size_t N = 0;
    int device = 0;
    tecto_settings settings{};
    uint32_t seed = 0;
    uint32_t iteration = 0;        // host mirror of ctl->iteration
    int cur_h = 0, cur_wsf = 0, cur_id = 0;  // which ping-pong half holds the state
    uint64_t launches = 0;         // kernels enqueued for this world
    void *arena = nullptr;
    size_t arena_bytes = 0;
    tecto::WorldDev dev{};         // host copy of the device descriptor
    tecto::Batch *own = nullptr;   // private batch of one, for stepping alone
    tecto::Batch *in_batch = nullptr;  // the batch it currently belongs to (own or public)
    float *pressure = nullptr;     // asthenosphere pressure texture (own allocation), or null
    int pw = 0, ph = 0;
};

struct tecto_batch {
    tecto::Batch b;
};

namespace tecto {

// Thread-local last error text for tecto_last_error_string.
void set_error(const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

#define TECTO_CUDA(call)                                          \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return ::tecto::cuda_fail(e_, #call); \
    } while (0)

// ---- device helpers ---------------------------------------------------------------------

// CudaTexture::wrapCoordinate (src/cuda_compute/types/cuda_texture.cuh:67-76)
__host__ __device__ __forceinline__ int wrapc(int c, int n)
{
    const int r = c % n;
    return r + (n & (r >> 31));
}

// Same result as wrapc; coordinates within one period of the grid (c in [-n, 2n), the case of
// every stencil halo and plate displacement) wrap without an integer division.
__host__ __device__ __forceinline__ int wrap_fast(int c, int n)
{
    if ((unsigned)(c + n) < 3u * (unsigned)n) {
        c = c < 0 ? c + n : c;
        return c >= n ? c - n : c;
    }
    return wrapc(c, n);
}

__host__ __device__ __forceinline__ uint32_t cidx(int x, int y, int W, int H)
{
    return (uint32_t)(wrap_fast(y, H) * W + wrap_fast(x, W));
}

// upperTriangleIndexUnchecked(i, j, 255), i < j (src/cuda_compute/cuda_helper.cuh:97-104)
__host__ __device__ __forceinline__ uint32_t tri_index(uint32_t i, uint32_t j)
{
    return i * (2u * kPlates - i - 1u) / 2u + (j - i - 1u);
}

// The world owning virtual cell v: largest b with vbase[b] <= v (vbase ascending, n entries).
__device__ __forceinline__ int find_world(const uint32_t *vbase, int n, uint32_t v)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (vbase[mid] <= v) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void tile_of(uint2 t, int *world, int *tx, int *ty)
{
    *world = (int)t.x;
    *tx = (int)(t.y & 0xffffu);
    *ty = (int)(t.y >> 16);
}

// ---- batch management (tecto_batch.cu) -----------------------------------------------------
int batch_prepare(Batch &b, cudaStream_t st);        // (re)build tables and buffers if dirty
int batch_enqueue_step(Batch &b, cudaStream_t st, int ccl);  // 0 none, 1 all, 2 where due
int batch_step(Batch &b, int nsteps, cudaStream_t st);
int batch_step_graph(Batch &b, int nsteps, cudaStream_t st, bool use_graph);
void batch_release(Batch &b);
int batch_join(Batch &b, tecto_world *w, cudaStream_t st);
int batch_leave(Batch &b, tecto_world *w);
int tile_extent(int kind, int variant, int *tx, int *ty);

// ---- phase launchers (each enqueues on `st` for every member of the batch) -----------------
int launch_plates(Batch &b, cudaStream_t st);
int launch_sort_keys(Batch &b, cudaStream_t st);
int launch_words(Batch &b, cudaStream_t st);
int launch_type_matrix(Batch &b, cudaStream_t st);
int launch_resolve(Batch &b, cudaStream_t st);
int launch_thermal(Batch &b, int iterations, cudaStream_t st);
int launch_hydraulic(Batch &b, int iterations, float dt, cudaStream_t st);
int launch_finish(Batch &b, cudaStream_t st);
// plate dynamics (TECTO_PLATE_DYNAMICS_REFERENCE): per-plate sums at the start of a step, and
// applyPlateMovementChanges at its end
int launch_plate_stats(Batch &b, cudaStream_t st);
int launch_plate_motion(Batch &b, cudaStream_t st);
// plate policy after a step (TECTO_PLATE_RELABEL / TECTO_PLATE_MERGE): ccl 0 no labelling ran, 1 it
// ran for the world (single world), 2 per world when due (batch)
int launch_plate_policy(Batch &b, int ccl, cudaStream_t st);
int launch_clear_marks(Batch &b, cudaStream_t st);
int launch_bump_iteration(Batch &b, cudaStream_t st);
// due_only: skip worlds whose step counter is not a multiple of iterationsForCCL
int launch_ccl(Batch &b, int connectivity, bool due_only, cudaStream_t st);
int launch_uplift_ref(Batch &b, cudaStream_t st);          // k_uplift.cu, after launch_resolve
int uplift_ref_prepare(Batch &b, cudaStream_t st);         // allocate the scratch when the mode needs it
void uplift_ref_release(Batch &b);
void gaussian_weights(float sigma, int radius, float *out);
int ensure_kernel_attributes();
int hydro_variant_for(const tecto_settings &s);  // 0 when the settings leave the choice open
constexpr int kDefaultRadixBits = 8;
constexpr int kHydroVariantCount = 9;
constexpr int kDefaultHydroVariant = 4;          // 64 x 32 cells, 1024 threads
constexpr int kHydroStripVariant = 8;            // marching column strips in registers (fused path only)
constexpr int kHydroMarchVariant = 9;            // marching row chunks in shared memory (fused path only)
constexpr int kStripInner = 56;                  // interior columns of one register strip (64 with the halo)
constexpr int kMarchInner = 120;                 // interior columns of one shared-memory strip (128 with it)
// the strip table of a batch: every member's columns cut into strips of kStripInner columns for
// kHydroStripVariant, of kMarchInner otherwise (the marching hydraulic and thermal kernels)
void build_strips(const Batch &b, std::vector<uint4> &out, unsigned long long *rows);
constexpr int kThermalVariantCount = 5;
constexpr int kDefaultThermalVariant = 4;        // 64 x 16 cells, 512 threads, 2 iterations per launch
constexpr int kThermalMarchVariant = 5;          // marching row chunks down column strips, one iteration per launch
int thermal_variant_for(const tecto_settings &s);  // 0 when the settings leave the choice open

// Autotuner cache (tecto_tune.cu): best hydraulic tile variant and sort digit width for a batch
// shape class on a device; false when nothing was tuned for that class.
bool tune_lookup(int device, size_t total_cells, size_t worlds, int *hydro, int *rb, int *thermal);
int tune_batch(Batch &b, cudaStream_t st, tecto_tuning *out);  // tune on the members' shapes, apply

// Radix sort core (k_sort.cu).  If worlds != nullptr the first pass generates the keys (the
// batch-virtual destination cell of every virtual cell) and values (the virtual source cell)
// from each world's plate ids and per-plate displacement; otherwise it reads keys_in/vals_in.
// Returns the half (0/1) of keys/vals holding the result.
struct SortArgs {
    const WorldDev *worlds;
    const uint32_t *vbase;
    int nworlds;
    int cur_id;
    const uint32_t *keys_in;
    const uint32_t *vals_in;
    uint32_t *keys[2];
    uint32_t *vals[2];
    size_t n;
    int key_bits;
};
bool valid_radix_bits(int rb);
int sort_passes_for(int key_bits, int rb);
size_t sort_scratch_bytes(size_t n, int key_bits, int rb);
void sort_scratch_carve(void *base, size_t n, int key_bits, int rb, SortScratch *out);
int run_sort(const SortArgs &a, const SortScratch &scr, cudaStream_t st, int *result_half);
int sort_kernel_attributes();  // once, outside graph capture, before any digit width above 8

int key_bits_for(size_t n);

}  // namespace tecto
