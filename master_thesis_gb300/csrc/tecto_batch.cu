// tecto_batch.cu - batches of worlds: device tables, per-phase (world, tile) work lists,
// batch-level buffers, ping-pong alignment of members, and the step driver with CUDA-graph
// replay.  A world stepped on its own uses a private batch of one.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "tecto_internal.cuh"

namespace tecto {

namespace {

size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

void drop_graphs(Batch &b)
{
    for (int i = 0; i < 16; ++i) {
        if (b.graph_valid[i]) cudaGraphExecDestroy(b.graphs[i]);
        b.graph_valid[i] = false;
    }
}

void build_tiles(const Batch &b, int kind, std::vector<uint2> &out)
{
    int tx = 0, ty = 0;
    tile_extent(kind, kind == TK_THERMAL ? b.thermal_variant : b.hydro_variant, &tx, &ty);
    out.clear();
    for (size_t wi = 0; wi < b.members.size(); ++wi) {
        const tecto_world *w = b.members[wi];
        const int nx = (w->W + tx - 1) / tx, ny = (w->H + ty - 1) / ty;
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) out.push_back(make_uint2((unsigned)wi, ((unsigned)y << 16) | (unsigned)x));
    }
}

}  // namespace

void build_strips(const Batch &b, std::vector<uint4> &out, unsigned long long *rows)
{
    out.clear();
    const int inner = b.hydro_variant == kHydroStripVariant ? kStripInner : kMarchInner;
    unsigned long long r = 0;
    for (size_t wi = 0; wi < b.members.size(); ++wi) {
        const tecto_world *w = b.members[wi];
        for (int x0 = 0; x0 < w->W; x0 += inner) {
            const int iw = std::min(inner, w->W - x0);
            out.push_back(make_uint4((unsigned)wi, (unsigned)x0, (unsigned)iw, (unsigned)r));
            r += (unsigned long long)w->H;
        }
    }
    *rows = r;
}

namespace {

// Copy the state of group `g` (0 height, 1 water/sediment/flux, 2 plate ids) of world w into
// ping-pong half `to`.
int move_half(tecto_world *w, int g, int to, cudaStream_t st)
{
    const size_t N = w->N;
    const int from = to ^ 1;
    if (g == 0) {
        TECTO_CUDA(cudaMemcpyAsync(w->dev.h[to], w->dev.h[from], N * 4, cudaMemcpyDeviceToDevice, st));
    } else if (g == 1) {
        TECTO_CUDA(cudaMemcpyAsync(w->dev.w[to], w->dev.w[from], N * 4, cudaMemcpyDeviceToDevice, st));
        TECTO_CUDA(cudaMemcpyAsync(w->dev.s[to], w->dev.s[from], N * 4, cudaMemcpyDeviceToDevice, st));
        TECTO_CUDA(cudaMemcpyAsync(w->dev.flux[to], w->dev.flux[from], N * 16, cudaMemcpyDeviceToDevice, st));
    } else {
        TECTO_CUDA(cudaMemcpyAsync(w->dev.id[to], w->dev.id[from], N, cudaMemcpyDeviceToDevice, st));
    }
    return TECTO_OK;
}

// Whether two worlds step alike: every parameter a step reads (the kernel and step settings and the
// CCL period).  The rest of SimulationSettings (plate count, seed, Voronoi generations) is read by
// the initialisation only, so worlds initialised differently may share a batch.
bool same_step_settings(const tecto_settings &a, const tecto_settings &b)
{
    return std::memcmp(&a.kernel, &b.kernel, sizeof(a.kernel)) == 0 &&
           std::memcmp(&a.step, &b.step, sizeof(a.step)) == 0 && a.sim.iterationsForCCL == b.sim.iterationsForCCL;
}

}  // namespace

int batch_join(Batch &b, tecto_world *w, cudaStream_t st)
{
    if (std::find(b.members.begin(), b.members.end(), w) != b.members.end()) return TECTO_OK;
    if ((int)b.members.size() >= kMaxBatchWorlds) {
        set_error("batch is full (1024 worlds)");
        return TECTO_ERR_INVALID;
    }
    if (b.members.empty()) {
        b.settings = w->settings;
        b.has_settings = true;
        b.device = w->device;
        b.cur_h = w->cur_h;
        b.cur_wsf = w->cur_wsf;
        b.cur_id = w->cur_id;
    } else {
        if (!same_step_settings(b.settings, w->settings)) {
            set_error("all worlds of a batch must share the same step settings");
            return TECTO_ERR_INVALID;
        }
        if (w->device != b.device) {
            set_error("all worlds of a batch must live on the same device");
            return TECTO_ERR_INVALID;
        }
        int rc;
        if (w->cur_h != b.cur_h && (rc = move_half(w, 0, b.cur_h, st)) != TECTO_OK) return rc;
        if (w->cur_wsf != b.cur_wsf && (rc = move_half(w, 1, b.cur_wsf, st)) != TECTO_OK) return rc;
        if (w->cur_id != b.cur_id && (rc = move_half(w, 2, b.cur_id, st)) != TECTO_OK) return rc;
        w->cur_h = b.cur_h;
        w->cur_wsf = b.cur_wsf;
        w->cur_id = b.cur_id;
    }
    b.members.push_back(w);
    b.dirty = true;
    return TECTO_OK;
}

int batch_leave(Batch &b, tecto_world *w)
{
    auto it = std::find(b.members.begin(), b.members.end(), w);
    if (it == b.members.end()) {
        set_error("world is not a member of this batch");
        return TECTO_ERR_INVALID;
    }
    b.members.erase(it);
    b.dirty = true;
    if (b.members.empty()) b.has_settings = false;
    return TECTO_OK;
}

void batch_release(Batch &b)
{
    drop_graphs(b);
    uplift_ref_release(b);
    if (b.table_arena) cudaFree(b.table_arena);
    if (b.arena) cudaFree(b.arena);
    if (b.stage) cudaFree(b.stage);
    for (int f = 0; f < 6; ++f) {
        for (int k = 0; k < 2; ++k) {
            if (b.up_stage[f][k]) cudaFree(b.up_stage[f][k]);
            if (b.down_stage[f][k]) cudaFree(b.down_stage[f][k]);
            b.up_stage[f][k] = b.down_stage[f][k] = nullptr;
            cudaEvent_t *evs[4] = {&b.ev_up_ready[f][k], &b.ev_up_free[f][k], &b.ev_down_ready[f][k],
                                   &b.ev_down_free[f][k]};
            for (cudaEvent_t *e : evs) {
                if (*e) cudaEventDestroy(*e);
                *e = nullptr;
            }
        }
        b.up_bytes[f] = b.down_bytes[f] = 0;
        b.n_staged[f] = b.n_committed[f] = b.n_gathered[f] = b.n_fetched[f] = 0;
    }
    b.table_arena = nullptr;
    b.arena = nullptr;
    b.stage = nullptr;
    b.stage_bytes = 0;
    b.capacity = 0;
    b.arena_bytes = 0;
    b.table_bytes = 0;
    b.members.clear();
}

// Tile variant and digit width: explicit settings first, then the autotuner's choice for this
// batch (or its cached choice for the shape class), then the defaults.
static void choose_tuning(const Batch &b, int *variant, int *rb, int *tvariant)
{
    *tvariant = thermal_variant_for(b.settings);
    if (*tvariant == 0) *tvariant = b.tuned_thermal ? b.tuned_thermal : kDefaultThermalVariant;
    *variant = hydro_variant_for(b.settings);
    if (*variant == 0) *variant = b.tuned_hydro ? b.tuned_hydro : kDefaultHydroVariant;
    *rb = b.settings.step.sortRadixBits;
    if (!valid_radix_bits(*rb)) *rb = valid_radix_bits(b.tuned_rb) ? b.tuned_rb : kDefaultRadixBits;
}

int batch_prepare(Batch &b, cudaStream_t st)
{
    if (b.dirty && !b.members.empty()) {  // membership changed: cached autotuner choice, if any
        size_t cells = 0;
        for (const tecto_world *w : b.members) cells += w->N;
        int th = 0, tr = 0, tt = 0;
        if (tune_lookup(b.device, cells, b.members.size(), &th, &tr, &tt)) {
            b.tuned_hydro = th;
            b.tuned_rb = tr;
            b.tuned_thermal = tt;
        }
    }
    int variant = 0, rb = 0, tvariant = 0;
    choose_tuning(b, &variant, &rb, &tvariant);
    if (!b.dirty && variant == b.hydro_variant && rb == b.sort.radix_bits && tvariant == b.thermal_variant)
        return TECTO_OK;
    if (b.members.empty()) {
        set_error("batch has no worlds");
        return TECTO_ERR_INVALID;
    }
    int rc = ensure_kernel_attributes();
    if (rc != TECTO_OK) return rc;
    if ((rc = sort_kernel_attributes()) != TECTO_OK) return rc;
    drop_graphs(b);
    b.hydro_variant = variant;
    b.thermal_variant = tvariant;
    const size_t n = b.members.size();
    std::vector<uint32_t> vbase(n + 1);
    size_t total = 0;
    for (size_t i = 0; i < n; ++i) {
        vbase[i] = (uint32_t)total;
        total += b.members[i]->N;
    }
    if (total > (size_t)kValueMask) {
        set_error("batch holds more than 2^30 cells");
        return TECTO_ERR_INVALID;
    }
    vbase[n] = (uint32_t)total;
    b.total = total;
    std::vector<WorldDev> table(n);
    for (size_t i = 0; i < n; ++i) {
        b.members[i]->dev.vbase = vbase[i];
        table[i] = b.members[i]->dev;
    }
    std::vector<uint2> tiles[TK_COUNT];
    size_t need = a256(n * sizeof(WorldDev)) + a256((n + 1) * 4);
    for (int k = 0; k < TK_COUNT; ++k) {
        build_tiles(b, k, tiles[k]);
        b.ntiles[k] = (int)tiles[k].size();
        need += a256(tiles[k].size() * sizeof(uint2));
    }
    std::vector<uint4> strips;
    build_strips(b, strips, &b.strip_rows);
    b.nstrips = (int)strips.size();
    need += a256(strips.size() * sizeof(uint4));
    if (need > b.table_bytes) {
        if (b.table_arena) cudaFree(b.table_arena);
        b.table_arena = nullptr;
        b.table_bytes = 0;
        TECTO_CUDA(cudaMalloc(&b.table_arena, need));
        b.table_bytes = need;
    }
    char *p = (char *)b.table_arena;
    b.d_worlds = (WorldDev *)p;
    p += a256(n * sizeof(WorldDev));
    b.d_vbase = (uint32_t *)p;
    p += a256((n + 1) * 4);
    for (int k = 0; k < TK_COUNT; ++k) {
        b.d_tiles[k] = (uint2 *)p;
        p += a256(tiles[k].size() * sizeof(uint2));
    }
    b.d_strips = (uint4 *)p;
    p += a256(strips.size() * sizeof(uint4));
    TECTO_CUDA(cudaMemcpyAsync(b.d_worlds, table.data(), n * sizeof(WorldDev), cudaMemcpyHostToDevice, st));
    TECTO_CUDA(cudaMemcpyAsync(b.d_vbase, vbase.data(), (n + 1) * 4, cudaMemcpyHostToDevice, st));
    for (int k = 0; k < TK_COUNT; ++k)
        TECTO_CUDA(cudaMemcpyAsync(b.d_tiles[k], tiles[k].data(), tiles[k].size() * sizeof(uint2),
                                   cudaMemcpyHostToDevice, st));
    TECTO_CUDA(cudaMemcpyAsync(b.d_strips, strips.data(), strips.size() * sizeof(uint4), cudaMemcpyHostToDevice,
                               st));
    // batch-level buffers: key/value ping-pong for `capacity` cells, the control block, then the
    // sort scratch of the current size and digit width
    const int kb = key_bits_for(total);
    {
        const size_t cap = std::max(b.capacity, total);
        const size_t need = 4 * a256(cap * 4) + a256(sizeof(BatchCtl)) + a256(sort_scratch_bytes(total, kb, rb));
        if (need > b.arena_bytes) {
            if (b.arena) cudaFree(b.arena);
            b.arena = nullptr;
            b.capacity = 0;
            b.arena_bytes = 0;
            TECTO_CUDA(cudaMalloc(&b.arena, need));
            TECTO_CUDA(cudaMemsetAsync(b.arena, 0, need, st));
            const size_t arr = a256(cap * 4);
            char *q = (char *)b.arena;
            b.keys[0] = (uint32_t *)q;
            b.keys[1] = (uint32_t *)(q + arr);
            b.vals[0] = (uint32_t *)(q + 2 * arr);
            b.vals[1] = (uint32_t *)(q + 3 * arr);
            b.bctl = (BatchCtl *)(q + 4 * arr);
            b.capacity = cap;
            b.arena_bytes = need;
        }
    }
    {
        char *q = (char *)b.arena + 4 * a256(b.capacity * 4) + a256(sizeof(BatchCtl));
        sort_scratch_carve(q, total, kb, rb, &b.sort);
    }
    if ((rc = uplift_ref_prepare(b, st)) != TECTO_OK) return rc;
    // the error word may now sit where a larger batch kept look-back status words
    TECTO_CUDA(cudaMemsetAsync(b.sort.error, 0, 4, st));
    TECTO_CUDA(cudaStreamSynchronize(st));
    b.dirty = false;
    return TECTO_OK;
}

// ccl: 0 none, 1 every member (the caller checked it is due), 2 members whose counter is due
int batch_enqueue_step(Batch &b, cudaStream_t st, int ccl)
{
    int rc;
    const tecto_settings &s = b.settings;
    if ((rc = launch_plates(b, st)) != TECTO_OK) return rc;
    if ((rc = launch_sort_keys(b, st)) != TECTO_OK) return rc;
    if ((rc = launch_words(b, st)) != TECTO_OK) return rc;
    if ((rc = launch_type_matrix(b, st)) != TECTO_OK) return rc;
    if ((rc = launch_resolve(b, st)) != TECTO_OK) return rc;
    if (s.step.upliftMode == TECTO_UPLIFT_REFERENCE && (rc = launch_uplift_ref(b, st)) != TECTO_OK) return rc;
    if ((rc = launch_thermal(b, s.step.thermalIterations, st)) != TECTO_OK) return rc;
    if ((rc = launch_hydraulic(b, s.step.hydraulicIterations, s.step.hydraulicDt, st)) != TECTO_OK) return rc;
    if ((rc = launch_finish(b, st)) != TECTO_OK) return rc;
    if (ccl && (rc = launch_ccl(b, s.step.cclConnectivity, ccl == 2, st)) != TECTO_OK) return rc;
    if (s.step.platePolicy && (rc = launch_plate_policy(b, ccl, st)) != TECTO_OK) return rc;
    return launch_bump_iteration(b, st);
}

static void sync_members(Batch &b)
{
    for (tecto_world *w : b.members) {
        w->cur_h = b.cur_h;
        w->cur_wsf = b.cur_wsf;
        w->cur_id = b.cur_id;
    }
}

int batch_step(Batch &b, int nsteps, cudaStream_t st) { return batch_step_graph(b, nsteps, st, true); }

// use_graph false: plain launches (worth it right after a membership change, when a captured
// graph would be used once)
int batch_step_graph(Batch &b, int nsteps, cudaStream_t st, bool use_graph)
{
    int rc = batch_prepare(b, st);
    if (rc != TECTO_OK) return rc;
    const int period = b.settings.sim.iterationsForCCL > 0 ? b.settings.sim.iterationsForCCL : 1;
    for (int s = 0; s < nsteps; ++s) {
        int ccl;
        if (b.members.size() == 1) ccl = (b.members[0]->iteration % (uint32_t)period == 0) ? 1 : 0;
        else ccl = 2;
        const uint64_t before = b.launches;
        if (st == nullptr || !use_graph) {  // the legacy stream cannot be captured
            if ((rc = batch_enqueue_step(b, st, ccl)) != TECTO_OK) return rc;
        } else {
            const int key = b.cur_h | (b.cur_wsf << 1) | (b.cur_id << 2) | ((ccl == 1 ? 1 : 0) << 3);
            if (!b.graph_valid[key]) {
                cudaGraph_t g = nullptr;
                TECTO_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                rc = batch_enqueue_step(b, st, ccl);
                const cudaError_t ce = cudaStreamEndCapture(st, &g);
                if (rc != TECTO_OK) {
                    if (g) cudaGraphDestroy(g);
                    return rc;
                }
                if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
                cudaGraphExec_t ex = nullptr;
                const cudaError_t ie = cudaGraphInstantiate(&ex, g, 0);
                cudaGraphDestroy(g);
                if (ie != cudaSuccess) return cuda_fail(ie, "cudaGraphInstantiate");
                b.graphs[key] = ex;
                b.graph_valid[key] = true;
                b.graph_end[key][0] = b.cur_h;
                b.graph_end[key][1] = b.cur_wsf;
                b.graph_end[key][2] = b.cur_id;
                b.graph_end[key][3] = b.sort_final;
                b.graph_launches[key] = b.launches - before;
                TECTO_CUDA(cudaGraphLaunch(ex, st));
            } else {
                TECTO_CUDA(cudaGraphLaunch(b.graphs[key], st));
                b.cur_h = b.graph_end[key][0];
                b.cur_wsf = b.graph_end[key][1];
                b.cur_id = b.graph_end[key][2];
                b.sort_final = b.graph_end[key][3];
                b.launches += b.graph_launches[key];
            }
        }
        const uint64_t step_launches = b.launches - before;
        for (tecto_world *w : b.members) {
            w->iteration += 1;
            w->launches += step_launches;
        }
        sync_members(b);
    }
    return TECTO_OK;
}

}  // namespace tecto

using namespace tecto;

extern "C" {

int tecto_batch_create(tecto_batch **out)
{
    if (!out) return TECTO_ERR_INVALID;
    *out = new (std::nothrow) tecto_batch();
    return *out ? TECTO_OK : TECTO_ERR_OOM;
}

int tecto_batch_destroy(tecto_batch *batch)
{
    if (!batch) return TECTO_OK;
    for (tecto_world *w : batch->b.members) w->in_batch = nullptr;
    batch_release(batch->b);
    delete batch;
    return TECTO_OK;
}

int tecto_batch_add(tecto_batch *batch, tecto_world *world, tecto_stream_t stream)
{
    if (!batch || !world) return TECTO_ERR_INVALID;
    if (world->in_batch && world->in_batch != world->own) {
        set_error("world already belongs to a batch");
        return TECTO_ERR_INVALID;
    }
    const int rc = batch_join(batch->b, world, (cudaStream_t)stream);
    if (rc == TECTO_OK) world->in_batch = &batch->b;
    return rc;
}

int tecto_batch_remove(tecto_batch *batch, tecto_world *world)
{
    if (!batch || !world) return TECTO_ERR_INVALID;
    const int rc = batch_leave(batch->b, world);
    if (rc == TECTO_OK) world->in_batch = nullptr;
    return rc;
}

int tecto_batch_step(tecto_batch *batch, int nSteps, tecto_stream_t stream)
{
    if (!batch || nSteps < 0) return TECTO_ERR_INVALID;
    if (batch->b.members.empty()) return TECTO_OK;
    return batch_step(batch->b, nSteps, (cudaStream_t)stream);
}

int tecto_batch_phase_hydraulic(tecto_batch *batch, int iterations, float dt, tecto_stream_t stream)
{
    if (!batch || iterations < 0 || !std::isfinite(dt)) return TECTO_ERR_INVALID;
    Batch &b = batch->b;
    if (b.members.empty()) return TECTO_OK;
    const cudaStream_t st = (cudaStream_t)stream;
    int rc = batch_prepare(b, st);
    if (rc != TECTO_OK) return rc;
    const uint64_t before = b.launches;
    rc = launch_hydraulic(b, iterations, dt, st);
    for (tecto_world *w : b.members) w->launches += b.launches - before;
    sync_members(b);
    return rc;
}

int tecto_batch_phase_thermal(tecto_batch *batch, int iterations, tecto_stream_t stream)
{
    if (!batch || iterations < 0) return TECTO_ERR_INVALID;
    Batch &b = batch->b;
    if (b.members.empty()) return TECTO_OK;
    const cudaStream_t st = (cudaStream_t)stream;
    int rc = batch_prepare(b, st);
    if (rc != TECTO_OK) return rc;
    const uint64_t before = b.launches;
    rc = launch_thermal(b, iterations, st);
    for (tecto_world *w : b.members) w->launches += b.launches - before;
    sync_members(b);
    return rc;
}

int tecto_batch_size(const tecto_batch *batch, int *worlds, size_t *cells)
{
    if (!batch) return TECTO_ERR_INVALID;
    size_t c = 0;
    for (const tecto_world *w : batch->b.members) c += w->N;
    if (worlds) *worlds = (int)batch->b.members.size();
    if (cells) *cells = c;
    return TECTO_OK;
}

int tecto_batch_launch_count(const tecto_batch *batch, uint64_t *count)
{
    if (!batch || !count) return TECTO_ERR_INVALID;
    *count = batch->b.launches;
    return TECTO_OK;
}

int tecto_batch_check(tecto_batch *batch, tecto_stream_t stream)
{
    if (!batch) return TECTO_ERR_INVALID;
    for (tecto_world *w : batch->b.members) {
        const int rc = tecto_world_check(w, stream);
        if (rc != TECTO_OK) return rc;
    }
    if (batch->b.sort.error) {
        uint32_t e = 0;
        TECTO_CUDA(cudaMemcpy(&e, batch->b.sort.error, 4, cudaMemcpyDeviceToHost));
        if (e) {
            cudaMemset(batch->b.sort.error, 0, 4);
            set_error("a bounded device-side wait gave up");
            return TECTO_ERR_DEVICE_TIMEOUT;
        }
    }
    return TECTO_OK;
}

}  // extern "C"
