// tecto_api.cu - the C ABI: world lifecycle and HBM arena, synthetic world generator, field I/O,
// phase entry points and the step driver with CUDA-graph replay.
// Replaces PlateTectonicSim (src/cuda_compute/plate_tectonic_sim.h:110-130,
// plate_tectonic_sim.cu:28-131) for the hot-path phases.
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "tecto_internal.cuh"

namespace tecto {

namespace {
thread_local std::string g_last_error;

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// splitmix64 (Steele, Lea and Flood, 2014): the generator's only source of randomness
inline uint64_t splitmix64(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline float u01(uint64_t r) { return (float)(r >> 40) * (1.0f / 16777216.0f); }

// Device-side world layout: every buffer of the world in one allocation.
struct Layout {
    size_t off[40];
    int n = 0;
    size_t total = 0;
    size_t add(size_t bytes)
    {
        const size_t o = total;
        off[n++] = o;
        total += align256(bytes);
        return o;
    }
};

int check_world(const tecto_world *w)
{
    if (!w || !w->arena) {
        set_error("null or destroyed world");
        return TECTO_ERR_INVALID;
    }
    return TECTO_OK;
}

void field_info(tecto_world *w, int field, void **ptr, size_t *bytes)
{
    const size_t N = w->N;
    *ptr = nullptr;
    *bytes = 0;
    switch (field) {
        case TECTO_FIELD_HEIGHT: *ptr = w->b.h[w->cur_h]; *bytes = N * 4; break;
        case TECTO_FIELD_WATER: *ptr = w->b.w[w->cur_wsf]; *bytes = N * 4; break;
        case TECTO_FIELD_SEDIMENT: *ptr = w->b.s[w->cur_wsf]; *bytes = N * 4; break;
        case TECTO_FIELD_FLUX: *ptr = w->b.flux[w->cur_wsf]; *bytes = N * 16; break;
        case TECTO_FIELD_PLATE_ID: *ptr = w->b.id[w->cur_id]; *bytes = N; break;
        case TECTO_FIELD_LABELS: *ptr = w->b.labels; *bytes = N * 4; break;
        case TECTO_FIELD_COLLISION: *ptr = w->b.word; *bytes = N * 4; break;
        case TECTO_FIELD_TYPE_BITMAP: *ptr = w->b.type_bitmap; *bytes = kPairs; break;
        case TECTO_FIELD_DIV_BITMAP: *ptr = w->b.div_bitmap; *bytes = kDivWords * 4; break;
        case TECTO_FIELD_SORT_KEYS: *ptr = w->b.keys[w->sort_final]; *bytes = N * 4; break;
        case TECTO_FIELD_SORT_VALS: *ptr = w->b.vals[w->sort_final]; *bytes = N * 4; break;
        case TECTO_FIELD_ACCRETION: *ptr = w->b.acc_u8; *bytes = N; break;
        default: break;
    }
}

int bind_device(const tecto_world *w)
{
    int cur = -1;
    TECTO_CUDA(cudaGetDevice(&cur));
    if (cur != w->device) TECTO_CUDA(cudaSetDevice(w->device));
    return TECTO_OK;
}

void drop_graphs(tecto_world *w)
{
    for (int i = 0; i < 16; ++i) {
        if (w->graph_valid[i]) cudaGraphExecDestroy(w->graphs[i]);
        w->graph_valid[i] = false;
    }
}

int enqueue_collide(tecto_world *w, cudaStream_t st)
{
    int rc;
    if ((rc = launch_plates(w, st)) != TECTO_OK) return rc;
    if ((rc = launch_sort_keys(w, st)) != TECTO_OK) return rc;
    if ((rc = launch_words(w, st)) != TECTO_OK) return rc;
    return launch_type_matrix(w, st);
}

bool ccl_due(const tecto_world *w)
{
    const int period = w->settings.sim.iterationsForCCL > 0 ? w->settings.sim.iterationsForCCL : 1;
    return w->iteration % (uint32_t)period == 0;
}

int enqueue_finish(tecto_world *w, cudaStream_t st, bool ccl)
{
    int rc;
    if ((rc = launch_finish(w, st)) != TECTO_OK) return rc;
    if (ccl && (rc = launch_ccl(w, w->settings.step.cclConnectivity, st)) != TECTO_OK) return rc;
    if ((rc = launch_bump_iteration(w, st)) != TECTO_OK) return rc;
    w->iteration += 1;
    return TECTO_OK;
}

int enqueue_step(tecto_world *w, cudaStream_t st, bool ccl)
{
    int rc;
    if ((rc = enqueue_collide(w, st)) != TECTO_OK) return rc;
    if ((rc = launch_resolve(w, st)) != TECTO_OK) return rc;
    if ((rc = launch_thermal(w, w->settings.step.thermalIterations, st)) != TECTO_OK) return rc;
    if ((rc = launch_hydraulic(w, w->settings.step.hydraulicIterations, w->settings.step.hydraulicDt,
                               st)) != TECTO_OK)
        return rc;
    return enqueue_finish(w, st, ccl);
}

}  // namespace

void set_error(const std::string &msg) { g_last_error = msg; }

int cuda_fail(cudaError_t e, const char *what)
{
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? TECTO_ERR_OOM : TECTO_ERR_CUDA;
}

int ensure_kernel_attributes();

}  // namespace tecto

using namespace tecto;

extern "C" {

const char *tecto_last_error_string(void) { return g_last_error.c_str(); }

const char *tecto_version(void) { return "tecto-gb300 0.1 (sm_103a)"; }

int tecto_world_create(const tecto_settings *settings, int width, int height, uint32_t seed,
                       tecto_world **out)
{
    if (!settings || !out || width < 1 || height < 1) {
        set_error("tecto_world_create: invalid argument");
        return TECTO_ERR_INVALID;
    }
    const size_t N = (size_t)width * (size_t)height;
    if (N > ((size_t)1 << 30)) {
        set_error("tecto_world_create: at most 2^30 cells per world");
        return TECTO_ERR_INVALID;
    }
    *out = nullptr;
    tecto_world *w = new (std::nothrow) tecto_world();
    if (!w) return TECTO_ERR_OOM;
    w->W = width;
    w->H = height;
    w->N = N;
    w->settings = *settings;
    w->seed = seed;
    cudaGetDevice(&w->device);
    const int kb = key_bits_for(N);
    Layout L;
    const size_t o_h0 = L.add(N * 4), o_h1 = L.add(N * 4);
    const size_t o_w0 = L.add(N * 4), o_w1 = L.add(N * 4);
    const size_t o_s0 = L.add(N * 4), o_s1 = L.add(N * 4);
    const size_t o_f0 = L.add(N * 16), o_f1 = L.add(N * 16);
    const size_t o_i0 = L.add(N), o_i1 = L.add(N);
    const size_t o_word = L.add(N * 4);
    const size_t o_k0 = L.add(N * 4), o_k1 = L.add(N * 4);
    const size_t o_v0 = L.add(N * 4), o_v1 = L.add(N * 4);
    const size_t o_lab = L.add(N * 4);
    const size_t o_rain = L.add(N * 4);
    const size_t o_vel = L.add(N * 8);
    const size_t o_s1b = L.add(N * 4);
    const size_t o_acc = L.add(N * 8);
    const size_t o_accl = L.add(N * 4);
    const size_t o_accu = L.add(N);
    const size_t o_bm = L.add(kPairs);
    const size_t o_div = L.add(kDivWords * 4);
    const size_t o_hd = L.add(kDivWords * 4);
    const size_t o_cnt = L.add(kPairs * sizeof(PairCounts));
    const size_t o_pl = L.add(kPlates * sizeof(tecto_plate));
    const size_t o_off = L.add((kPlates + 1) * sizeof(int2));
    const size_t o_ctl = L.add(sizeof(Control));
    const size_t o_sort = L.add(sort_scratch_bytes(N, kb));
    cudaError_t e = cudaMalloc(&w->arena, L.total);
    if (e != cudaSuccess) {
        delete w;
        return cuda_fail(e, "cudaMalloc(world arena)");
    }
    w->arena_bytes = L.total;
    char *base = (char *)w->arena;
    WorldBuffers &b = w->b;
    b.h[0] = (float *)(base + o_h0);
    b.h[1] = (float *)(base + o_h1);
    b.w[0] = (float *)(base + o_w0);
    b.w[1] = (float *)(base + o_w1);
    b.s[0] = (float *)(base + o_s0);
    b.s[1] = (float *)(base + o_s1);
    b.flux[0] = (float4 *)(base + o_f0);
    b.flux[1] = (float4 *)(base + o_f1);
    b.id[0] = (uint8_t *)(base + o_i0);
    b.id[1] = (uint8_t *)(base + o_i1);
    b.word = (uint32_t *)(base + o_word);
    b.keys[0] = (uint32_t *)(base + o_k0);
    b.keys[1] = (uint32_t *)(base + o_k1);
    b.vals[0] = (uint32_t *)(base + o_v0);
    b.vals[1] = (uint32_t *)(base + o_v1);
    b.labels = (uint32_t *)(base + o_lab);
    b.rain = (float *)(base + o_rain);
    b.vel = (float2 *)(base + o_vel);
    b.s1 = (float *)(base + o_s1b);
    b.acc = (unsigned long long *)(base + o_acc);
    b.acc_list = (uint32_t *)(base + o_accl);
    b.acc_u8 = (uint8_t *)(base + o_accu);
    b.type_bitmap = (uint8_t *)(base + o_bm);
    b.div_bitmap = (uint32_t *)(base + o_div);
    b.has_div = (uint32_t *)(base + o_hd);
    b.counts = (PairCounts *)(base + o_cnt);
    b.plates = (tecto_plate *)(base + o_pl);
    b.off = (int2 *)(base + o_off);
    b.ctl = (Control *)(base + o_ctl);
    sort_scratch_carve(base + o_sort, N, kb, &b.sort);
    e = cudaMemset(w->arena, 0, L.total);
    if (e == cudaSuccess) {
        Control c{};
        c.seed = seed;
        e = cudaMemcpy(b.ctl, &c, sizeof(c), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        cudaFree(w->arena);
        delete w;
        return cuda_fail(e, "world init");
    }
    const int rc = ensure_kernel_attributes();
    if (rc != TECTO_OK) {
        cudaFree(w->arena);
        delete w;
        return rc;
    }
    *out = w;
    return TECTO_OK;
}

int tecto_world_destroy(tecto_world *w)
{
    if (!w) return TECTO_OK;
    drop_graphs(w);
    if (w->arena) cudaFree(w->arena);
    w->arena = nullptr;
    delete w;
    return TECTO_OK;
}

int tecto_world_set_settings(tecto_world *w, const tecto_settings *s)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if (!s) return TECTO_ERR_INVALID;
    w->settings = *s;
    drop_graphs(w);
    return TECTO_OK;
}

int tecto_world_get_settings(const tecto_world *w, tecto_settings *out)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if (!out) return TECTO_ERR_INVALID;
    *out = w->settings;
    return TECTO_OK;
}

int tecto_world_size(const tecto_world *w, int *width, int *height)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if (width) *width = w->W;
    if (height) *height = w->H;
    return TECTO_OK;
}

int tecto_generate_world_host(int W, int H, int P, float velRange, uint64_t genSeed, float *height_out,
                              uint8_t *id_out, tecto_plate *plates_out)
{
    if (W < 1 || H < 1 || P < 1 || P > kPlates) {
        set_error("tecto_generate_world_host: invalid size or plate count (1..255)");
        return TECTO_ERR_INVALID;
    }
    uint64_t st = genSeed;
    std::vector<float> sx(P), sy(P);
    std::vector<tecto_plate> pl(kPlates);
    std::memset(pl.data(), 0, sizeof(tecto_plate) * kPlates);
    for (int k = 0; k < P; ++k) {
        sx[k] = u01(splitmix64(st)) * (float)W;
        sy[k] = u01(splitmix64(st)) * (float)H;
        const float vx = (2.0f * u01(splitmix64(st)) - 1.0f) * velRange;
        const float vy = (2.0f * u01(splitmix64(st)) - 1.0f) * velRange;
        const float v = sqrtf(vx * vx + vy * vy);
        pl[k].velocity = v;
        pl[k].direction_x = v > 0.0f ? vx / v : 1.0f;
        pl[k].direction_y = v > 0.0f ? vy / v : 0.0f;
        pl[k].pixelCenter_x = sx[k] - floorf(sx[k]);
        pl[k].pixelCenter_y = sy[k] - floorf(sy[k]);
    }
    if (plates_out) std::memcpy(plates_out, pl.data(), sizeof(tecto_plate) * kPlates);
    const float fW = (float)W, fH = (float)H;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            const size_t i = (size_t)y * W + x;
            float best = 3.4e38f;
            int bid = 0;
            for (int k = 0; k < P; ++k) {
                const float dx = fabsf((float)x - sx[k]), dy = fabsf((float)y - sy[k]);
                const float wx = fminf(dx, fW - dx), wy = fminf(dy, fH - dy);
                const float d2 = wx * wx + wy * wy;
                if (d2 < best) {
                    best = d2;
                    bid = k;
                }
            }
            if (id_out) id_out[i] = (uint8_t)bid;
            if (height_out) {
                // Irwin-Hall: the sum of 12 uniforms minus 6 approximates N(0, 1)
                uint64_t cs = genSeed ^ (0xD1B54A32D192ED03ull * (uint64_t)(i + 1));
                float sum = 0.0f;
                for (int r = 0; r < 12; ++r) sum = sum + u01(splitmix64(cs));
                const float n = sum - 6.0f;
                height_out[i] = (bid % 2 == 0) ? 0.5f + 0.05f * n : -0.5f + 0.02f * n;
            }
        }
    }
    return TECTO_OK;
}

int tecto_world_init_synthetic(tecto_world *w, int P, float velRange, uint64_t genSeed,
                               tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    std::vector<float> h(w->N);
    std::vector<uint8_t> id(w->N);
    std::vector<tecto_plate> pl(kPlates);
    rc = tecto_generate_world_host(w->W, w->H, P, velRange, genSeed, h.data(), id.data(), pl.data());
    if (rc != TECTO_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    drop_graphs(w);
    w->cur_h = w->cur_wsf = w->cur_id = 0;
    w->sort_final = 0;
    w->iteration = 0;
    const size_t N = w->N;
    TECTO_CUDA(cudaMemsetAsync(w->arena, 0, w->arena_bytes, st));
    TECTO_CUDA(cudaMemcpyAsync(w->b.h[0], h.data(), N * 4, cudaMemcpyHostToDevice, st));
    TECTO_CUDA(cudaMemcpyAsync(w->b.id[0], id.data(), N, cudaMemcpyHostToDevice, st));
    TECTO_CUDA(cudaMemcpyAsync(w->b.plates, pl.data(), sizeof(tecto_plate) * kPlates,
                               cudaMemcpyHostToDevice, st));
    Control c{};
    c.seed = w->seed;
    TECTO_CUDA(cudaMemcpyAsync(w->b.ctl, &c, sizeof(c), cudaMemcpyHostToDevice, st));
    TECTO_CUDA(cudaStreamSynchronize(st));
    return TECTO_OK;
}

int tecto_world_field(tecto_world *w, int field, void **device_ptr, size_t *bytes)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    void *p;
    size_t n;
    field_info(w, field, &p, &n);
    if (!p) {
        set_error("unknown field");
        return TECTO_ERR_INVALID;
    }
    if (device_ptr) *device_ptr = p;
    if (bytes) *bytes = n;
    return TECTO_OK;
}

int tecto_world_upload(tecto_world *w, int field, const void *host, size_t bytes, tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    void *p;
    size_t n;
    field_info(w, field, &p, &n);
    if (!p || !host || bytes != n) {
        set_error("tecto_world_upload: unknown field or size mismatch");
        return TECTO_ERR_INVALID;
    }
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    TECTO_CUDA(cudaMemcpyAsync(p, host, n, cudaMemcpyHostToDevice, st));
    TECTO_CUDA(cudaStreamSynchronize(st));
    return TECTO_OK;
}

int tecto_world_download(tecto_world *w, int field, void *host, size_t bytes, tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    void *p;
    size_t n;
    field_info(w, field, &p, &n);
    if (!p || !host || bytes != n) {
        set_error("tecto_world_download: unknown field or size mismatch");
        return TECTO_ERR_INVALID;
    }
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    TECTO_CUDA(cudaMemcpyAsync(host, p, n, cudaMemcpyDeviceToHost, st));
    TECTO_CUDA(cudaStreamSynchronize(st));
    return TECTO_OK;
}

int tecto_world_set_plates(tecto_world *w, const tecto_plate *plates, int count, tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if (!plates || count < 0 || count > kPlates) return TECTO_ERR_INVALID;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    TECTO_CUDA(cudaMemcpyAsync(w->b.plates, plates, sizeof(tecto_plate) * count, cudaMemcpyHostToDevice, st));
    TECTO_CUDA(cudaStreamSynchronize(st));
    return TECTO_OK;
}

int tecto_world_get_plates(tecto_world *w, tecto_plate *plates, int count, tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if (!plates || count < 0 || count > kPlates) return TECTO_ERR_INVALID;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    TECTO_CUDA(cudaMemcpyAsync(plates, w->b.plates, sizeof(tecto_plate) * count, cudaMemcpyDeviceToHost, st));
    TECTO_CUDA(cudaStreamSynchronize(st));
    return TECTO_OK;
}

int tecto_world_set_iteration(tecto_world *w, uint32_t iteration)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    TECTO_CUDA(cudaDeviceSynchronize());
    w->iteration = iteration;
    TECTO_CUDA(cudaMemcpy(&w->b.ctl->iteration, &iteration, 4, cudaMemcpyHostToDevice));
    return TECTO_OK;
}

int tecto_world_get_iteration(const tecto_world *w, uint32_t *iteration)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if (!iteration) return TECTO_ERR_INVALID;
    *iteration = w->iteration;
    return TECTO_OK;
}

int tecto_phase_collide(tecto_world *w, tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    return enqueue_collide(w, (cudaStream_t)stream);
}

int tecto_phase_resolve(tecto_world *w, tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    return launch_resolve(w, (cudaStream_t)stream);
}

int tecto_phase_thermal(tecto_world *w, int iterations, tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if (iterations < 0) return TECTO_ERR_INVALID;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    return launch_thermal(w, iterations, (cudaStream_t)stream);
}

int tecto_phase_hydraulic(tecto_world *w, int iterations, float dt, tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if (iterations < 0 || !std::isfinite(dt)) return TECTO_ERR_INVALID;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    return launch_hydraulic(w, iterations, dt, (cudaStream_t)stream);
}

int tecto_phase_finish(tecto_world *w, tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    return enqueue_finish(w, (cudaStream_t)stream, ccl_due(w));
}

int tecto_phase_ccl(tecto_world *w, int connectivity, tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    return launch_ccl(w, connectivity, (cudaStream_t)stream);
}

int tecto_world_step(tecto_world *w, int nSteps, tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if (nSteps < 0) return TECTO_ERR_INVALID;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    for (int s = 0; s < nSteps; ++s) {
        const bool ccl = ccl_due(w);
        if (st == nullptr) {  // the legacy stream cannot be captured: plain launches
            if ((rc = enqueue_step(w, st, ccl)) != TECTO_OK) return rc;
            continue;
        }
        const int key = w->cur_h | (w->cur_wsf << 1) | (w->cur_id << 2) | ((ccl ? 1 : 0) << 3);
        if (!w->graph_valid[key]) {
            cudaGraph_t g = nullptr;
            const uint64_t before = w->launches;
            TECTO_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            rc = enqueue_step(w, st, ccl);
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
            w->graphs[key] = ex;
            w->graph_valid[key] = true;
            w->graph_end[key][0] = w->cur_h;
            w->graph_end[key][1] = w->cur_wsf;
            w->graph_end[key][2] = w->cur_id;
            w->graph_end[key][3] = w->sort_final;
            w->graph_launches[key] = w->launches - before;
            TECTO_CUDA(cudaGraphLaunch(ex, st));
        } else {
            TECTO_CUDA(cudaGraphLaunch(w->graphs[key], st));
            w->cur_h = w->graph_end[key][0];
            w->cur_wsf = w->graph_end[key][1];
            w->cur_id = w->graph_end[key][2];
            w->sort_final = w->graph_end[key][3];
            w->iteration += 1;
            w->launches += w->graph_launches[key];
        }
    }
    return TECTO_OK;
}

int tecto_world_launch_count(const tecto_world *w, uint64_t *count)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if (!count) return TECTO_ERR_INVALID;
    *count = w->launches;
    return TECTO_OK;
}

int tecto_world_check(tecto_world *w, tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    TECTO_CUDA(cudaStreamSynchronize(st));
    TECTO_CUDA(cudaGetLastError());
    uint32_t err[2] = {0, 0};
    TECTO_CUDA(cudaMemcpy(&err[0], &w->b.ctl->error, 4, cudaMemcpyDeviceToHost));
    TECTO_CUDA(cudaMemcpy(&err[1], w->b.sort.error, 4, cudaMemcpyDeviceToHost));
    if (err[0] | err[1]) {
        cudaMemset(&w->b.ctl->error, 0, 4);
        cudaMemset(w->b.sort.error, 0, 4);
        set_error("a bounded device-side wait gave up");
        return TECTO_ERR_DEVICE_TIMEOUT;
    }
    return TECTO_OK;
}

}  // extern "C"
