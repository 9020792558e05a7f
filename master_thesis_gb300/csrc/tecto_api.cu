// tecto_api.cu - the C ABI for single worlds: lifecycle and HBM arena, synthetic world
// generator, field I/O, phase entry points and the step driver.  Replaces PlateTectonicSim
// (src/cuda_compute/plate_tectonic_sim.h:110-130, plate_tectonic_sim.cu:28-131) for the
// hot-path phases.  A world stepped on its own runs as a private batch of one (tecto_batch.cu).
#include <algorithm>
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
    size_t total = 0;
    size_t add(size_t bytes)
    {
        const size_t o = total;
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

int bind_device(const tecto_world *w)
{
    int cur = -1;
    TECTO_CUDA(cudaGetDevice(&cur));
    if (cur != w->device) TECTO_CUDA(cudaSetDevice(w->device));
    return TECTO_OK;
}

// The world's private batch of one, aligned with the world's current ping-pong halves.  Fails
// while the world belongs to a public batch (its state is then stepped by that batch).
int own_batch(tecto_world *w, Batch **out)
{
    if (w->in_batch && w->in_batch != w->own) {
        set_error("world belongs to a batch: step it through tecto_batch_step or remove it first");
        return TECTO_ERR_INVALID;
    }
    if (!w->own) {
        w->own = new (std::nothrow) Batch();
        if (!w->own) return TECTO_ERR_OOM;
        const int rc = batch_join(*w->own, w, nullptr);
        if (rc != TECTO_OK) return rc;
    }
    Batch &b = *w->own;
    if (std::memcmp(&b.settings, &w->settings, sizeof(tecto_settings)) != 0) {
        b.settings = w->settings;
        b.dirty = true;
    }
    b.cur_h = w->cur_h;
    b.cur_wsf = w->cur_wsf;
    b.cur_id = w->cur_id;
    w->in_batch = w->own;
    *out = w->own;
    return batch_prepare(b, nullptr);
}

void from_batch(tecto_world *w, const Batch &b)
{
    w->cur_h = b.cur_h;
    w->cur_wsf = b.cur_wsf;
    w->cur_id = b.cur_id;
}

void field_info(tecto_world *w, int field, void **ptr, size_t *bytes)
{
    const size_t N = w->N;
    const WorldDev &d = w->dev;
    *ptr = nullptr;
    *bytes = 0;
    switch (field) {
        case TECTO_FIELD_HEIGHT: *ptr = d.h[w->cur_h]; *bytes = N * 4; break;
        case TECTO_FIELD_WATER: *ptr = d.w[w->cur_wsf]; *bytes = N * 4; break;
        case TECTO_FIELD_SEDIMENT: *ptr = d.s[w->cur_wsf]; *bytes = N * 4; break;
        case TECTO_FIELD_FLUX: *ptr = d.flux[w->cur_wsf]; *bytes = N * 16; break;
        case TECTO_FIELD_PLATE_ID: *ptr = d.id[w->cur_id]; *bytes = N; break;
        case TECTO_FIELD_LABELS: *ptr = d.labels; *bytes = N * 4; break;
        case TECTO_FIELD_COLLISION: *ptr = d.word; *bytes = N * 4; break;
        case TECTO_FIELD_TYPE_BITMAP: *ptr = d.type_bitmap; *bytes = kPairs; break;
        case TECTO_FIELD_DIV_BITMAP: *ptr = d.div_bitmap; *bytes = kDivWords * 4; break;
        case TECTO_FIELD_SORT_KEYS:
            if (w->own && w->own->arena) { *ptr = w->own->keys[w->own->sort_final]; *bytes = N * 4; }
            break;
        case TECTO_FIELD_SORT_VALS:
            if (w->own && w->own->arena) { *ptr = w->own->vals[w->own->sort_final]; *bytes = N * 4; }
            break;
        case TECTO_FIELD_ACCRETION: *ptr = d.acc_u8; *bytes = N; break;
        case TECTO_FIELD_JFA_SEED:
            if (w->own && w->own->upref.arena) { *ptr = w->own->upref.jfa[w->own->upref_final]; *bytes = N * 4; }
            break;
        case TECTO_FIELD_JFA_DIST:
            if (w->own && w->own->upref.arena) { *ptr = w->own->upref.dist; *bytes = N * 4; }
            break;
        default: break;
    }
}

}  // namespace

void set_error(const std::string &msg) { g_last_error = msg; }

int cuda_fail(cudaError_t e, const char *what)
{
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? TECTO_ERR_OOM : TECTO_ERR_CUDA;
}

// Bytes of device memory one world of W x H cells holds (its arena, and its share of the
// batch-level buffers: sort keys/values, accretion list, sort status).
size_t world_footprint(int W, int H)
{
    const size_t N = (size_t)W * (size_t)H;
    Layout L;
    L.add(N * 4); L.add(N * 4); L.add(N * 4); L.add(N * 4); L.add(N * 4); L.add(N * 4);
    L.add(N * 16); L.add(N * 16); L.add(N); L.add(N);
    L.add(N * 4); L.add(N * 4); L.add(N * 4); L.add(N * 8); L.add(N * 4); L.add(N * 8); L.add(N * 4); L.add(N);
    L.add(kPairs); L.add(kDivWords * 4); L.add(kDivWords * 4); L.add(kPairs * sizeof(PairCounts));
    L.add(kPlates * sizeof(tecto_plate)); L.add(kPlates * sizeof(tecto_plate));
    L.add((kPlates + 1) * sizeof(int2)); L.add(kPlates * sizeof(tecto_plate_dynamics));
    L.add(kPlates * sizeof(PlateAcc)); L.add(sizeof(PolicyState)); L.add(sizeof(Control));
    // its share of a batch's sort: key/value ping-pong plus the scratch of the widest digit choice
    size_t scratch = 0;
    for (int rb = 8; rb <= kMaxRadixBits; ++rb)
        scratch = std::max(scratch, sort_scratch_bytes(N, key_bits_for(N), rb));
    return L.total + 4 * N * 4 + scratch;
}

}  // namespace tecto

using namespace tecto;

extern "C" {

const char *tecto_last_error_string(void) { return g_last_error.c_str(); }

const char *tecto_version(void) { return "tecto-gb300 0.2 (sm_103a)"; }

size_t tecto_world_bytes(int width, int height)
{
    if (width < 1 || height < 1) return 0;
    return world_footprint(width, height);
}

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
    Layout L;
    const size_t o_h0 = L.add(N * 4), o_h1 = L.add(N * 4);
    const size_t o_w0 = L.add(N * 4), o_w1 = L.add(N * 4);
    const size_t o_s0 = L.add(N * 4), o_s1 = L.add(N * 4);
    const size_t o_f0 = L.add(N * 16), o_f1 = L.add(N * 16);
    const size_t o_i0 = L.add(N), o_i1 = L.add(N);
    const size_t o_word = L.add(N * 4);
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
    const size_t o_plp = L.add(kPlates * sizeof(tecto_plate));
    const size_t o_off = L.add((kPlates + 1) * sizeof(int2));
    const size_t o_dyn = L.add(kPlates * sizeof(tecto_plate_dynamics));
    const size_t o_pacc = L.add(kPlates * sizeof(PlateAcc));
    const size_t o_pol = L.add(sizeof(PolicyState));
    const size_t o_ctl = L.add(sizeof(Control));
    cudaError_t e = cudaMalloc(&w->arena, L.total);
    if (e != cudaSuccess) {
        delete w;
        return cuda_fail(e, "cudaMalloc(world arena)");
    }
    w->arena_bytes = L.total;
    char *base = (char *)w->arena;
    WorldDev &d = w->dev;
    d.W = width;
    d.H = height;
    d.N = (uint32_t)N;
    d.vbase = 0;
    d.h[0] = (float *)(base + o_h0);
    d.h[1] = (float *)(base + o_h1);
    d.w[0] = (float *)(base + o_w0);
    d.w[1] = (float *)(base + o_w1);
    d.s[0] = (float *)(base + o_s0);
    d.s[1] = (float *)(base + o_s1);
    d.flux[0] = (float4 *)(base + o_f0);
    d.flux[1] = (float4 *)(base + o_f1);
    d.id[0] = (uint8_t *)(base + o_i0);
    d.id[1] = (uint8_t *)(base + o_i1);
    d.word = (uint32_t *)(base + o_word);
    d.labels = (uint32_t *)(base + o_lab);
    d.rain = (float *)(base + o_rain);
    d.vel = (float2 *)(base + o_vel);
    d.s1 = (float *)(base + o_s1b);
    d.acc = (unsigned long long *)(base + o_acc);
    d.acc_list = (uint32_t *)(base + o_accl);
    d.acc_u8 = (uint8_t *)(base + o_accu);
    d.type_bitmap = (uint8_t *)(base + o_bm);
    d.div_bitmap = (uint32_t *)(base + o_div);
    d.has_div = (uint32_t *)(base + o_hd);
    d.counts = (PairCounts *)(base + o_cnt);
    d.plates = (tecto_plate *)(base + o_pl);
    d.plates_prev = (tecto_plate *)(base + o_plp);
    d.off = (int2 *)(base + o_off);
    d.dyn = (tecto_plate_dynamics *)(base + o_dyn);
    d.pacc = (PlateAcc *)(base + o_pacc);
    d.policy = (PolicyState *)(base + o_pol);
    d.pressure = nullptr;
    d.pw = d.ph = 0;
    d.ctl = (Control *)(base + o_ctl);
    e = cudaMemset(w->arena, 0, L.total);
    if (e == cudaSuccess) {
        Control c{};
        c.seed = seed;
        e = cudaMemcpy(d.ctl, &c, sizeof(c), cudaMemcpyHostToDevice);
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
    if (w->in_batch && w->in_batch != w->own) batch_leave(*w->in_batch, w);
    if (w->own) {
        batch_release(*w->own);
        delete w->own;
        w->own = nullptr;
    }
    if (w->arena) cudaFree(w->arena);
    w->arena = nullptr;
    if (w->pressure) cudaFree(w->pressure);
    w->pressure = nullptr;
    delete w;
    return TECTO_OK;
}

int tecto_world_set_settings(tecto_world *w, const tecto_settings *s)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if (!s) return TECTO_ERR_INVALID;
    if (w->in_batch && w->in_batch != w->own) {
        set_error("world belongs to a batch: remove it before changing its settings");
        return TECTO_ERR_INVALID;
    }
    w->settings = *s;
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

}  // extern "C"

namespace tecto {
namespace gen {

// Seed points and plate kinematics of the synthetic generator (host, cheap: P <= 255).
void gen_seeds(int W, int H, int P, float velRange, uint64_t genSeed, std::vector<float> &sx,
               std::vector<float> &sy, std::vector<tecto_plate> &pl)
{
    uint64_t st = genSeed;
    sx.assign(P, 0.0f);
    sy.assign(P, 0.0f);
    pl.assign(kPlates, tecto_plate{});
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
}

__device__ __forceinline__ uint64_t splitmix64_d(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Per-cell part of the generator on the GPU, operation for operation the host loop below.
__global__ void k_generate(float *h, uint8_t *id, int W, int H, int P, const float *sx, const float *sy,
                           uint64_t genSeed)
{
    __shared__ float s_x[kPlates], s_y[kPlates];
    for (int k = threadIdx.x; k < P; k += blockDim.x) {
        s_x[k] = sx[k];
        s_y[k] = sy[k];
    }
    __syncthreads();
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)W * (size_t)H) return;
    const int y = (int)(i / (size_t)W), x = (int)(i - (size_t)y * W);
    const float fW = (float)W, fH = (float)H;
    float best = 3.4e38f;
    int bid = 0;
    for (int k = 0; k < P; ++k) {
        const float dx = fabsf((float)x - s_x[k]), dy = fabsf((float)y - s_y[k]);
        const float wx = fminf(dx, fW - dx), wy = fminf(dy, fH - dy);
        const float d2 = wx * wx + wy * wy;
        if (d2 < best) {
            best = d2;
            bid = k;
        }
    }
    id[i] = (uint8_t)bid;
    uint64_t cs = genSeed ^ (0xD1B54A32D192ED03ull * (uint64_t)(i + 1));
    float sum = 0.0f;
    for (int r = 0; r < 12; ++r) sum = sum + (float)(splitmix64_d(cs) >> 40) * (1.0f / 16777216.0f);
    const float n = sum - 6.0f;
    h[i] = (bid % 2 == 0) ? 0.5f + 0.05f * n : -0.5f + 0.02f * n;
}

}  // namespace gen
}  // namespace tecto

using namespace tecto::gen;

extern "C" {

int tecto_world_init_synthetic_device(tecto_world *w, int P, float velRange, uint64_t genSeed,
                                      tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if (P < 1 || P > kPlates) {
        set_error("tecto_world_init_synthetic_device: plate count must be 1..255");
        return TECTO_ERR_INVALID;
    }
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    std::vector<float> sx, sy;
    std::vector<tecto_plate> pl;
    gen_seeds(w->W, w->H, P, velRange, genSeed, sx, sy, pl);
    cudaStream_t st = (cudaStream_t)stream;
    const WorldDev &d = w->dev;
    w->iteration = 0;
    TECTO_CUDA(cudaMemsetAsync(w->arena, 0, w->arena_bytes, st));
    // the seed coordinates ride in the (just cleared) split-path scratch until the kernel ran
    float *dsx = d.s1, *dsy = d.s1 + kPlates;
    TECTO_CUDA(cudaMemcpyAsync(dsx, sx.data(), P * sizeof(float), cudaMemcpyHostToDevice, st));
    TECTO_CUDA(cudaMemcpyAsync(dsy, sy.data(), P * sizeof(float), cudaMemcpyHostToDevice, st));
    TECTO_CUDA(cudaMemcpyAsync(d.plates, pl.data(), sizeof(tecto_plate) * kPlates, cudaMemcpyHostToDevice, st));
    TECTO_CUDA(cudaMemsetAsync(d.dyn, 0, sizeof(tecto_plate_dynamics) * kPlates, st));  // fresh PlateData
    TECTO_CUDA(cudaMemsetAsync(d.pacc, 0, sizeof(PlateAcc) * kPlates, st));
    Control c{};
    c.seed = w->seed;
    TECTO_CUDA(cudaMemcpyAsync(d.ctl, &c, sizeof(c), cudaMemcpyHostToDevice, st));
    if (w->N < 2 * (size_t)kPlates) {  // too small to borrow the scratch: generate on the host
        TECTO_CUDA(cudaStreamSynchronize(st));
        return tecto_world_init_synthetic(w, P, velRange, genSeed, stream);
    }
    k_generate<<<(unsigned)((w->N + 255) / 256), 256, 0, st>>>(d.h[w->cur_h], d.id[w->cur_id], w->W, w->H, P,
                                                             dsx, dsy, genSeed);
    TECTO_CUDA(cudaGetLastError());
    TECTO_CUDA(cudaMemsetAsync(d.s1, 0, 2 * kPlates * sizeof(float), st));
    TECTO_CUDA(cudaStreamSynchronize(st));
    return TECTO_OK;
}

int tecto_generate_world_host(int W, int H, int P, float velRange, uint64_t genSeed, float *height_out,
                              uint8_t *id_out, tecto_plate *plates_out)
{
    if (W < 1 || H < 1 || P < 1 || P > kPlates) {
        set_error("tecto_generate_world_host: invalid size or plate count (1..255)");
        return TECTO_ERR_INVALID;
    }
    std::vector<float> sx, sy;
    std::vector<tecto_plate> pl;
    gen_seeds(W, H, P, velRange, genSeed, sx, sy, pl);
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
    const size_t N = w->N;
    const WorldDev &d = w->dev;
    w->iteration = 0;
    TECTO_CUDA(cudaMemsetAsync(w->arena, 0, w->arena_bytes, st));
    TECTO_CUDA(cudaMemcpyAsync(d.h[w->cur_h], h.data(), N * 4, cudaMemcpyHostToDevice, st));
    TECTO_CUDA(cudaMemcpyAsync(d.id[w->cur_id], id.data(), N, cudaMemcpyHostToDevice, st));
    TECTO_CUDA(cudaMemcpyAsync(d.plates, pl.data(), sizeof(tecto_plate) * kPlates, cudaMemcpyHostToDevice, st));
    TECTO_CUDA(cudaMemsetAsync(d.dyn, 0, sizeof(tecto_plate_dynamics) * kPlates, st));  // fresh PlateData
    TECTO_CUDA(cudaMemsetAsync(d.pacc, 0, sizeof(PlateAcc) * kPlates, st));
    Control c{};
    c.seed = w->seed;
    TECTO_CUDA(cudaMemcpyAsync(d.ctl, &c, sizeof(c), cudaMemcpyHostToDevice, st));
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
        set_error("unknown field (or sort output of a world never stepped alone)");
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

// Stream-ordered copies with no synchronisation: the caller keeps the host buffer alive (and, for
// a download, unread) until the stream has reached this point.
static int copy_field_async(tecto_world *w, int field, void *host, size_t bytes, cudaStream_t st, bool up,
                            const char *who)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    void *p;
    size_t n;
    field_info(w, field, &p, &n);
    if (!p || !host || bytes != n) {
        set_error(std::string(who) + ": unknown field or size mismatch");
        return TECTO_ERR_INVALID;
    }
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    if (up) TECTO_CUDA(cudaMemcpyAsync(p, host, n, cudaMemcpyHostToDevice, st));
    else TECTO_CUDA(cudaMemcpyAsync(host, p, n, cudaMemcpyDeviceToHost, st));
    return TECTO_OK;
}

int tecto_world_upload_async(tecto_world *w, int field, const void *host, size_t bytes, tecto_stream_t stream)
{
    return copy_field_async(w, field, const_cast<void *>(host), bytes, (cudaStream_t)stream, true,
                            "tecto_world_upload_async");
}

int tecto_world_download_async(tecto_world *w, int field, void *host, size_t bytes, tecto_stream_t stream)
{
    return copy_field_async(w, field, host, bytes, (cudaStream_t)stream, false, "tecto_world_download_async");
}

int tecto_world_set_plates(tecto_world *w, const tecto_plate *plates, int count, tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if (!plates || count < 0 || count > kPlates) return TECTO_ERR_INVALID;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    TECTO_CUDA(cudaMemcpyAsync(w->dev.plates, plates, sizeof(tecto_plate) * count, cudaMemcpyHostToDevice, st));
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
    TECTO_CUDA(cudaMemcpyAsync(plates, w->dev.plates, sizeof(tecto_plate) * count, cudaMemcpyDeviceToHost, st));
    TECTO_CUDA(cudaStreamSynchronize(st));
    return TECTO_OK;
}

int tecto_world_set_plate_dynamics(tecto_world *w, const tecto_plate_dynamics *plates, int count,
                                   tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if (!plates || count < 0 || count > kPlates) return TECTO_ERR_INVALID;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    TECTO_CUDA(cudaMemcpyAsync(w->dev.dyn, plates, sizeof(tecto_plate_dynamics) * count, cudaMemcpyHostToDevice, st));
    TECTO_CUDA(cudaStreamSynchronize(st));
    return TECTO_OK;
}

int tecto_world_get_plate_dynamics(tecto_world *w, tecto_plate_dynamics *plates, int count, tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if (!plates || count < 0 || count > kPlates) return TECTO_ERR_INVALID;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    TECTO_CUDA(cudaMemcpyAsync(plates, w->dev.dyn, sizeof(tecto_plate_dynamics) * count, cudaMemcpyDeviceToHost, st));
    TECTO_CUDA(cudaStreamSynchronize(st));
    return TECTO_OK;
}

int tecto_world_set_asthenosphere(tecto_world *w, const float *pressure, int pw, int ph, tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if (pressure && (pw < 1 || ph < 1 || (size_t)pw * (size_t)ph > ((size_t)1 << 30))) {
        set_error("tecto_world_set_asthenosphere: invalid texture size");
        return TECTO_ERR_INVALID;
    }
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    TECTO_CUDA(cudaStreamSynchronize(st));  // no step in flight reads the old texture
    TECTO_CUDA(cudaDeviceSynchronize());
    if (w->pressure) cudaFree(w->pressure);
    w->pressure = nullptr;
    w->pw = w->ph = 0;
    if (pressure) {
        const size_t bytes = (size_t)pw * (size_t)ph * 4;
        TECTO_CUDA(cudaMalloc(&w->pressure, bytes));
        w->pw = pw;
        w->ph = ph;
        TECTO_CUDA(cudaMemcpy(w->pressure, pressure, bytes, cudaMemcpyHostToDevice));
    }
    w->dev.pressure = w->pressure;
    w->dev.pw = w->pw;
    w->dev.ph = w->ph;
    if (w->in_batch) w->in_batch->dirty = true;  // the batch's device table holds the pointer
    return TECTO_OK;
}

int tecto_world_set_iteration(tecto_world *w, uint32_t iteration)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    TECTO_CUDA(cudaDeviceSynchronize());
    w->iteration = iteration;
    TECTO_CUDA(cudaMemcpy(&w->dev.ctl->iteration, &iteration, 4, cudaMemcpyHostToDevice));
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

// Phase entry points: each enqueues one phase of the world's own batch of one.
#define TECTO_PHASE_PROLOGUE                               \
    int rc = check_world(w);                               \
    if (rc != TECTO_OK) return rc;                         \
    if ((rc = bind_device(w)) != TECTO_OK) return rc;      \
    Batch *b = nullptr;                                    \
    if ((rc = own_batch(w, &b)) != TECTO_OK) return rc;    \
    cudaStream_t st = (cudaStream_t)stream;                \
    const uint64_t before = b->launches;

#define TECTO_PHASE_EPILOGUE           \
    from_batch(w, *b);                 \
    w->launches += b->launches - before; \
    return rc;

int tecto_world_autotune(tecto_world *w, tecto_stream_t stream, tecto_tuning *out)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    Batch *b = nullptr;
    if ((rc = own_batch(w, &b)) != TECTO_OK) return rc;
    return tune_batch(*b, (cudaStream_t)stream, out);
}

int tecto_phase_collide(tecto_world *w, tecto_stream_t stream)
{
    TECTO_PHASE_PROLOGUE
    if ((rc = launch_plates(*b, st)) == TECTO_OK && (rc = launch_sort_keys(*b, st)) == TECTO_OK &&
        (rc = launch_words(*b, st)) == TECTO_OK)
        rc = launch_type_matrix(*b, st);
    TECTO_PHASE_EPILOGUE
}

int tecto_phase_resolve(tecto_world *w, tecto_stream_t stream)
{
    TECTO_PHASE_PROLOGUE
    rc = launch_resolve(*b, st);
    if (rc == TECTO_OK && b->settings.step.upliftMode == TECTO_UPLIFT_REFERENCE) rc = launch_uplift_ref(*b, st);
    TECTO_PHASE_EPILOGUE
}

int tecto_phase_thermal(tecto_world *w, int iterations, tecto_stream_t stream)
{
    if (iterations < 0) return TECTO_ERR_INVALID;
    TECTO_PHASE_PROLOGUE
    rc = launch_thermal(*b, iterations, st);
    TECTO_PHASE_EPILOGUE
}

int tecto_phase_hydraulic(tecto_world *w, int iterations, float dt, tecto_stream_t stream)
{
    if (iterations < 0 || !std::isfinite(dt)) return TECTO_ERR_INVALID;
    TECTO_PHASE_PROLOGUE
    rc = launch_hydraulic(*b, iterations, dt, st);
    TECTO_PHASE_EPILOGUE
}

int tecto_phase_finish(tecto_world *w, tecto_stream_t stream)
{
    TECTO_PHASE_PROLOGUE
    const int period = w->settings.sim.iterationsForCCL > 0 ? w->settings.sim.iterationsForCCL : 1;
    const bool due = w->iteration % (uint32_t)period == 0;
    if ((rc = launch_finish(*b, st)) == TECTO_OK &&
        (!due || (rc = launch_ccl(*b, w->settings.step.cclConnectivity, false, st)) == TECTO_OK) &&
        (!w->settings.step.platePolicy || (rc = launch_plate_policy(*b, due ? 1 : 0, st)) == TECTO_OK) &&
        (rc = launch_bump_iteration(*b, st)) == TECTO_OK)
        w->iteration += 1;
    TECTO_PHASE_EPILOGUE
}

int tecto_phase_ccl(tecto_world *w, int connectivity, tecto_stream_t stream)
{
    TECTO_PHASE_PROLOGUE
    rc = launch_ccl(*b, connectivity, false, st);
    TECTO_PHASE_EPILOGUE
}

int tecto_world_step(tecto_world *w, int nSteps, tecto_stream_t stream)
{
    int rc = check_world(w);
    if (rc != TECTO_OK) return rc;
    if (nSteps < 0) return TECTO_ERR_INVALID;
    if ((rc = bind_device(w)) != TECTO_OK) return rc;
    Batch *b = nullptr;
    if ((rc = own_batch(w, &b)) != TECTO_OK) return rc;
    return batch_step(*b, nSteps, (cudaStream_t)stream);  // updates the world's halves and counters
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
    TECTO_CUDA(cudaMemcpy(&err[0], &w->dev.ctl->error, 4, cudaMemcpyDeviceToHost));
    if (w->own && w->own->arena && w->own->sort.error)
        TECTO_CUDA(cudaMemcpy(&err[1], w->own->sort.error, 4, cudaMemcpyDeviceToHost));
    if (err[0] | err[1]) {
        cudaMemset(&w->dev.ctl->error, 0, 4);
        if (w->own && w->own->sort.error) cudaMemset(w->own->sort.error, 0, 4);
        if ((err[0] & kErrUpliftCapacity) && !((err[0] & ~kErrUpliftCapacity) | err[1])) {
            set_error("reference uplift: more propagation events than its scratch holds");
            return TECTO_ERR_UNSUPPORTED;
        }
        set_error("a bounded device-side wait gave up");
        return TECTO_ERR_DEVICE_TIMEOUT;
    }
    return TECTO_OK;
}

}  // extern "C"
