// tecto_tune.cu - the autotuner: picks the hydraulic and thermal tile variants and the collision
// sort's digit width for a batch by timing each candidate on the device.
//
// The reference has one fixed launch shape per kernel (src/cuda_compute/plate_tectonic_sim.cu);
// this engine runs worlds of any size in batches, where the best tile (halo overhead against
// occupancy and barrier cost) and the best digit width (sort passes against per-tile histogram
// and look-back cost) depend on the sizes.  Tuning never touches the caller's worlds: it builds scratch
// worlds of the same shapes with synthetic content, times the candidates, and frees them.
// Choices are cached per device and batch shape class (total cells, mean world size, both in
// half-octave steps); a batch whose settings leave hydraulicTile / thermalTile / sortRadixBits at
// 0 uses the choice of its class, else of the nearest tuned class on its device.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <new>
#include <tuple>
#include <vector>

#include "tecto_internal.cuh"

namespace tecto {

namespace {

struct TuneChoice {
    int hydro;
    int rb;
    int thermal;
};

using ClassKey = std::tuple<int, int, int>;  // device, total-cells class, mean-world-cells class

std::mutex g_tune_mu;
std::map<ClassKey, TuneChoice> g_tune;

int size_class(double cells) { return (int)std::lround(2.0 * std::log2(std::max(cells, 1.0))); }

ClassKey class_of(int device, size_t total, size_t worlds)
{
    const double t = (double)total, m = (double)total / (double)std::max<size_t>(worlds, 1);
    return ClassKey(device, size_class(t), size_class(m));
}

// Time `fn` (enqueues work on st): one warm-up call, then the best of `reps` timed calls.
template <typename F>
int time_best(cudaStream_t st, int reps, float *best_ms, F &&fn)
{
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    TECTO_CUDA(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return cuda_fail(cudaErrorUnknown, "cudaEventCreate");
    }
    int rc = fn();
    float best = INFINITY;
    for (int r = 0; rc == TECTO_OK && r < reps; ++r) {
        cudaEventRecord(e0, st);
        rc = fn();
        cudaEventRecord(e1, st);
        if (rc != TECTO_OK) break;
        const cudaError_t ce = cudaEventSynchronize(e1);
        if (ce != cudaSuccess) {
            rc = cuda_fail(ce, "cudaEventSynchronize");
            break;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        best = std::min(best, ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *best_ms = best;
    return rc;
}

int tune_shapes(const tecto_settings &settings, const std::vector<int2> &shapes, cudaStream_t st,
                tecto_tuning *out)
{
    if (shapes.empty() || (int)shapes.size() > kMaxBatchWorlds) {
        set_error("tecto_autotune: 1 to 1024 worlds");
        return TECTO_ERR_INVALID;
    }
    std::vector<tecto_world *> worlds;
    Batch tb;
    int rc = TECTO_OK;
    tecto_tuning res{};
    size_t total = 0;
    for (size_t i = 0; i < shapes.size() && rc == TECTO_OK; ++i) {
        tecto_world *w = nullptr;
        rc = tecto_world_create(&settings, shapes[i].x, shapes[i].y, 7000u + (uint32_t)i, &w);
        if (rc != TECTO_OK) break;
        worlds.push_back(w);
        total += w->N;
        rc = tecto_world_init_synthetic_device(w, 16, 1.0f, 9000u + (uint64_t)i, (tecto_stream_t)st);
        if (rc == TECTO_OK) rc = batch_join(tb, w, st);
    }
    const float dt = settings.step.hydraulicDt;
    if (rc == TECTO_OK) {
        tb.settings.step.hydraulicTile = kDefaultHydroVariant;
        tb.settings.step.thermalTile = kDefaultThermalVariant;
        tb.settings.step.sortRadixBits = kDefaultRadixBits;
        tb.dirty = true;
        rc = batch_step_graph(tb, 1, st, false);  // plate offsets and a settled state to time on
    }
    // hydraulic tile variants: one sub-iteration each, best of a few
    int best_v = kDefaultHydroVariant;
    float best_vms = INFINITY;
    for (int v = 1; v <= kHydroVariantCount && rc == TECTO_OK; ++v) {
        tb.settings.step.hydraulicTile = v;
        if ((rc = batch_prepare(tb, st)) != TECTO_OK) break;
        float ms = 0;
        rc = time_best(st, 3, &ms, [&]() { return launch_hydraulic(tb, 2, dt, st); });
        ms *= 0.5f;
        res.hydraulic_ms[v - 1] = ms;
        if (rc == TECTO_OK && ms < best_vms) {
            best_vms = ms;
            best_v = v;
        }
    }
    tb.settings.step.hydraulicTile = best_v;
    // thermal tile variants: ten iterations each
    int best_t = kDefaultThermalVariant;
    float best_tms = INFINITY;
    for (int v = 1; v <= kThermalVariantCount && rc == TECTO_OK; ++v) {
        tb.settings.step.thermalTile = v;
        if ((rc = batch_prepare(tb, st)) != TECTO_OK) break;
        float ms = 0;
        rc = time_best(st, 3, &ms, [&]() { return launch_thermal(tb, 10, st); });
        res.thermal_ms[v - 1] = ms;
        if (rc == TECTO_OK && ms < best_tms) {
            best_tms = ms;
            best_t = v;
        }
    }
    tb.settings.step.thermalTile = best_t;
    // sort digit widths: the key-generating collision sort of the batch
    int best_rb = kDefaultRadixBits;
    float best_sms = INFINITY;
    for (int rb = 8; rb <= kMaxRadixBits && rc == TECTO_OK; ++rb) {
        tb.settings.step.sortRadixBits = rb;
        if ((rc = batch_prepare(tb, st)) != TECTO_OK) break;
        float ms = 0;
        rc = time_best(st, 3, &ms, [&]() { return launch_sort_keys(tb, st); });
        res.sort_ms[rb - 8] = ms;
        if (rc == TECTO_OK && ms < best_sms) {
            best_sms = ms;
            best_rb = rb;
        }
    }
    if (rc == TECTO_OK && tb.sort.error) {
        uint32_t e = 0;
        const cudaError_t ce = cudaMemcpy(&e, tb.sort.error, 4, cudaMemcpyDeviceToHost);
        if (ce != cudaSuccess) rc = cuda_fail(ce, "cudaMemcpy");
        else if (e) {
            set_error("tecto_autotune: a bounded device-side wait gave up");
            rc = TECTO_ERR_DEVICE_TIMEOUT;
        }
    }
    batch_release(tb);
    for (tecto_world *w : worlds) tecto_world_destroy(w);
    if (rc != TECTO_OK) return rc;
    res.hydraulicTile = best_v;
    res.sortRadixBits = best_rb;
    res.thermalTile = best_t;
    int dev = 0;
    cudaGetDevice(&dev);
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune[class_of(dev, total, shapes.size())] = TuneChoice{best_v, best_rb, best_t};
    }
    if (out) *out = res;
    return TECTO_OK;
}

}  // namespace

bool tune_lookup(int device, size_t total, size_t worlds, int *hydro, int *rb, int *thermal)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    const ClassKey k = class_of(device, total, worlds);
    auto it = g_tune.find(k);
    if (it == g_tune.end()) {  // nearest tuned class on the same device
        int best = -1;
        for (auto jt = g_tune.begin(); jt != g_tune.end(); ++jt) {
            if (std::get<0>(jt->first) != device) continue;
            const int d = std::abs(std::get<1>(jt->first) - std::get<1>(k)) +
                          std::abs(std::get<2>(jt->first) - std::get<2>(k));
            if (best < 0 || d < best) {
                best = d;
                it = jt;
            }
        }
        if (best < 0) return false;
    }
    *hydro = it->second.hydro;
    *rb = it->second.rb;
    *thermal = it->second.thermal;
    return true;
}

int tune_batch(Batch &b, cudaStream_t st, tecto_tuning *out)
{
    if (b.members.empty()) {
        set_error("tecto_batch_autotune: batch has no worlds");
        return TECTO_ERR_INVALID;
    }
    std::vector<int2> shapes;
    for (const tecto_world *w : b.members) shapes.push_back(make_int2(w->W, w->H));
    tecto_tuning t{};
    const int rc = tune_shapes(b.settings, shapes, st, &t);
    if (rc != TECTO_OK) return rc;
    b.tuned_hydro = t.hydraulicTile;
    b.tuned_rb = t.sortRadixBits;
    b.tuned_thermal = t.thermalTile;
    b.dirty = true;
    if (out) *out = t;
    return TECTO_OK;
}

}  // namespace tecto

using namespace tecto;

extern "C" {

int tecto_autotune(const tecto_settings *settings, const int *widths, const int *heights, int count,
                   tecto_stream_t stream, tecto_tuning *out)
{
    if (!settings || !widths || !heights || count < 1 || count > kMaxBatchWorlds) {
        set_error("tecto_autotune: invalid argument");
        return TECTO_ERR_INVALID;
    }
    std::vector<int2> shapes;
    for (int i = 0; i < count; ++i) {
        if (widths[i] < 1 || heights[i] < 1) {
            set_error("tecto_autotune: invalid world size");
            return TECTO_ERR_INVALID;
        }
        shapes.push_back(make_int2(widths[i], heights[i]));
    }
    return tune_shapes(*settings, shapes, (cudaStream_t)stream, out);
}

int tecto_batch_autotune(tecto_batch *batch, tecto_stream_t stream, tecto_tuning *out)
{
    if (!batch) return TECTO_ERR_INVALID;
    return tune_batch(batch->b, (cudaStream_t)stream, out);
}

int tecto_autotune_record(int device, size_t total_cells, int worlds, int hydraulicTile, int sortRadixBits,
                          int thermalTile)
{
    if (device < 0 || total_cells == 0 || worlds < 1 || hydraulicTile < 1 ||
        hydraulicTile > kHydroVariantCount || !valid_radix_bits(sortRadixBits) || thermalTile < 1 ||
        thermalTile > kThermalVariantCount)
        return TECTO_ERR_INVALID;
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune[class_of(device, total_cells, (size_t)worlds)] = TuneChoice{hydraulicTile, sortRadixBits, thermalTile};
    return TECTO_OK;
}

int tecto_autotune_lookup(int device, size_t total_cells, int worlds, int *hydraulicTile, int *sortRadixBits,
                          int *thermalTile)
{
    if (!hydraulicTile || !sortRadixBits || !thermalTile || worlds < 1) return TECTO_ERR_INVALID;
    if (!tune_lookup(device, total_cells, (size_t)worlds, hydraulicTile, sortRadixBits, thermalTile)) {
        *hydraulicTile = 0;
        *sortRadixBits = 0;
        *thermalTile = 0;
        return TECTO_ERR_NOT_FOUND;
    }
    return TECTO_OK;
}

int tecto_autotune_clear(void)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune.clear();
    return TECTO_OK;
}

}  // extern "C"
