// tecto_server.cu - continuous batching of world-generation requests (host runtime).
//
// The reference runs one interactive world (PlateTectonicSim driven by the GUI loop,
// src/main.cpp:122-161); serving many worlds is this engine's own layer.  Every tick advances all
// admitted worlds one step as one batch (one launch per phase); waiting requests are admitted
// first-come first-served whenever their footprint fits the HBM budget; finished worlds leave the
// batch at once so that newcomers join while others are mid-flight.  World state stays resident
// in HBM from admission to completion.
//
// Size-aware admission: a world of at least `heavy_cells` cells (2^20 by default) already runs near
// the GPU's full rate on its own, so sharing ticks with another such world only slows both, while
// smaller worlds gain from riding along in a batch.  At most `heavy_slots` (1) heavy requests are
// live at a time, admitted first-come first-served among themselves; light requests are admitted
// past a heavy one that waits for its slot (never past one that waits for budget).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <deque>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "tecto_internal.cuh"

namespace tecto {
size_t world_footprint(int W, int H);
int batch_step_graph(Batch &b, int nsteps, cudaStream_t st, bool use_graph);
}  // namespace tecto

using namespace tecto;

namespace {

using Clock = std::chrono::steady_clock;

struct Live {
    int idx;
    tecto_world *world;
    size_t bytes;
    size_t cells;
    int steps_left;
};

// Continuous-batching state, shared by a trace replay and the live API: the requests waiting for
// admission (first come first served), the admitted worlds and the bytes they hold.
struct Serving {
    std::deque<int> waiting;
    std::vector<Live> live;
    size_t used = 0;
    double peak = 0;
    int ticks = 0, max_active = 0, done = 0;
    bool changed = true;  // membership changed since the last tick
};

// Seconds since `t0`, or the simulated clock of a dry run (advanced by the cost model).
struct ServeClock {
    bool dry = false;
    double v = 0;
    Clock::time_point t0 = Clock::now();
    double now() const { return dry ? v : std::chrono::duration<double>(Clock::now() - t0).count(); }
};

}  // namespace

struct tecto_server {
    tecto_settings settings{};
    size_t budget = 0;
    int max_worlds = 0;
    bool dry = false;
    double dry_cost = 2e-4;  // seconds per tick per million active cells
    size_t heavy_cells = (size_t)1 << 20;  // tecto_server_set_policy
    int heavy_slots = 1;                    // 0: no limit (every request joins once it fits)
    tecto_batch *batch = nullptr;
    std::string out_dir;     // where finished requests are written (tecto_server_set_output)
    int out_what = 0;        // TECTO_SERVER_OUT_* bits
    int init_mode = TECTO_SERVER_INIT_SYNTHETIC;
    float out_lo = 0.0f, out_hi = 1.0f;  // height range of the 16-bit export
    // live API (tecto_server_submit / tick / poll): requests and results by ticket
    Serving q;
    ServeClock clock;
    std::vector<tecto_request> reqs;
    std::vector<tecto_request_result> results;
};

namespace {

double percentile(std::vector<double> v, double q)
{
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = q * (double)(v.size() - 1);
    const size_t lo = (size_t)std::floor(pos), hi = (size_t)std::ceil(pos);
    return v[lo] + (v[hi] - v[lo]) * (pos - (double)lo);
}

void finish_stats(const tecto_request *req, int n, const tecto_request_result *res, double wall,
                  int ticks, int max_active, double peak, tecto_server_stats *stats)
{
    if (!stats) return;
    std::vector<double> lat;
    tecto_server_stats s{};
    for (int i = 0; i < n; ++i) {
        if (res[i].status == TECTO_OK && res[i].finish_s >= 0) {
            ++s.completed;
            lat.push_back(res[i].finish_s - res[i].arrival_s);
            s.cell_updates += (double)req[i].width * (double)req[i].height * (double)req[i].steps;
        } else if (res[i].status == TECTO_ERR_BUDGET) {
            ++s.rejected;
        }
    }
    s.wall_s = wall;
    s.ticks = ticks;
    s.max_active = max_active;
    s.peak_bytes = peak;
    s.cell_updates_per_s = wall > 0 ? s.cell_updates / wall : 0.0;
    s.latency_p50_s = percentile(lat, 0.50);
    s.latency_p99_s = percentile(lat, 0.99);
    double sum = 0;
    for (double x : lat) sum += x;
    s.latency_mean_s = lat.empty() ? 0.0 : sum / (double)lat.size();
    *stats = s;
}

int make_world(tecto_server *sv, const tecto_request &r, cudaStream_t st, tecto_world **out)
{
    tecto_settings ws = sv->settings;
    if (sv->init_mode == TECTO_SERVER_INIT_REFERENCE) ws.sim.numStartingPlates = r.plates;
    int rc = tecto_world_create(&ws, r.width, r.height, r.worldSeed, out);
    if (rc != TECTO_OK) return rc;
    if (sv->init_mode == TECTO_SERVER_INIT_REFERENCE)
        rc = tecto_world_init_reference(*out, (tecto_stream_t)st);
    else
        rc = tecto_world_init_synthetic_device(*out, r.plates, r.velRange, r.genSeed, (tecto_stream_t)st);
    if (rc != TECTO_OK) {
        tecto_world_destroy(*out);
        *out = nullptr;
    }
    return rc;
}

float checksum(tecto_world *w, cudaStream_t st)
{
    std::vector<float> h(w->N);
    if (tecto_world_download(w, TECTO_FIELD_HEIGHT, h.data(), h.size() * 4, (tecto_stream_t)st) != TECTO_OK)
        return NAN;
    double s = 0;
    for (float v : h) s += v;
    return (float)s;
}

// The outputs a finished request asked for, named by its index in the trace.
int write_outputs(const tecto_server *sv, tecto_world *w, int idx, cudaStream_t st)
{
    const std::string base = sv->out_dir + "/request_" + std::to_string(idx);
    int rc = TECTO_OK;
    if (sv->out_what & TECTO_SERVER_OUT_HEIGHT_PNG)
        rc = tecto_world_export_png(w, TECTO_EXPORT_HEIGHT_GRAY16, (base + "_height.png").c_str(), sv->out_lo,
                                    sv->out_hi, (tecto_stream_t)st);
    if (rc == TECTO_OK && (sv->out_what & TECTO_SERVER_OUT_PLATES_PNG))
        rc = tecto_world_export_png(w, TECTO_EXPORT_PLATES_RGB, (base + "_plates.png").c_str(), 0.0f, 0.0f,
                                    (tecto_stream_t)st);
    if (rc == TECTO_OK && (sv->out_what & TECTO_SERVER_OUT_SNAPSHOT))
        rc = tecto_world_save_snapshot(w, (base + ".snap").c_str(), (tecto_stream_t)st);
    return rc;
}

// A finished request's result: its checksum and the outputs it asked for (a failed write marks the
// request failed; serving goes on).
void finish_world(const tecto_server *sv, tecto_world *w, int idx, cudaStream_t st, tecto_request_result &res)
{
    const int ok = tecto_world_check(w, (tecto_stream_t)st);  // a device-side wait that gave up fails the request
    if (ok != TECTO_OK) {
        res.status = ok;
        return;
    }
    res.height_checksum = checksum(w, st);
    if (sv->out_what) {
        const int rc = write_outputs(sv, w, idx, st);
        if (rc != TECTO_OK) res.status = rc;
    }
}

bool valid_request(const tecto_request &r)
{
    return r.width >= 1 && r.height >= 1 && r.plates >= 1 && r.plates <= kPlates && r.steps >= 0 &&
           (size_t)r.width * (size_t)r.height <= ((size_t)1 << 30);
}

// Whether a waiting request can never be served (invalid, or larger than the whole budget): its
// status is set and it leaves the queue.
bool reject(const tecto_server *sv, Serving &q, std::deque<int>::iterator &it, const tecto_request *req,
            tecto_request_result *res)
{
    const int i = *it;
    const tecto_request &r = req[i];
    int status = TECTO_OK;
    if (!valid_request(r)) status = TECTO_ERR_INVALID;
    else if (world_footprint(r.width, r.height) > sv->budget) status = TECTO_ERR_BUDGET;
    if (status == TECTO_OK) return false;
    res[i].status = status;
    it = q.waiting.erase(it);
    ++q.done;
    return true;
}

bool heavy(const tecto_server *sv, size_t cells) { return sv->heavy_slots > 0 && cells >= sv->heavy_cells; }

// Admission, in arrival order: a request joins while its footprint fits the budget and fewer than
// max_worlds are active, and the first that does not fit stops admission (no overtaking past it).
// A heavy request also needs a free heavy slot and no earlier heavy request waiting; while it waits
// for that, later light requests may join.
void admit(tecto_server *sv, Serving &q, const tecto_request *req, tecto_request_result *res, cudaStream_t st,
          const ServeClock &c)
{
    int heavy_live = 0;
    for (const Live &L : q.live) heavy_live += heavy(sv, L.cells) ? 1 : 0;
    bool heavy_waits = false;  // an earlier heavy request waits for its slot
    for (auto it = q.waiting.begin(); it != q.waiting.end();) {
        if (reject(sv, q, it, req, res)) continue;
        const int i = *it;
        const tecto_request &r = req[i];
        const size_t cells = (size_t)r.width * (size_t)r.height;
        const bool hv = heavy(sv, cells);
        if (hv && (heavy_waits || heavy_live >= sv->heavy_slots)) {
            heavy_waits = true;
            ++it;
            continue;
        }
        const size_t bytes = world_footprint(r.width, r.height);
        if (q.used + bytes > sv->budget || (int)q.live.size() >= sv->max_worlds) break;
        Live L{i, nullptr, bytes, cells, r.steps};
        if (!sv->dry) {
            // a world that cannot be created (out of memory, say) fails its own request only
            int rc = make_world(sv, r, st, &L.world);
            if (rc == TECTO_OK && (rc = tecto_batch_add(sv->batch, L.world, (tecto_stream_t)st)) != TECTO_OK)
                tecto_world_destroy(L.world);
            if (rc != TECTO_OK) {
                res[i].status = rc;
                it = q.waiting.erase(it);
                ++q.done;
                continue;
            }
        }
        q.used += bytes;
        q.peak = std::max(q.peak, (double)q.used);
        res[i].admit_s = c.now();
        q.live.push_back(L);
        it = q.waiting.erase(it);
        q.changed = true;
        heavy_live += hv ? 1 : 0;
    }
}

// Retires every admitted world with no steps left: its result (checksum, outputs named by `idx`),
// then it leaves the batch and its memory returns to the budget.
void retire(tecto_server *sv, Serving &q, tecto_request_result *res, cudaStream_t st, const ServeClock &c)
{
    for (size_t k = 0; k < q.live.size();) {
        if (q.live[k].steps_left > 0) { ++k; continue; }
        const int i = q.live[k].idx;
        if (!sv->dry) {
            finish_world(sv, q.live[k].world, i, st, res[i]);
            tecto_batch_remove(sv->batch, q.live[k].world);
            tecto_world_destroy(q.live[k].world);
        }
        res[i].finish_s = c.now();
        q.used -= q.live[k].bytes;
        q.live.erase(q.live.begin() + (long)k);
        ++q.done;
        q.changed = true;
    }
}

// One tick: every admitted world advances one step as one batch, then the finished ones retire.
int tick(tecto_server *sv, Serving &q, tecto_request_result *res, cudaStream_t st, ServeClock &c)
{
    q.max_active = std::max(q.max_active, (int)q.live.size());
    if (sv->dry) {
        size_t cells = 0;
        for (const Live &L : q.live) cells += L.cells;
        c.v += sv->dry_cost * (double)cells / 1e6;
    } else {
        // graphs pay off once the membership is stable; right after a change launch directly
        const int rc = batch_step_graph(sv->batch->b, 1, st, !q.changed);
        if (rc != TECTO_OK) return rc;
        TECTO_CUDA(cudaStreamSynchronize(st));
        if (sv->batch->b.sort.error) {  // the batch's sort look-back flag (per-world flags: at retire)
            uint32_t e = 0;
            TECTO_CUDA(cudaMemcpy(&e, sv->batch->b.sort.error, 4, cudaMemcpyDeviceToHost));
            if (e) {
                cudaMemset(sv->batch->b.sort.error, 0, 4);
                set_error("a bounded device-side wait gave up");
                return TECTO_ERR_DEVICE_TIMEOUT;
            }
        }
    }
    q.changed = false;
    ++q.ticks;
    for (Live &L : q.live) --L.steps_left;
    retire(sv, q, res, st, c);
    return TECTO_OK;
}

// After a failure: every admitted world leaves the batch and is freed, waiting requests are dropped.
void drop_all(tecto_server *sv, Serving &q)
{
    for (Live &L : q.live) {
        if (L.world) {
            tecto_batch_remove(sv->batch, L.world);
            tecto_world_destroy(L.world);
        }
    }
    q = Serving{};
}

int ensure_batch(tecto_server *sv)
{
    if (sv->dry || sv->batch) return TECTO_OK;
    return tecto_batch_create(&sv->batch);
}

}  // namespace

extern "C" {

int tecto_server_create(const tecto_settings *settings, size_t budget_bytes, int max_worlds, int flags,
                        tecto_server **out)
{
    if (!settings || !out || budget_bytes == 0) return TECTO_ERR_INVALID;
    tecto_server *sv = new (std::nothrow) tecto_server();
    if (!sv) return TECTO_ERR_OOM;
    sv->settings = *settings;
    sv->budget = budget_bytes;
    sv->max_worlds = (max_worlds <= 0 || max_worlds > kMaxBatchWorlds) ? kMaxBatchWorlds : max_worlds;
    sv->dry = (flags & TECTO_SERVER_DRY_RUN) != 0;
    sv->clock.dry = sv->dry;
    *out = sv;
    return TECTO_OK;
}

int tecto_server_destroy(tecto_server *sv)
{
    if (!sv) return TECTO_OK;
    drop_all(sv, sv->q);
    if (sv->batch) tecto_batch_destroy(sv->batch);
    delete sv;
    return TECTO_OK;
}

int tecto_server_set_output(tecto_server *server, const char *directory, int what, float height_min,
                            float height_max)
{
    if (!server || what < 0 || what > 7 || (what && !directory) ||
        ((what & TECTO_SERVER_OUT_HEIGHT_PNG) && !(height_max > height_min))) {
        set_error("tecto_server_set_output: invalid argument");
        return TECTO_ERR_INVALID;
    }
    server->out_dir = what ? directory : "";
    server->out_what = what;
    server->out_lo = height_min;
    server->out_hi = height_max;
    return TECTO_OK;
}

int tecto_server_set_init(tecto_server *server, int mode)
{
    if (!server || (mode != TECTO_SERVER_INIT_SYNTHETIC && mode != TECTO_SERVER_INIT_REFERENCE)) {
        set_error("tecto_server_set_init: invalid argument");
        return TECTO_ERR_INVALID;
    }
    server->init_mode = mode;
    return TECTO_OK;
}

int tecto_server_set_dry_cost(tecto_server *sv, double s)
{
    if (!sv || !(s >= 0)) return TECTO_ERR_INVALID;
    sv->dry_cost = s;
    return TECTO_OK;
}

int tecto_server_set_policy(tecto_server *sv, size_t heavy_cells, int heavy_slots)
{
    if (!sv || heavy_slots < 0 || (heavy_slots > 0 && heavy_cells == 0)) {
        set_error("tecto_server_set_policy: invalid argument");
        return TECTO_ERR_INVALID;
    }
    sv->heavy_cells = heavy_cells;
    sv->heavy_slots = heavy_slots;
    return TECTO_OK;
}

int tecto_server_run_trace(tecto_server *sv, const tecto_request *req, int n, tecto_stream_t stream,
                           tecto_request_result *res, tecto_server_stats *stats)
{
    if (!sv || (n > 0 && (!req || !res))) return TECTO_ERR_INVALID;
    if (!sv->q.live.empty() || !sv->q.waiting.empty()) {
        set_error("tecto_server_run_trace: live requests are pending on this server");
        return TECTO_ERR_INVALID;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int rc = ensure_batch(sv);
    if (rc != TECTO_OK) return rc;
    // arrival order (stable on ties)
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) {
        order[i] = i;
        res[i] = tecto_request_result{TECTO_OK, req[i].arrival_s, -1.0, -1.0, 0.0f};
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return req[a].arrival_s < req[b].arrival_s; });
    Serving q;
    ServeClock c;
    c.dry = sv->dry;
    int next = 0;
    while (q.done < n) {
        while (next < n && req[order[next]].arrival_s <= c.now()) q.waiting.push_back(order[next++]);
        admit(sv, q, req, res, st, c);
        retire(sv, q, res, st, c);  // zero-step requests leave at once
        if (q.live.empty()) {
            if (next < n && q.done < n) {  // idle until the next arrival
                const double wait = req[order[next]].arrival_s - c.now();
                if (sv->dry) c.v += std::max(wait, 0.0);
                else if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(wait));
            }
            continue;
        }
        if ((rc = tick(sv, q, res, st, c)) != TECTO_OK) break;
    }
    if (rc != TECTO_OK) {
        drop_all(sv, q);
        return rc;
    }
    finish_stats(req, n, res, c.now(), q.ticks, q.max_active, q.peak, stats);
    if (!sv->dry) return tecto_batch_check(sv->batch, stream);
    return TECTO_OK;
}

int tecto_server_run_trace_sequential(tecto_server *sv, const tecto_request *req, int n, tecto_stream_t stream,
                                      tecto_request_result *res, tecto_server_stats *stats)
{
    if (!sv || (n > 0 && (!req || !res))) return TECTO_ERR_INVALID;
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) {
        order[i] = i;
        res[i] = tecto_request_result{TECTO_OK, req[i].arrival_s, -1.0, -1.0, 0.0f};
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return req[a].arrival_s < req[b].arrival_s; });
    double vclock = 0, peak = 0;
    const auto t0 = Clock::now();
    auto now = [&]() {
        return sv->dry ? vclock : std::chrono::duration<double>(Clock::now() - t0).count();
    };
    int ticks = 0;
    for (int k = 0; k < n; ++k) {
        const int i = order[k];
        const tecto_request &r = req[i];
        if (!valid_request(r)) {
            res[i].status = TECTO_ERR_INVALID;
            continue;
        }
        const size_t bytes = world_footprint(r.width, r.height);
        if (bytes > sv->budget) {
            res[i].status = TECTO_ERR_BUDGET;
            continue;
        }
        const double wait = r.arrival_s - now();
        if (wait > 0) {
            if (sv->dry) vclock += wait;
            else std::this_thread::sleep_for(std::chrono::duration<double>(wait));
        }
        res[i].admit_s = now();
        peak = std::max(peak, (double)bytes);
        if (sv->dry) {
            vclock += sv->dry_cost * (double)r.width * (double)r.height / 1e6 * (double)r.steps;
        } else {
            tecto_world *w = nullptr;
            int rc = make_world(sv, r, st, &w);
            if (rc != TECTO_OK) return rc;
            rc = tecto_world_step(w, r.steps, stream);
            if (rc == TECTO_OK) rc = tecto_world_check(w, stream);
            if (rc != TECTO_OK) {
                tecto_world_destroy(w);
                return rc;
            }
            finish_world(sv, w, i, st, res[i]);
            tecto_world_destroy(w);
        }
        ticks += r.steps;
        res[i].finish_s = now();
    }
    finish_stats(req, n, res, now(), ticks, 1, peak, stats);
    return TECTO_OK;
}

/* ---- live serving: requests submitted as they come, the caller drives the ticks ---------- */

int tecto_server_submit(tecto_server *sv, const tecto_request *request, int *ticket)
{
    if (!sv || !request || !ticket || sv->reqs.size() >= ((size_t)1 << 30)) {
        set_error("tecto_server_submit: invalid argument");
        return TECTO_ERR_INVALID;
    }
    const int i = (int)sv->reqs.size();
    const double t = sv->clock.now();
    sv->reqs.push_back(*request);
    sv->reqs.back().arrival_s = t;
    sv->results.push_back(tecto_request_result{TECTO_OK, t, -1.0, -1.0, 0.0f});
    // a request that can never be served is answered at once
    const tecto_request &r = sv->reqs.back();
    if (!valid_request(r)) sv->results.back().status = TECTO_ERR_INVALID;
    else if (world_footprint(r.width, r.height) > sv->budget) sv->results.back().status = TECTO_ERR_BUDGET;
    else sv->q.waiting.push_back(i);
    *ticket = i;
    return TECTO_OK;
}

int tecto_server_tick(tecto_server *sv, tecto_stream_t stream, int *active, int *waiting)
{
    if (!sv) return TECTO_ERR_INVALID;
    cudaStream_t st = (cudaStream_t)stream;
    Serving &q = sv->q;
    int rc = ensure_batch(sv);
    if (rc == TECTO_OK) admit(sv, q, sv->reqs.data(), sv->results.data(), st, sv->clock);
    if (rc == TECTO_OK) {
        retire(sv, q, sv->results.data(), st, sv->clock);  // zero-step requests leave at once
        if (!q.live.empty()) rc = tick(sv, q, sv->results.data(), st, sv->clock);
    }
    if (rc != TECTO_OK) {  // every request still pending fails with the error
        for (const Live &L : q.live) sv->results[L.idx].status = rc;
        for (int i : q.waiting) sv->results[i].status = rc;
        drop_all(sv, q);
    }
    if (active) *active = (int)q.live.size();
    if (waiting) *waiting = (int)q.waiting.size();
    return rc;
}

int tecto_server_poll(tecto_server *sv, int ticket, int *state, tecto_request_result *result)
{
    if (!sv || ticket < 0 || ticket >= (int)sv->reqs.size()) {
        set_error("tecto_server_poll: unknown ticket");
        return TECTO_ERR_INVALID;
    }
    const tecto_request_result &r = sv->results[(size_t)ticket];
    if (state)
        *state = (r.status != TECTO_OK || r.finish_s >= 0) ? TECTO_REQUEST_DONE
                 : r.admit_s >= 0                         ? TECTO_REQUEST_RUNNING
                                                          : TECTO_REQUEST_WAITING;
    if (result) *result = r;
    return TECTO_OK;
}

int tecto_server_live_stats(tecto_server *sv, tecto_server_stats *stats)
{
    if (!sv || !stats) return TECTO_ERR_INVALID;
    finish_stats(sv->reqs.data(), (int)sv->reqs.size(), sv->results.data(), sv->clock.now(), sv->q.ticks,
                 sv->q.max_active, sv->q.peak, stats);
    return TECTO_OK;
}

}  // extern "C"
