// tecto_packed.cu - one field of every world of a batch to or from one packed host buffer: one
// host<->device copy through a batch staging buffer and one scatter (or gather) kernel, instead of
// a copy per world.  A serving loop that moves hundreds of small worlds per step pays one copy's
// setup per field instead of one per world.
#include <algorithm>

#include "tecto_internal.cuh"

namespace tecto {

namespace {

__device__ __forceinline__ void *field_base(const WorldDev &wd, int field, int cur_h, int cur_wsf, int cur_id)
{
    switch (field) {
        case TECTO_FIELD_HEIGHT: return wd.h[cur_h];
        case TECTO_FIELD_WATER: return wd.w[cur_wsf];
        case TECTO_FIELD_SEDIMENT: return wd.s[cur_wsf];
        case TECTO_FIELD_FLUX: return wd.flux[cur_wsf];
        case TECTO_FIELD_PLATE_ID: return wd.id[cur_id];
        default: return wd.labels;  // TECTO_FIELD_LABELS
    }
}

// The packed buffer holds the worlds' elements in batch order, world w's from its virtual base
// vbase[w] on.  Each block copies kPackSpan consecutive virtual cells, 8 independent elements per
// thread, between the packed buffer and the fields of the one or few worlds they belong to (found
// by a binary search of the bases).  T is the element type (a 16-byte flux cell, 4-byte scalars,
// plate-id bytes).
constexpr int kPackThreads = 256;
constexpr int kPackSpan = kPackThreads * 8;

template <typename T, bool TO_WORLD>
__global__ __launch_bounds__(kPackThreads) void k_pack(const WorldDev *worlds, const uint32_t *vbase, int nworlds,
                                                       int field, int cur_h, int cur_wsf, int cur_id, T *packed)
{
    __shared__ int s_first;
    const uint32_t b0 = blockIdx.x * (uint32_t)kPackSpan;
    const uint32_t b1 = min(b0 + (uint32_t)kPackSpan, vbase[nworlds]);
    if (threadIdx.x == 0) {  // the last world whose base is <= b0
        int lo = 0, hi = nworlds - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (vbase[mid] <= b0) lo = mid;
            else hi = mid - 1;
        }
        s_first = lo;
    }
    __syncthreads();
    for (int w = s_first; w < nworlds && vbase[w] < b1; ++w) {
        const WorldDev &wd = worlds[w];
        T *fld = reinterpret_cast<T *>(field_base(wd, field, cur_h, cur_wsf, cur_id));
        const uint32_t vb = vbase[w], lo = max(b0, vb), hi = min(b1, vbase[w + 1]);
#pragma unroll
        for (int k = 0; k < kPackSpan / kPackThreads; ++k) {
            const uint32_t i = lo + (uint32_t)(k * kPackThreads) + threadIdx.x;
            if (i < hi) {
                if (TO_WORLD) fld[i - vb] = packed[i];
                else packed[i] = fld[i - vb];
            }
        }
    }
}

size_t field_elem(int field)
{
    switch (field) {
        case TECTO_FIELD_HEIGHT:
        case TECTO_FIELD_WATER:
        case TECTO_FIELD_SEDIMENT:
        case TECTO_FIELD_LABELS: return 4;
        case TECTO_FIELD_FLUX: return 16;
        case TECTO_FIELD_PLATE_ID: return 1;
        default: return 0;
    }
}

// Scatter (to the worlds) or gather (from the worlds) between a packed device buffer and the
// members' fields, on stream st.
int launch_pack(Batch &b, int field, void *buf, bool to_world, cudaStream_t st)
{
    const size_t esz = field_elem(field);
    const unsigned grid = (unsigned)((b.total + kPackSpan - 1) / kPackSpan);
    const int n = (int)b.members.size();
    if (grid == 0) return TECTO_OK;
#define TECTO_PACK(T)                                                                                               \
    (to_world ? k_pack<T, true><<<grid, kPackThreads, 0, st>>>(b.d_worlds, b.d_vbase, n, field, b.cur_h, b.cur_wsf, \
                                                               b.cur_id, (T *)buf)                                  \
              : k_pack<T, false><<<grid, kPackThreads, 0, st>>>(b.d_worlds, b.d_vbase, n, field, b.cur_h,          \
                                                                b.cur_wsf, b.cur_id, (T *)buf))
    switch (esz) {
        case 16: TECTO_PACK(float4); break;
        case 4: TECTO_PACK(uint32_t); break;
        default: TECTO_PACK(uint8_t); break;
    }
#undef TECTO_PACK
    TECTO_CUDA(cudaGetLastError());
    b.launches += 1;
    return TECTO_OK;
}

// Index of a field among the packed-transfer fields, or -1.
int field_slot(int field)
{
    switch (field) {
        case TECTO_FIELD_HEIGHT: return 0;
        case TECTO_FIELD_WATER: return 1;
        case TECTO_FIELD_SEDIMENT: return 2;
        case TECTO_FIELD_FLUX: return 3;
        case TECTO_FIELD_PLATE_ID: return 4;
        case TECTO_FIELD_LABELS: return 5;
        default: return -1;
    }
}

int ensure_event(cudaEvent_t *e)
{
    if (!*e) TECTO_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    return TECTO_OK;
}

// The per-field staging buffers (two, allocated for the batch's cells) and their events.  A change
// of size drops both buffers and restarts the field's counters.
int pipe_prepare(tecto_batch *batch, int field, size_t bytes, bool up, int *slot_out, cudaStream_t st)
{
    if (!batch) return TECTO_ERR_INVALID;
    Batch &b = batch->b;
    const int slot = field_slot(field);
    if (b.members.empty() || slot < 0) {
        set_error("pipelined transfer: empty batch or a field without packed transfers");
        return TECTO_ERR_INVALID;
    }
    int rc = TECTO_OK;
    if (b.dirty) {  // tables rebuilt on this stream: let them land before the other stream uses them
        if ((rc = batch_prepare(b, st)) != TECTO_OK) return rc;
        TECTO_CUDA(cudaStreamSynchronize(st));
    }
    if (bytes != b.total * field_elem(field)) {
        set_error("pipelined transfer: bytes must be the batch's cells times the field's element size");
        return TECTO_ERR_INVALID;
    }
    size_t *cap = up ? &b.up_bytes[slot] : &b.down_bytes[slot];
    if (*cap != bytes) {
        TECTO_CUDA(cudaDeviceSynchronize());  // the old buffers may still be in flight on any stream
        for (int k = 0; k < 2; ++k) {
            void **buf = up ? &b.up_stage[slot][k] : &b.down_stage[slot][k];
            if (*buf) cudaFree(*buf);
            *buf = nullptr;
        }
        *cap = 0;
        for (int k = 0; k < 2; ++k) TECTO_CUDA(cudaMalloc(up ? &b.up_stage[slot][k] : &b.down_stage[slot][k], bytes));
        *cap = bytes;
        if (up) b.n_staged[slot] = b.n_committed[slot] = 0;
        else b.n_gathered[slot] = b.n_fetched[slot] = 0;
    }
    for (int k = 0; k < 2; ++k) {
        if ((rc = ensure_event(up ? &b.ev_up_ready[slot][k] : &b.ev_down_ready[slot][k])) != TECTO_OK) return rc;
        if ((rc = ensure_event(up ? &b.ev_up_free[slot][k] : &b.ev_down_free[slot][k])) != TECTO_OK) return rc;
    }
    *slot_out = slot;
    return TECTO_OK;
}

int packed_transfer(tecto_batch *batch, int field, void *host, size_t bytes, cudaStream_t st, bool up)
{
    if (!batch || !host) return TECTO_ERR_INVALID;
    Batch &b = batch->b;
    const size_t esz = field_elem(field);
    if (b.members.empty() || esz == 0) {
        set_error("packed transfer: empty batch or a field without packed transfers");
        return TECTO_ERR_INVALID;
    }
    int rc = batch_prepare(b, st);
    if (rc != TECTO_OK) return rc;
    if (bytes != b.total * esz) {
        set_error("packed transfer: bytes must be the batch's cells times the field's element size");
        return TECTO_ERR_INVALID;
    }
    if (bytes > b.stage_bytes) {
        if (b.stage) {
            TECTO_CUDA(cudaStreamSynchronize(st));
            cudaFree(b.stage);
        }
        b.stage = nullptr;
        b.stage_bytes = 0;
        TECTO_CUDA(cudaMalloc(&b.stage, bytes));
        b.stage_bytes = bytes;
    }
    if (up) TECTO_CUDA(cudaMemcpyAsync(b.stage, host, bytes, cudaMemcpyHostToDevice, st));
    if ((rc = launch_pack(b, field, b.stage, up, st)) != TECTO_OK) return rc;
    if (!up) TECTO_CUDA(cudaMemcpyAsync(host, b.stage, bytes, cudaMemcpyDeviceToHost, st));
    return TECTO_OK;
}

}  // namespace

}  // namespace tecto

using namespace tecto;

extern "C" {

int tecto_batch_upload_async(tecto_batch *batch, int field, const void *host, size_t bytes, tecto_stream_t stream)
{
    return packed_transfer(batch, field, const_cast<void *>(host), bytes, (cudaStream_t)stream, true);
}

int tecto_batch_download_async(tecto_batch *batch, int field, void *host, size_t bytes, tecto_stream_t stream)
{
    return packed_transfer(batch, field, host, bytes, (cudaStream_t)stream, false);
}

int tecto_batch_stage_upload_async(tecto_batch *batch, int field, const void *host, size_t bytes,
                                   tecto_stream_t copy_stream)
{
    const cudaStream_t cs = (cudaStream_t)copy_stream;
    int slot = 0;
    int rc = pipe_prepare(batch, field, bytes, true, &slot, cs);
    if (rc != TECTO_OK) return rc;
    Batch &b = batch->b;
    if (b.n_staged[slot] >= b.n_committed[slot] + 2) {
        set_error("tecto_batch_stage_upload_async: two stages of this field already wait for their commits");
        return TECTO_ERR_INVALID;
    }
    const int k = (int)(b.n_staged[slot] & 1);
    TECTO_CUDA(cudaStreamWaitEvent(cs, b.ev_up_free[slot][k], 0));  // the commit that last read this buffer
    TECTO_CUDA(cudaMemcpyAsync(b.up_stage[slot][k], host, bytes, cudaMemcpyHostToDevice, cs));
    TECTO_CUDA(cudaEventRecord(b.ev_up_ready[slot][k], cs));
    b.n_staged[slot] += 1;
    return TECTO_OK;
}

int tecto_batch_commit_upload(tecto_batch *batch, int field, tecto_stream_t stream)
{
    if (!batch) return TECTO_ERR_INVALID;
    Batch &b = batch->b;
    const int slot = field_slot(field);
    if (slot < 0 || b.up_bytes[slot] != b.total * field_elem(field) || b.n_committed[slot] >= b.n_staged[slot]) {
        set_error("tecto_batch_commit_upload: nothing staged for this field and batch");
        return TECTO_ERR_INVALID;
    }
    const cudaStream_t st = (cudaStream_t)stream;
    int rc = batch_prepare(b, st);
    if (rc != TECTO_OK) return rc;
    const int k = (int)(b.n_committed[slot] & 1);
    TECTO_CUDA(cudaStreamWaitEvent(st, b.ev_up_ready[slot][k], 0));
    if ((rc = launch_pack(b, field, b.up_stage[slot][k], true, st)) != TECTO_OK) return rc;
    TECTO_CUDA(cudaEventRecord(b.ev_up_free[slot][k], st));
    b.n_committed[slot] += 1;
    return TECTO_OK;
}

int tecto_batch_gather_download(tecto_batch *batch, int field, tecto_stream_t stream)
{
    if (!batch) return TECTO_ERR_INVALID;
    const cudaStream_t st = (cudaStream_t)stream;
    const size_t bytes = batch->b.total * field_elem(field);
    int slot = 0;
    int rc = pipe_prepare(batch, field, bytes, false, &slot, st);
    if (rc != TECTO_OK) return rc;
    Batch &b = batch->b;
    if (b.n_gathered[slot] >= b.n_fetched[slot] + 2) {
        set_error("tecto_batch_gather_download: two gathers of this field already wait for their fetches");
        return TECTO_ERR_INVALID;
    }
    const int k = (int)(b.n_gathered[slot] & 1);
    TECTO_CUDA(cudaStreamWaitEvent(st, b.ev_down_free[slot][k], 0));  // the fetch that last read this buffer
    if ((rc = launch_pack(b, field, b.down_stage[slot][k], false, st)) != TECTO_OK) return rc;
    TECTO_CUDA(cudaEventRecord(b.ev_down_ready[slot][k], st));
    b.n_gathered[slot] += 1;
    return TECTO_OK;
}

int tecto_batch_fetch_download_async(tecto_batch *batch, int field, void *host, size_t bytes,
                                     tecto_stream_t copy_stream)
{
    if (!batch || !host) return TECTO_ERR_INVALID;
    Batch &b = batch->b;
    const int slot = field_slot(field);
    if (slot < 0 || bytes != b.down_bytes[slot] || b.n_fetched[slot] >= b.n_gathered[slot]) {
        set_error("tecto_batch_fetch_download_async: no gathered field of this size");
        return TECTO_ERR_INVALID;
    }
    const cudaStream_t cs = (cudaStream_t)copy_stream;
    const int k = (int)(b.n_fetched[slot] & 1);
    TECTO_CUDA(cudaStreamWaitEvent(cs, b.ev_down_ready[slot][k], 0));
    TECTO_CUDA(cudaMemcpyAsync(host, b.down_stage[slot][k], bytes, cudaMemcpyDeviceToHost, cs));
    TECTO_CUDA(cudaEventRecord(b.ev_down_free[slot][k], cs));
    b.n_fetched[slot] += 1;
    return TECTO_OK;
}

int tecto_batch_offsets(const tecto_batch *batch, size_t *cell_offsets, int capacity)
{
    if (!batch || !cell_offsets) return TECTO_ERR_INVALID;
    const Batch &b = batch->b;
    if (capacity < (int)b.members.size() + 1) return TECTO_ERR_INVALID;
    size_t off = 0;
    for (size_t i = 0; i < b.members.size(); ++i) {
        cell_offsets[i] = off;
        off += b.members[i]->N;
    }
    cell_offsets[b.members.size()] = off;
    return TECTO_OK;
}

}  // extern "C"
