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

// Grid (blocks, worlds): world blockIdx.y's cells, grid-stride; the packed buffer holds world b's
// elements from its virtual base on.  T is the element type (a 16-byte flux cell, 4-byte scalars).
template <typename T, bool TO_WORLD>
__global__ __launch_bounds__(256) void k_pack(const WorldDev *worlds, int field, int cur_h, int cur_wsf, int cur_id,
                                              T *packed)
{
    const WorldDev &wd = worlds[blockIdx.y];
    T *fld = reinterpret_cast<T *>(field_base(wd, field, cur_h, cur_wsf, cur_id));
    T *pk = packed + wd.vbase;
    const uint32_t n = wd.N;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (TO_WORLD) fld[i] = pk[i];
        else pk[i] = fld[i];
    }
}

template <bool TO_WORLD>
__global__ __launch_bounds__(256) void k_pack_bytes(const WorldDev *worlds, int cur_id, uint8_t *packed)
{
    const WorldDev &wd = worlds[blockIdx.y];
    uint8_t *fld = wd.id[cur_id];
    uint8_t *pk = packed + wd.vbase;
    const uint32_t n = wd.N;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (TO_WORLD) fld[i] = pk[i];
        else pk[i] = fld[i];
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
    size_t maxn = 0;
    for (const tecto_world *w : b.members) maxn = std::max(maxn, w->N);
    const dim3 grid((unsigned)std::min<size_t>((maxn + 1023) / 1024, 1024), (unsigned)b.members.size());
    switch (esz) {
        case 16:
            if (to_world) k_pack<float4, true><<<grid, 256, 0, st>>>(b.d_worlds, field, b.cur_h, b.cur_wsf, b.cur_id, (float4 *)buf);
            else k_pack<float4, false><<<grid, 256, 0, st>>>(b.d_worlds, field, b.cur_h, b.cur_wsf, b.cur_id, (float4 *)buf);
            break;
        case 4:
            if (to_world) k_pack<uint32_t, true><<<grid, 256, 0, st>>>(b.d_worlds, field, b.cur_h, b.cur_wsf, b.cur_id, (uint32_t *)buf);
            else k_pack<uint32_t, false><<<grid, 256, 0, st>>>(b.d_worlds, field, b.cur_h, b.cur_wsf, b.cur_id, (uint32_t *)buf);
            break;
        default:
            if (to_world) k_pack_bytes<true><<<grid, 256, 0, st>>>(b.d_worlds, b.cur_id, (uint8_t *)buf);
            else k_pack_bytes<false><<<grid, 256, 0, st>>>(b.d_worlds, b.cur_id, (uint8_t *)buf);
            break;
    }
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

// The per-field staging buffer (allocated for the batch's cells) and its two events.
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
    void **buf = up ? &b.up_stage[slot] : &b.down_stage[slot];
    size_t *cap = up ? &b.up_bytes[slot] : &b.down_bytes[slot];
    if (*cap != bytes) {
        TECTO_CUDA(cudaDeviceSynchronize());  // the old buffer may still be in flight on either stream
        if (*buf) cudaFree(*buf);
        *buf = nullptr;
        *cap = 0;
        TECTO_CUDA(cudaMalloc(buf, bytes));
        *cap = bytes;
    }
    if ((rc = ensure_event(up ? &b.ev_up_ready[slot] : &b.ev_down_ready[slot])) != TECTO_OK) return rc;
    if ((rc = ensure_event(up ? &b.ev_up_free[slot] : &b.ev_down_free[slot])) != TECTO_OK) return rc;
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
    TECTO_CUDA(cudaStreamWaitEvent(cs, b.ev_up_free[slot], 0));  // the last commit has read the buffer
    TECTO_CUDA(cudaMemcpyAsync(b.up_stage[slot], host, bytes, cudaMemcpyHostToDevice, cs));
    TECTO_CUDA(cudaEventRecord(b.ev_up_ready[slot], cs));
    return TECTO_OK;
}

int tecto_batch_commit_upload(tecto_batch *batch, int field, tecto_stream_t stream)
{
    if (!batch) return TECTO_ERR_INVALID;
    Batch &b = batch->b;
    const int slot = field_slot(field);
    if (slot < 0 || !b.up_stage[slot] || b.up_bytes[slot] != b.total * field_elem(field)) {
        set_error("tecto_batch_commit_upload: nothing staged for this field and batch");
        return TECTO_ERR_INVALID;
    }
    const cudaStream_t st = (cudaStream_t)stream;
    int rc = batch_prepare(b, st);
    if (rc != TECTO_OK) return rc;
    TECTO_CUDA(cudaStreamWaitEvent(st, b.ev_up_ready[slot], 0));
    if ((rc = launch_pack(b, field, b.up_stage[slot], true, st)) != TECTO_OK) return rc;
    TECTO_CUDA(cudaEventRecord(b.ev_up_free[slot], st));
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
    TECTO_CUDA(cudaStreamWaitEvent(st, b.ev_down_free[slot], 0));  // the last fetch has read the buffer
    if ((rc = launch_pack(b, field, b.down_stage[slot], false, st)) != TECTO_OK) return rc;
    TECTO_CUDA(cudaEventRecord(b.ev_down_ready[slot], st));
    return TECTO_OK;
}

int tecto_batch_fetch_download_async(tecto_batch *batch, int field, void *host, size_t bytes,
                                     tecto_stream_t copy_stream)
{
    if (!batch || !host) return TECTO_ERR_INVALID;
    Batch &b = batch->b;
    const int slot = field_slot(field);
    if (slot < 0 || !b.down_stage[slot] || bytes != b.down_bytes[slot]) {
        set_error("tecto_batch_fetch_download_async: no gathered field of this size");
        return TECTO_ERR_INVALID;
    }
    const cudaStream_t cs = (cudaStream_t)copy_stream;
    TECTO_CUDA(cudaStreamWaitEvent(cs, b.ev_down_ready[slot], 0));
    TECTO_CUDA(cudaMemcpyAsync(host, b.down_stage[slot], bytes, cudaMemcpyDeviceToHost, cs));
    TECTO_CUDA(cudaEventRecord(b.ev_down_free[slot], cs));
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
