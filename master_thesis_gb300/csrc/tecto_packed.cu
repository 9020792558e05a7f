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
    size_t maxn = 0;
    for (const tecto_world *w : b.members) maxn = std::max(maxn, w->N);
    const dim3 grid((unsigned)std::min<size_t>((maxn + 1023) / 1024, 1024), (unsigned)b.members.size());
    if (up) TECTO_CUDA(cudaMemcpyAsync(b.stage, host, bytes, cudaMemcpyHostToDevice, st));
    switch (esz) {
        case 16:
            if (up) k_pack<float4, true><<<grid, 256, 0, st>>>(b.d_worlds, field, b.cur_h, b.cur_wsf, b.cur_id, (float4 *)b.stage);
            else k_pack<float4, false><<<grid, 256, 0, st>>>(b.d_worlds, field, b.cur_h, b.cur_wsf, b.cur_id, (float4 *)b.stage);
            break;
        case 4:
            if (up) k_pack<uint32_t, true><<<grid, 256, 0, st>>>(b.d_worlds, field, b.cur_h, b.cur_wsf, b.cur_id, (uint32_t *)b.stage);
            else k_pack<uint32_t, false><<<grid, 256, 0, st>>>(b.d_worlds, field, b.cur_h, b.cur_wsf, b.cur_id, (uint32_t *)b.stage);
            break;
        default:
            if (up) k_pack_bytes<true><<<grid, 256, 0, st>>>(b.d_worlds, b.cur_id, (uint8_t *)b.stage);
            else k_pack_bytes<false><<<grid, 256, 0, st>>>(b.d_worlds, b.cur_id, (uint8_t *)b.stage);
            break;
    }
    TECTO_CUDA(cudaGetLastError());
    b.launches += 1;
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
