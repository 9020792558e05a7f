// ref_relabel.cu - TEST INFRASTRUCTURE ONLY: the reference's CCL relabel of plate fragments
// (PlateTectonicSim::applyCCL, MarWo22/master_thesis src/cuda_compute/plate_tectonic_sim.cu:374-467)
// run on this GPU with the reference's own device code (oracle/_ref/ref_kernels.cubin, compiled
// from its sources by oracle/Makefile) and the same thrust calls between the kernels, to produce
// golden vectors for the oracle's relabel.  Launch shapes are the reference's: 256 threads per
// block, one thread per cell (W * H a multiple of 256), one block for createLabelIdLookup.  The
// fill loop (assignUnassignedIdsToNeighbor until no cell waits, :450-466) stops after max_rounds
// passes; the reference has no such limit.  The engine never links this file.
//
// Kernels, in applyCCL's order: init, analyzeClamped, reduce, analyzeUnclamped (ccl.cu),
// createPlateIdLabelMap (plate_tectonics_kernel.cu:1394-1407), thrust sort / reduce_by_key /
// sort_by_key (plate_tectonic_sim.cu:404-420), getMaxSizeLabels (:3114-3128),
// createLabelIdLookup (:3130-3185), postCClIdReassign (:3187-3206), assignUnassignedIdsToNeighbor
// (:2052-2101).
#include <cuda.h>
#include <cuda_runtime.h>
#include <thrust/device_ptr.h>
#include <thrust/functional.h>
#include <thrust/iterator/constant_iterator.h>
#include <thrust/reduce.h>
#include <thrust/sort.h>

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/tecto.h"

namespace {

// The reference's PlateData (types/plate_data.h), 84 bytes, and CudaTexture<T> (16 bytes).
struct RVec2 {
    float x, y;
};
struct RPlate {
    float velocity, velocitySmoothed;
    RVec2 direction, directionSmoothed, pixelCenter, velocityChange, geometricCenter, asthenosphereVelocity;
    int size;
    float mass;
    int perimeter;
    float breakScore, circularity;
    bool used, hasMoved;
    int mergeWaitTime;
};
static_assert(sizeof(RPlate) == 84, "PlateData layout");
struct RTex {
    void *arr;
    int w, h;
};
static_assert(sizeof(RTex) == 16, "CudaTexture layout");

const char *kRelabelNames[] = {
    "_Z4initPK11CudaTextureIhEPS_IjE",
    "_Z14analyzeClampedP11CudaTextureIjE",
    "_Z6reducePK11CudaTextureIhEPS_IjE",
    "_Z16analyzeUnclampedP11CudaTextureIjE",
    "_Z21createPlateIdLabelMapPK11CudaTextureIhEPKS_IjEPS_ImE",
    "_Z16getMaxSizeLabelsPK11CudaTextureImEPKS_IjEPS_IiEi",
    "_Z19createLabelIdLookupPK11CudaTextureImEPKS_IjEPKS_IiEP9PlateDataPS_IhEi",
    "_Z17postCClIdReassignPK11CudaTextureIhEPKS_IjEPS0_PS3_Pi",
    "_Z29assignUnassignedIdsToNeighborP11CudaTextureIhEPKjjPb",
};
enum R { RINIT, RCLAMP, RRED, RUNCL, RMAP, RMAX, RLOOKUP, RPOST, RFILL, NR };

CUmodule g_rmod = nullptr;
CUfunction g_rfn[NR] = {};
CUdeviceptr g_rsettings = 0;
std::string g_rerr;

int rfail(const std::string &m)
{
    g_rerr = m;
    return -1;
}

#define RDRV(call)                                                         \
    do {                                                                   \
        CUresult r_ = (call);                                              \
        if (r_ != CUDA_SUCCESS) {                                          \
            const char *s_ = nullptr;                                      \
            cuGetErrorString(r_, &s_);                                     \
            return rfail(std::string(#call) + ": " + (s_ ? s_ : "?"));     \
        }                                                                  \
    } while (0)
#define RRT(call)                                                                          \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) return rfail(std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int rlaunch(R k, unsigned blocks, void **args)
{
    RDRV(cuLaunchKernel(g_rfn[k], blocks, 1, 1, 256, 1, 1, 0, nullptr, args, nullptr));
    return 0;
}

// Device buffers of one run, freed together.
struct Bufs {
    std::vector<void *> p;
    ~Bufs()
    {
        for (void *q : p) cudaFree(q);
    }
    void *get(size_t n, int fill)
    {
        void *q = nullptr;
        if (cudaMalloc(&q, n) != cudaSuccess) return nullptr;
        cudaMemset(q, fill, n);
        p.push_back(q);
        return q;
    }
};

int run(int W, int H, uint8_t *ids, const int *plate_sizes, uint32_t *labels_out, float *markers_out,
        int max_rounds, int *rounds_out, int *unassigned_out)
{
    const size_t N = (size_t)W * (size_t)H;
    const unsigned blocks = (unsigned)(N / 256);
    const int labelCountSize = (int)((double)W * (double)H * 0.01);  // as plate_tectonic_sim.cu:391
    Bufs b;
    uint8_t *d_ids = (uint8_t *)b.get(N, 0);
    uint32_t *d_labels = (uint32_t *)b.get(N * 4, 0);
    uint64_t *d_packed = (uint64_t *)b.get(N * 8, 0);
    // capacity N (the reference allocates labelCountSize; the run refuses more labels than that)
    uint32_t *d_counts = (uint32_t *)b.get(N * 4, 0);
    uint64_t *d_unique = (uint64_t *)b.get(N * 8, 0);
    int *d_maxcounts = (int *)b.get(255 * 4, 0);
    uint8_t *d_lookup = (uint8_t *)b.get(N, 255);
    uint32_t *d_unassigned = (uint32_t *)b.get(N * 4, 0);
    int *d_ucount = (int *)b.get(4, 0);
    bool *d_work = (bool *)b.get(1, 0);
    RPlate *d_plates = (RPlate *)b.get(255 * sizeof(RPlate), 0);
    RTex *d_tex = (RTex *)b.get(8 * sizeof(RTex), 0);
    if (!d_ids || !d_labels || !d_packed || !d_counts || !d_unique || !d_maxcounts || !d_lookup || !d_unassigned ||
        !d_ucount || !d_work || !d_plates || !d_tex)
        return rfail("cudaMalloc failed");
    // plate records: velocity carries the plate's own index (a marker of which record a slot holds
    // after createLabelIdLookup's copies), size the caller's sizes
    std::vector<RPlate> pl(255);
    std::memset(pl.data(), 0, pl.size() * sizeof(RPlate));
    for (int k = 0; k < 255; ++k) {
        pl[k].velocity = (float)k;
        pl[k].size = plate_sizes[k];
        pl[k].mass = 1.0f;
    }
    const RTex host[8] = {{d_ids, W, H},          {d_labels, W, H},          {d_packed, W, H},
                          {d_counts, labelCountSize, 1}, {d_unique, labelCountSize, 1}, {d_maxcounts, 255, 1},
                          {d_lookup, W, H},       {d_unassigned, W, H}};
    RRT(cudaMemcpy(d_tex, host, sizeof(host), cudaMemcpyHostToDevice));
    RRT(cudaMemcpy(d_ids, ids, N, cudaMemcpyHostToDevice));
    RRT(cudaMemcpy(d_plates, pl.data(), pl.size() * sizeof(RPlate), cudaMemcpyHostToDevice));
    RTex *tIds = d_tex + 0, *tLabels = d_tex + 1, *tPacked = d_tex + 2, *tCounts = d_tex + 3, *tUnique = d_tex + 4;
    RTex *tMax = d_tex + 5, *tLookup = d_tex + 6, *tUnassigned = d_tex + 7;

    // 8-way CCL (plate_tectonic_sim.cu:380-387)
    {
        void *a[] = {&tIds, &tLabels};
        if (rlaunch(RINIT, blocks, a)) return -1;
    }
    {
        void *a[] = {&tLabels};
        if (rlaunch(RCLAMP, blocks, a)) return -1;
    }
    {
        void *a[] = {&tIds, &tLabels};
        if (rlaunch(RRED, blocks, a)) return -1;
    }
    {
        void *a[] = {&tLabels};
        if (rlaunch(RUNCL, blocks, a)) return -1;
    }
    {
        void *a[] = {&tIds, &tLabels, &tPacked};
        if (rlaunch(RMAP, blocks, a)) return -1;
    }
    // the thrust calls of plate_tectonic_sim.cu:404-420, as written there
    const thrust::device_ptr<uint64_t> packed(d_packed);
    const thrust::device_ptr<unsigned int> counts(d_counts);
    const thrust::device_ptr<uint64_t> uniq(d_unique);
    thrust::sort(packed, packed + N, thrust::greater<unsigned int>());
    const auto end = thrust::reduce_by_key(packed, packed + N, thrust::make_constant_iterator<int>(1), uniq, counts);
    const int size = static_cast<int>(end.first - uniq);
    if (size > labelCountSize) return rfail("more components than the reference's label buffer holds (1% of cells)");
    thrust::sort_by_key(counts, counts + size, uniq, thrust::greater<unsigned int>());
    RRT(cudaDeviceSynchronize());
    int numLabels = size;
    {
        void *a[] = {&tUnique, &tCounts, &tMax, &numLabels};
        if (rlaunch(RMAX, (unsigned)((size + 255) / 256), a)) return -1;
    }
    {
        void *a[] = {&tUnique, &tCounts, &tMax, &d_plates, &tLookup, &numLabels};
        if (rlaunch(RLOOKUP, 1, a)) return -1;  // NUM_BLOCKS_PLATES
    }
    {
        void *a[] = {&tLookup, &tLabels, &tIds, &tUnassigned, &d_ucount};
        if (rlaunch(RPOST, blocks, a)) return -1;
    }
    int remaining = 0;
    RRT(cudaMemcpy(&remaining, d_ucount, 4, cudaMemcpyDeviceToHost));
    int rounds = 0;
    if (remaining) {
        unsigned len = (unsigned)remaining;
        bool work = true;
        while (work && rounds < max_rounds) {
            RRT(cudaMemset(d_work, 0, 1));
            void *a[] = {&tIds, &d_unassigned, &len, &d_work};
            if (rlaunch(RFILL, (unsigned)((remaining + 255) / 256), a)) return -1;
            RRT(cudaMemcpy(&work, d_work, 1, cudaMemcpyDeviceToHost));
            ++rounds;
        }
    }
    RRT(cudaDeviceSynchronize());
    RRT(cudaMemcpy(ids, d_ids, N, cudaMemcpyDeviceToHost));
    RRT(cudaMemcpy(labels_out, d_labels, N * 4, cudaMemcpyDeviceToHost));
    RRT(cudaMemcpy(pl.data(), d_plates, pl.size() * sizeof(RPlate), cudaMemcpyDeviceToHost));
    for (int k = 0; k < 255; ++k) markers_out[k] = pl[k].velocity;
    *rounds_out = rounds;
    *unassigned_out = remaining;
    return 0;
}

}  // namespace

extern "C" {

const char *refgpu_relabel_error(void) { return g_rerr.c_str(); }

// The relabel of plate ids `ids` (W x H, updated in place) with plate sizes plate_sizes[255] (the
// PlateData sizes that mark free ids) and the kernel settings ks (minPlateSize).  labels_out gets
// the reference's CCL labels, markers_out[k] the index of the plate record slot k holds afterwards,
// rounds_out the fill passes run, unassigned_out the cells postCClIdReassign left without an id.
int refgpu_relabel(const char *cubin_path, int W, int H, uint8_t *ids, const int *plate_sizes,
                   const tecto_kernel_settings *ks, uint32_t *labels_out, float *markers_out, int max_rounds,
                   int *rounds_out, int *unassigned_out)
{
    if (W < 1 || H < 1 || ((size_t)W * (size_t)H) % 256 != 0)
        return rfail("the reference kernels need W * H to be a multiple of 256");
    if (!g_rmod) {
        RRT(cudaFree(nullptr));  // the runtime's primary context becomes current
        RDRV(cuModuleLoad(&g_rmod, cubin_path));
        for (int k = 0; k < NR; ++k) RDRV(cuModuleGetFunction(&g_rfn[k], g_rmod, kRelabelNames[k]));
        size_t bytes = 0;
        RDRV(cuModuleGetGlobal(&g_rsettings, &bytes, g_rmod, "kernelSettings"));
        if (bytes != sizeof(tecto_kernel_settings)) return rfail("kernelSettings size differs from tecto_kernel_settings");
    }
    RDRV(cuMemcpyHtoD(g_rsettings, ks, sizeof(tecto_kernel_settings)));
    return run(W, H, ids, plate_sizes, labels_out, markers_out, max_rounds, rounds_out, unassigned_out);
}

}  // extern "C"
