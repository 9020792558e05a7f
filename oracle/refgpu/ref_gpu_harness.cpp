// ref_gpu_harness.cpp - MEASUREMENT INFRASTRUCTURE ONLY (the reference arm of bench.py): times the
// reference's own CUDA kernels (MarWo22/master_thesis src/cuda_compute, compiled from the
// reference's sources into oracle/_ref/ref_kernels.cubin by oracle/Makefile's `refgpu` target)
// on this GPU, in the order of PlateTectonicSim::executeIteration (plate_tectonic_sim.cu:54-131)
// with the benchmark physics mapped onto its parameters.  It is loaded with the CUDA driver API
// and launched with the reference's own launch shapes (256 threads per block, one thread per
// cell).  The engine never links it.
//
// Kernels run: getPixelMovements, registerPlateCollisions, determineCollisionType,
// createCollisionTypeMatrix, thermalErosionKernel, the hydraulic chain rain / flux / flow /
// sediment / transport / evaporate with its two device copies per sub-iteration
// (plate_tectonic_sim.cu:331-373), the copies back of copyAndReleaseTexture, applyAccretion, and
// the CCL kernels when due.  processCollisions is not launched: its applyInelasticCollision
// reads past a local array (plate_tectonics_kernel.cu:453); a device copy of the heights stands
// in for its writes.  The uplift kernels are not launched either (the benchmark physics uses the
// Gaussian uplift the reference does not have).
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/tecto.h"

namespace {

// The reference's PlateData (types/plate_data.h), 84 bytes.
struct RefVec2 {
    float x, y;
};
struct RefPlateData {
    float velocity, velocitySmoothed;
    RefVec2 direction, directionSmoothed, pixelCenter, velocityChange, geometricCenter, asthenosphereVelocity;
    int size;
    float mass;
    int perimeter;
    float breakScore, circularity;
    bool used, hasMoved;
    int mergeWaitTime;
};
static_assert(sizeof(RefPlateData) == 84, "PlateData layout");

// CudaTexture<T> (types/cuda_texture.cuh): the element pointer and the size.
struct RefTex {
    void *arr;
    int w, h;
};
static_assert(sizeof(RefTex) == 16, "CudaTexture layout");

struct PlateTexturesRead {
    const RefTex *plateIds;
    const RefTex *heightMap;
    const RefPlateData *plateData;
};

const char *kNames[] = {
    "_Z17getPixelMovementsPK11CudaTextureIhEPK9PlateDataPS_IjEPS0_",
    "_Z23registerPlateCollisionsPK11CudaTextureIhEPKS_IjEPS_IiEPS3_",
    "_Z22determineCollisionType17PlateTexturesReadPK11CudaTextureIjEPKhP19CollisionTypeCounts",
    "_Z25createCollisionTypeMatrixPK19CollisionTypeCountsPh",
    "_Z20thermalErosionKernelP11CudaTextureIfE",
    "_Z4rainP11CudaTextureIfEfj",
    "_Z4fluxPK11CudaTextureIfES2_PKS_I6float4EPS4_f",
    "_Z4flowP11CudaTextureIfEPKS_I6float4EPS3_PS_I4Vec2IfEEf",
    "_Z8sedimentPK11CudaTextureIfEPS0_S3_PS_I4Vec2IfEEf",
    "_Z9transportP11CudaTextureIfES1_PS_I4Vec2IfEEf",
    "_Z9evaporateP11CudaTextureIfEf",
    "_Z14applyAccretionPK11CudaTextureIfEPKS_IhEPS3_",
    "_Z4initPK11CudaTextureIhEPS_IjE",
    "_Z14analyzeClampedP11CudaTextureIjE",
    "_Z6reducePK11CudaTextureIhEPS_IjE",
    "_Z16analyzeUnclampedP11CudaTextureIjE",
};
enum K { PIX, REG, DET, MAT, THERM, RAIN, FLUX, FLOW, SED, TRANS, EVAP, ACC, CINIT, CCLAMP, CRED, CUNCL, NK };

CUmodule g_mod = nullptr;
CUfunction g_fn[NK] = {};
CUdeviceptr g_settings = 0;
std::string g_err;

int fail(const std::string &m)
{
    g_err = m;
    return -1;
}

#define DRV(call)                                                          \
    do {                                                                   \
        CUresult r_ = (call);                                              \
        if (r_ != CUDA_SUCCESS) {                                          \
            const char *s_ = nullptr;                                      \
            cuGetErrorString(r_, &s_);                                     \
            return fail(std::string(#call) + ": " + (s_ ? s_ : "?"));      \
        }                                                                  \
    } while (0)
#define RT(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) return fail(std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int launch(K k, unsigned blocks, void **args, CUstream st)
{
    DRV(cuLaunchKernel(g_fn[k], blocks, 1, 1, 256, 1, 1, 0, st, args, nullptr));
    return 0;
}

}  // namespace

extern "C" {

const char *refgpu_error(void) { return g_err.c_str(); }

// Load the linked cubin (the reference's device code, linked with the device runtime library by
// oracle/Makefile) in the runtime's primary context.
int refgpu_load(const char *cubin_path)
{
    if (g_mod) return 0;
    RT(cudaFree(nullptr));  // the runtime's primary context becomes current
    DRV(cuModuleLoad(&g_mod, cubin_path));
    for (int k = 0; k < NK; ++k) DRV(cuModuleGetFunction(&g_fn[k], g_mod, kNames[k]));
    size_t bytes = 0;
    DRV(cuModuleGetGlobal(&g_settings, &bytes, g_mod, "kernelSettings"));
    if (bytes != sizeof(tecto_kernel_settings)) return fail("kernelSettings size differs from tecto_kernel_settings");
    return 0;
}

// Time `steps` steps (after `warmup`) of the reference kernels on a W x H world (W * H a multiple
// of 256, the reference's unguarded launch shape).  Returns the mean milliseconds per step from
// CUDA events on one stream.
int refgpu_time_steps(int W, int H, const float *h_host, const uint8_t *id_host, const tecto_plate *plates,
                      const tecto_kernel_settings *ks, int hyd_iters, float dt, int thermal_iters, int ccl_period,
                      int steps, int warmup, double *ms_per_step)
{
    if (!g_mod) return fail("refgpu_load first");
    const size_t N = (size_t)W * H;
    if (N == 0 || N % 256 != 0) return fail("the reference kernels need W * H to be a multiple of 256");
    const unsigned blocks = (unsigned)(N / 256);
    DRV(cuMemcpyHtoD(g_settings, ks, sizeof(tecto_kernel_settings)));
    std::vector<RefPlateData> pd(255);
    std::memset(pd.data(), 0, pd.size() * sizeof(RefPlateData));
    for (int k = 0; k < 255; ++k) {
        pd[k].velocity = plates[k].velocity;
        pd[k].direction = {plates[k].direction_x, plates[k].direction_y};
        pd[k].pixelCenter = {plates[k].pixelCenter_x, plates[k].pixelCenter_y};
        pd[k].mass = 1.0f;
        pd[k].breakScore = 1.0f;
    }
    // device buffers
    std::vector<void *> bufs;
    bool oom = false;
    auto dalloc = [&](size_t n) -> void * {
        void *p = nullptr;
        if (cudaMalloc(&p, n) != cudaSuccess) {
            oom = true;
            return nullptr;
        }
        cudaMemset(p, 0, n);
        bufs.push_back(p);
        return p;
    };
    float *hmap = (float *)dalloc(N * 4), *hw = (float *)dalloc(N * 4), *mat = (float *)dalloc(N * 4);
    float *water = (float *)dalloc(N * 4), *sed = (float *)dalloc(N * 4), *sedb = (float *)dalloc(N * 4);
    void *flux = dalloc(N * 16), *fluxb = dalloc(N * 16), *vel = dalloc(N * 8);
    uint8_t *ids = (uint8_t *)dalloc(N), *idsw = (uint8_t *)dalloc(N), *idcopy = (uint8_t *)dalloc(N);
    uint8_t *acc = (uint8_t *)dalloc(N);
    uint32_t *pix = (uint32_t *)dalloc(N * 4), *coll = (uint32_t *)dalloc(N * 4), *labels = (uint32_t *)dalloc(N * 4);
    int *cnt = (int *)dalloc(N * 4);
    uint8_t *bitmap = (uint8_t *)dalloc(32385);
    void *typecounts = dalloc((size_t)255 * 255 * 20);
    RefPlateData *dplates = (RefPlateData *)dalloc(pd.size() * sizeof(RefPlateData));
    RefTex *tex = (RefTex *)dalloc(17 * sizeof(RefTex));
    int rc = oom ? fail("cudaMalloc failed") : 0;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (rc == 0) {
        RefTex host[17] = {{hmap, W, H},  {hw, W, H},   {mat, W, H},  {water, W, H},  {sed, W, H},    {sedb, W, H},
                           {flux, W, H},  {fluxb, W, H}, {vel, W, H},  {ids, W, H},    {idsw, W, H},   {idcopy, W, H},
                           {acc, W, H},   {pix, W, H},   {coll, W, H}, {labels, W, H}, {cnt, W, H}};
        cudaMemcpy(tex, host, sizeof(host), cudaMemcpyHostToDevice);
        cudaMemcpy(hmap, h_host, N * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(ids, id_host, N, cudaMemcpyHostToDevice);
        cudaMemcpy(dplates, pd.data(), pd.size() * sizeof(RefPlateData), cudaMemcpyHostToDevice);
        if (cudaStreamCreate(&st) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
            cudaEventCreate(&e1) != cudaSuccess)
            rc = fail("stream or event creation failed");
    }
    RefTex *tH = tex + 0, *tHW = tex + 1, *tMat = tex + 2, *tWater = tex + 3, *tSed = tex + 4, *tSedB = tex + 5;
    RefTex *tFlux = tex + 6, *tFluxB = tex + 7, *tVel = tex + 8, *tIds = tex + 9, *tIdsW = tex + 10;
    RefTex *tIdCopy = tex + 11, *tAcc = tex + 12, *tPix = tex + 13, *tColl = tex + 14, *tLabels = tex + 15;
    RefTex *tCount = tex + 16;
    const CUstream cst = (CUstream)st;
    unsigned iteration = 0;
    const unsigned seed = 1000;
    auto step = [&]() -> int {
        // getPlateCollisions (plate_tectonic_sim.cu:135-222)
        RT(cudaMemsetAsync(coll, 0, N * 4, st));
        RT(cudaMemsetAsync(cnt, 0, N * 4, st));
        {
            void *a[] = {&tIds, &dplates, &tPix, &tIdCopy};
            if (launch(PIX, blocks, a, cst)) return -1;
        }
        {
            void *a[] = {&tIds, &tPix, &tCount, &tColl};
            if (launch(REG, blocks, a, cst)) return -1;
        }
        // processCollisionUplift up to processCollisions (plate_tectonic_sim.cu:225-262)
        RT(cudaMemsetAsync(typecounts, 0, (size_t)255 * 255 * 20, st));
        {
            PlateTexturesRead rd = {tIds, tH, dplates};
            void *a[] = {&rd, &tColl, &bitmap, &typecounts};
            if (launch(DET, blocks, a, cst)) return -1;
        }
        {
            void *a[] = {&typecounts, &bitmap};
            if (launch(MAT, (32385 + 255) / 256, a, cst)) return -1;
        }
        RT(cudaMemsetAsync(acc, 0, N, st));
        // stands in for processCollisions' writes of the new heights and ids
        RT(cudaMemcpyAsync(hw, hmap, N * 4, cudaMemcpyDeviceToDevice, st));
        RT(cudaMemcpyAsync(idsw, ids, N, cudaMemcpyDeviceToDevice, st));
        // thermal (plate_tectonic_sim.cu:73), once per thermal iteration of the benchmark physics
        for (int i = 0; i < thermal_iters; ++i) {
            void *a[] = {&tHW};
            if (launch(THERM, blocks, a, cst)) return -1;
        }
        // applyHydraulicErosion (plate_tectonic_sim.cu:331-373)
        unsigned rseed = seed + iteration;
        for (int i = 0; i < hyd_iters; ++i) {
            void *ar[] = {&tWater, &dt, &rseed};
            if (launch(RAIN, blocks, ar, cst)) return -1;
            void *af[] = {&tHW, &tWater, &tFlux, &tFluxB, &dt};
            if (launch(FLUX, blocks, af, cst)) return -1;
            void *afl[] = {&tWater, &tFluxB, &tFlux, &tVel, &dt};
            if (launch(FLOW, blocks, afl, cst)) return -1;
            RT(cudaMemcpyAsync(mat, hw, N * 4, cudaMemcpyDeviceToDevice, st));
            void *as[] = {&tMat, &tHW, &tSed, &tVel, &dt};
            if (launch(SED, blocks, as, cst)) return -1;
            void *at[] = {&tSed, &tSedB, &tVel, &dt};
            if (launch(TRANS, blocks, at, cst)) return -1;
            void *ae[] = {&tWater, &dt};
            if (launch(EVAP, blocks, ae, cst)) return -1;
            RT(cudaMemcpyAsync(sed, sedb, N * 4, cudaMemcpyDeviceToDevice, st));
        }
        // copyAndReleaseTexture (plate_tectonic_sim.cu:79-80), applyAccretion, CCL when due
        RT(cudaMemcpyAsync(hmap, hw, N * 4, cudaMemcpyDeviceToDevice, st));
        RT(cudaMemcpyAsync(ids, idsw, N, cudaMemcpyDeviceToDevice, st));
        {
            void *a[] = {&tH, &tAcc, &tIds};
            if (launch(ACC, blocks, a, cst)) return -1;
        }
        if (ccl_period > 0 && iteration % (unsigned)ccl_period == 0) {
            void *ai[] = {&tIds, &tLabels};
            if (launch(CINIT, blocks, ai, cst)) return -1;
            void *ac[] = {&tLabels};
            if (launch(CCLAMP, blocks, ac, cst)) return -1;
            if (launch(CRED, blocks, ai, cst)) return -1;
            if (launch(CUNCL, blocks, ac, cst)) return -1;
        }
        ++iteration;
        return 0;
    };
    for (int i = 0; rc == 0 && i < warmup; ++i) rc = step();
    if (rc == 0 && cudaStreamSynchronize(st) != cudaSuccess) rc = fail("warm-up failed");
    if (rc == 0) {
        cudaEventRecord(e0, st);
        for (int i = 0; rc == 0 && i < steps; ++i) rc = step();
        cudaEventRecord(e1, st);
        if (rc == 0 && cudaEventSynchronize(e1) != cudaSuccess) rc = fail("timed steps failed");
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        *ms_per_step = (double)ms / (double)steps;
    }
    if (st) cudaStreamDestroy(st);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    for (void *p : bufs) cudaFree(p);
    return rc;
}

}  // extern "C"

// ---- the reference's image export (oracle/_ref/ref_export.cubin, texture_save.cu) ----------------

namespace {
CUmodule g_exp = nullptr;
CUfunction g_gray16 = nullptr, g_rgb = nullptr;

// One conversion kernel over n cells: its input texture (RefTex in device memory) and output.
int run_export(CUfunction fn, const void *in_host, size_t in_bytes, int W, int H, void *out_host,
               size_t out_bytes, float minv, float maxv)
{
    void *din = nullptr, *dout = nullptr;
    RefTex *dtex = nullptr;
    int rc = 0;
    if (cudaMalloc(&din, in_bytes) != cudaSuccess || cudaMalloc(&dout, out_bytes) != cudaSuccess ||
        cudaMalloc((void **)&dtex, sizeof(RefTex)) != cudaSuccess)
        rc = fail("cudaMalloc failed");
    if (rc == 0) {
        const RefTex t{din, W, H};
        if (cudaMemcpy(dtex, &t, sizeof(t), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(din, in_host, in_bytes, cudaMemcpyHostToDevice) != cudaSuccess)
            rc = fail("cudaMemcpy failed");
    }
    if (rc == 0) {
        const size_t n = (size_t)W * H;
        const unsigned blocks = (unsigned)((n + 255) / 256);  // the kernels check their bounds
        void *gray_args[] = {&dtex, &dout, &minv, &maxv};
        void *rgb_args[] = {&dtex, &dout};
        const CUresult r = cuLaunchKernel(fn, blocks, 1, 1, 256, 1, 1, 0, nullptr,
                                          fn == g_gray16 ? gray_args : rgb_args, nullptr);
        if (r != CUDA_SUCCESS) rc = fail("cuLaunchKernel failed");
        else if (cudaMemcpy(out_host, dout, out_bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = fail("cudaMemcpy back failed");
    }
    cudaFree(din);
    cudaFree(dout);
    cudaFree(dtex);
    return rc;
}
}  // namespace

extern "C" {

int refgpu_export_load(const char *cubin_path)
{
    if (g_exp) return 0;
    RT(cudaFree(nullptr));
    DRV(cuModuleLoad(&g_exp, cubin_path));
    DRV(cuModuleGetFunction(&g_gray16, g_exp,
                            "_ZN19texture_save_detail26convertFloatToGray16KernelEPK11CudaTextureIfEPtff"));
    DRV(cuModuleGetFunction(&g_rgb, g_exp,
                            "_ZN19texture_save_detail27convertGrayscaleToRgbKernelEPK11CudaTextureIhEPh"));
    return 0;
}

// convertFloatToGray16Kernel over a W x H height map.
int refgpu_gray16(const float *h, int W, int H, float minv, float maxv, uint16_t *out)
{
    if (!g_exp) return fail("refgpu_export_load first");
    const size_t n = (size_t)W * H;
    return run_export(g_gray16, h, n * 4, W, H, out, n * 2, minv, maxv);
}

// convertGrayscaleToRgbKernel over a W x H plate-id map (3 bytes per cell out).
int refgpu_ids_rgb(const uint8_t *ids, int W, int H, uint8_t *out)
{
    if (!g_exp) return fail("refgpu_export_load first");
    const size_t n = (size_t)W * H;
    return run_export(g_rgb, ids, n, W, H, out, n * 3, 0.0f, 0.0f);
}

}  // extern "C"
