/*
 * ref_harness.cpp - runs the reference's own hot-path kernels (MarWo22/master_thesis,
 * src/cuda_compute/, compiled for the CPU through refshim/shim.h by oracle/Makefile) on host
 * arrays.  TEST INFRASTRUCTURE ONLY: it produces the golden vectors under tests/golden/ that pin
 * the C oracle.  Each kernel launch is emulated sequentially, threads in ascending global index.
 *
 * Launch shapes follow the reference: pixel kernels over W*H threads in blocks of 256
 * (plate_tectonic_sim.h:15); the six unguarded hydraulic kernels need W*H % 256 == 0, which the
 * entry points check.
 */
#include <cstdint>
#include <cstring>
#include <utility>
#include <vector>

#include "plate_tectonics_kernel.cuh"
#include "ccl.cuh"
#include "kernel_settings.cuh"
#include "plate_tectonic_sim.h"
#include "../include/tecto.h"

/* the two conversion kernels of the reference's image export (texture_save.cu:10-97, compiled by
 * oracle/Makefile from the lines where they lie) */
namespace texture_save_detail {
void convertGrayscaleToRgbKernel(const CudaTexture<uint8_t> *r_texture, uint8_t *w_texture);
void convertFloatToGray16Kernel(const CudaTexture<float> *r_texture, uint16_t *w_texture, float minVal,
                                float maxVal);
}  // namespace texture_save_detail

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;
/* storage behind the one dynamically sized shared array in the kernel file (findPlausibleSplitLine,
 * plate_tectonics_kernel.cu:2242, off the hot path and never launched here) */
float w_l_buffer[1];

static_assert(sizeof(KernelSettings) == sizeof(tecto_kernel_settings),
              "tecto_kernel_settings must mirror KernelSettings");

namespace {

constexpr unsigned TPB = 256;

template <class F>
void launch(unsigned blocks, unsigned threads, F &&f)
{
    gridDim.x = blocks;
    blockDim.x = threads;
    for (unsigned b = 0; b < blocks; ++b)
        for (unsigned t = 0; t < threads; ++t) {
            blockIdx.x = b;
            threadIdx.x = t;
            f();
        }
}

unsigned blocks_for(size_t n) { return (unsigned)((n + TPB - 1) / TPB); }

std::vector<PlateData> make_plates(const tecto_plate *p)
{
    std::vector<PlateData> out(MAX_PLATE_COUNT);
    for (unsigned k = 0; k < MAX_PLATE_COUNT; ++k) {
        out[k].velocity = p[k].velocity;
        out[k].direction = Vec2<float>(p[k].direction_x, p[k].direction_y);
        out[k].pixelCenter = Vec2<float>(p[k].pixelCenter_x, p[k].pixelCenter_y);
        out[k].mass = 1.0f;
    }
    return out;
}

} // namespace

extern "C" {

void ref_set_settings(const tecto_kernel_settings *ks)
{
    std::memcpy(&kernelSettingsHost, ks, sizeof(KernelSettings));
    copyHostKernelSettingsToDevice();
}

/* getPixelMovements (plate_tectonics_kernel.cu:232-271) */
void ref_pixel_movements(int W, int H, const uint8_t *id, const tecto_plate *plates, uint32_t *dest)
{
    std::vector<uint8_t> idc(id, id + (size_t)W * H), idcopy((size_t)W * H);
    auto pd = make_plates(plates);
    CudaTexture<uint8_t> tId(idc.data(), Vec2<int>(W, H)), tIdOut(idcopy.data(), Vec2<int>(W, H));
    CudaTexture<unsigned int> tDest(dest, Vec2<int>(W, H));
    launch(blocks_for((size_t)W * H), TPB,
           [&] { getPixelMovements(&tId, pd.data(), &tDest, &tIdOut); });
}

/* registerPlateCollisions (plate_tectonics_kernel.cu:273-298) */
void ref_register_collisions(int W, int H, const uint8_t *id, const uint32_t *dest, uint32_t *word)
{
    const size_t N = (size_t)W * H;
    std::vector<uint8_t> idc(id, id + N);
    std::vector<unsigned int> destc(dest, dest + N);
    std::vector<int> counts(N, 0);
    std::memset(word, 0, N * sizeof(uint32_t));
    CudaTexture<uint8_t> tId(idc.data(), Vec2<int>(W, H));
    CudaTexture<unsigned int> tDest(destc.data(), Vec2<int>(W, H));
    CudaTexture<int> tCnt(counts.data(), Vec2<int>(W, H));
    CudaTexture<uint32_t> tWord(word, Vec2<int>(W, H));
    launch(blocks_for(N), TPB, [&] { registerPlateCollisions(&tId, &tDest, &tCnt, &tWord); });
}

/* determineCollisionType kernel + createCollisionTypeMatrix (plate_tectonic_sim.cu:232-241) */
void ref_collision_types(int W, int H, const uint8_t *id_old, const float *h_old, const uint32_t *word,
                         const tecto_plate *plates, uint8_t *type_bitmap)
{
    const size_t N = (size_t)W * H;
    std::vector<uint8_t> idc(id_old, id_old + N);
    std::vector<float> hc(h_old, h_old + N);
    std::vector<uint32_t> wc(word, word + N);
    auto pd = make_plates(plates);
    std::vector<CollisionTypeCounts> counts(MAX_PLATE_COUNT * MAX_PLATE_COUNT);
    std::memset(counts.data(), 0, counts.size() * sizeof(CollisionTypeCounts));
    CudaTexture<uint8_t> tId(idc.data(), Vec2<int>(W, H));
    CudaTexture<float> tH(hc.data(), Vec2<int>(W, H));
    CudaTexture<uint32_t> tWord(wc.data(), Vec2<int>(W, H));
    const PlateTexturesRead rd = {&tId, &tH, pd.data()};
    launch(blocks_for(N), TPB, [&] { determineCollisionType(rd, &tWord, type_bitmap, counts.data()); });
    launch(NUM_BLOCKS_TRIANGLE_ENTRIES, TPB,
           [&] { createCollisionTypeMatrix(counts.data(), type_bitmap); });
}

/* processCollisions + flipDivergedBitmap (plate_tectonic_sim.cu:246-262) */
void ref_process_collisions(int W, int H, const uint8_t *id_old, const float *h_old,
                            const uint32_t *word, const tecto_plate *plates,
                            const uint8_t *type_bitmap, uint32_t *div_bitmap, int seed,
                            unsigned iteration, float *h_new, uint8_t *id_new, uint8_t *acc,
                            float *uplift_height, uint8_t *uplift_types)
{
    const size_t N = (size_t)W * H;
    std::vector<uint8_t> idc(id_old, id_old + N);
    std::vector<float> hc(h_old, h_old + N);
    std::vector<uint32_t> wc(word, word + N);
    std::vector<uint8_t> bm(type_bitmap, type_bitmap + NUM_TRIANGLE_ENTRIES);
    auto pd = make_plates(plates);
    std::vector<uint32_t> hasDiv(NUM_WORDS_TRIANGLE_SINGLE_BITS, 0);
    std::vector<UpliftData> up(N);
    std::vector<CollisionVelocityChanges> vchg(MAX_PLATE_COUNT);
    std::memset(acc, 0, N);
    CudaTexture<uint8_t> tId(idc.data(), Vec2<int>(W, H)), tIdNew(id_new, Vec2<int>(W, H)),
        tAcc(acc, Vec2<int>(W, H));
    CudaTexture<float> tH(hc.data(), Vec2<int>(W, H)), tHNew(h_new, Vec2<int>(W, H));
    CudaTexture<uint32_t> tWord(wc.data(), Vec2<int>(W, H));
    CudaTexture<UpliftData> tUp(up.data(), Vec2<int>(W, H));
    const PlateTexturesRead rd = {&tId, &tH, pd.data()};
    const PlateTexturesWrite wr = {&tIdNew, &tHNew};
    const NoiseParameters np = {seed, iteration};
    launch(blocks_for(N), TPB, [&] {
        processCollisions(rd, &tWord, div_bitmap, bm.data(), wr, hasDiv.data(), &tUp, &tAcc,
                          vchg.data(), np);
    });
    launch(NUM_BLOCKS_TRIANGLE_SINGLE_BITS, TPB,
           [&] { flipDivergedBitmap(div_bitmap, hasDiv.data()); });
    for (size_t i = 0; i < N; ++i) {
        if (uplift_height) uplift_height[i] = up[i].cumulativeHeight;
        if (uplift_types) uplift_types[i] = up[i].collisionTypes;
    }
}

/* The reference uplift (plate_tectonic_sim.cu:270-317): moveContinentalCollisions,
 * combinePropagatedCollisions, JFAInitialize, JFAPass from the largest power of two below
 * max(W, H) down to 1, JFAComputeDistance, applyUplift.  word / up_h / up_t: this step's arrival
 * words and processConvergence records; h_old: heights before the step; plates: plate records
 * before their centre update; h_new updated in place.  The plate table gets a 256th, all-zero
 * record: applyUplift can name plate 255 when merged type bits point at an empty slot, which reads
 * past the reference's 255-entry table. */
void ref_uplift(int W, int H, const uint32_t *word, const float *up_h, const uint8_t *up_t,
                const float *h_old, const tecto_plate *plates, const uint8_t *id_new, float *h_new,
                int32_t *jfa_seed, int32_t *jfa_dist)
{
    const size_t N = (size_t)W * H;
    std::vector<UpliftData> up(N);
    for (size_t i = 0; i < N; ++i) up[i] = UpliftData(up_h[i], up_t[i]);
    std::vector<uint32_t> wc(word, word + N);
    std::vector<float> hc(h_old, h_old + N);
    std::vector<uint8_t> idc(id_new, id_new + N);
    std::vector<PropagatedUpliftData> prop(N);
    std::vector<PlateData> pd = make_plates(plates);
    pd.resize(MAX_PLATE_COUNT + 1);
    pd[MAX_PLATE_COUNT].direction = Vec2<float>(0.0f, 0.0f);
    pd[MAX_PLATE_COUNT].pixelCenter = Vec2<float>(0.0f, 0.0f);
    pd[MAX_PLATE_COUNT].velocity = 0.0f;
    CudaTexture<UpliftData> tUp(up.data(), Vec2<int>(W, H));
    CudaTexture<uint32_t> tWord(wc.data(), Vec2<int>(W, H));
    CudaTexture<float> tH(hc.data(), Vec2<int>(W, H)), tHNew(h_new, Vec2<int>(W, H));
    CudaTexture<PropagatedUpliftData> tProp(prop.data(), Vec2<int>(W, H));
    CudaTexture<uint8_t> tId(idc.data(), Vec2<int>(W, H));
    launch(blocks_for(N), TPB, [&] { moveContinentalCollisions(&tUp, &tWord, &tH, &tProp, pd.data()); });
    launch(blocks_for(N), TPB, [&] { combinePropagatedCollisions(&tUp, &tWord, &tProp); });
    std::vector<int> ja(N), jb(N);
    CudaTexture<int> tA(ja.data(), Vec2<int>(W, H)), tB(jb.data(), Vec2<int>(W, H));
    launch(blocks_for(N), TPB, [&] { JFAInitialize(&tProp, &tA); });
    const int maxDim = W > H ? W : H;
    int step = 1;
    while (step < maxDim) step <<= 1;
    step >>= 1;
    CudaTexture<int> *a = &tA, *b = &tB;
    while (step > 0) {
        launch(blocks_for(N), TPB, [&] { JFAPass(a, b, step); });
        std::swap(a, b);
        step >>= 1;
    }
    std::vector<DistanceFieldBuffer> dfb(N);
    CudaTexture<DistanceFieldBuffer> tD(dfb.data(), Vec2<int>(W, H));
    launch(blocks_for(N), TPB, [&] { JFAComputeDistance(a, &tD); });
    launch(blocks_for(N), TPB, [&] { applyUplift(&tId, &tProp, &tD, pd.data(), &tHNew); });
    for (size_t i = 0; i < N; ++i) {
        if (jfa_seed) jfa_seed[i] = (*a)[Vec2<int>((int)(i % W), (int)(i / W))];
        if (jfa_dist) jfa_dist[i] = dfb[i].dist;
    }
}

/* thermalErosionKernel (plate_tectonics_kernel.cu:2735-2786), one launch, in place */
void ref_thermal(int W, int H, float *h)
{
    CudaTexture<float> tH(h, Vec2<int>(W, H));
    launch(blocks_for((size_t)W * H), TPB, [&] { thermalErosionKernel(&tH); });
}

/* applyHydraulicErosion's loop body (plate_tectonic_sim.cu:336-371), `iters` times */
int ref_hydraulic(int W, int H, float *h, float *w, float *s, float *flux, int iters, float dt,
                  unsigned rain_seed)
{
    const size_t N = (size_t)W * H;
    if (N % TPB != 0) return -1;
    std::vector<float4> f(N), fbuf(N);
    std::memcpy(f.data(), flux, N * sizeof(float4));
    std::vector<float> hcopy(N), sbuf(N);
    std::vector<Vec2<float>> vel(N);
    CudaTexture<float> tH(h, Vec2<int>(W, H)), tW(w, Vec2<int>(W, H)), tS(s, Vec2<int>(W, H)),
        tHc(hcopy.data(), Vec2<int>(W, H)), tSb(sbuf.data(), Vec2<int>(W, H));
    CudaTexture<float4> tF(f.data(), Vec2<int>(W, H)), tFb(fbuf.data(), Vec2<int>(W, H));
    CudaTexture<Vec2<float>> tV(vel.data(), Vec2<int>(W, H));
    const unsigned nb = (unsigned)(N / TPB);
    for (int i = 0; i < iters; ++i) {
        launch(nb, TPB, [&] { rain(&tW, dt, rain_seed); });
        launch(nb, TPB, [&] { ::flux(&tH, &tW, &tF, &tFb, dt); });
        launch(nb, TPB, [&] { flow(&tW, &tFb, &tF, &tV, dt); });
        std::memcpy(hcopy.data(), h, N * sizeof(float));
        launch(nb, TPB, [&] { sediment(&tHc, &tH, &tS, &tV, dt); });
        launch(nb, TPB, [&] { transport(&tS, &tSb, &tV, dt); });
        launch(nb, TPB, [&] { evaporate(&tW, dt); });
        std::memcpy(s, sbuf.data(), N * sizeof(float));
    }
    std::memcpy(flux, f.data(), N * sizeof(float4));
    return 0;
}

/* applyAccretion (plate_tectonics_kernel.cu:747-770), in place on id */
void ref_accretion(int W, int H, const float *h, const uint8_t *acc, uint8_t *id)
{
    const size_t N = (size_t)W * H;
    std::vector<float> hc(h, h + N);
    std::vector<uint8_t> ac(acc, acc + N);
    CudaTexture<float> tH(hc.data(), Vec2<int>(W, H));
    CudaTexture<uint8_t> tAcc(ac.data(), Vec2<int>(W, H)), tId(id, Vec2<int>(W, H));
    launch(blocks_for(N), TPB, [&] { applyAccretion(&tH, &tAcc, &tId); });
}

/* applyCCL's labelling kernels (plate_tectonic_sim.cu:380-389, ccl.cu:90-177) */
void ref_ccl(int W, int H, const uint8_t *id, uint32_t *labels)
{
    const size_t N = (size_t)W * H;
    std::vector<uint8_t> idc(id, id + N);
    CudaTexture<uint8_t> tId(idc.data(), Vec2<int>(W, H));
    CudaTexture<unsigned int> tL(labels, Vec2<int>(W, H));
    launch(blocks_for(N), TPB, [&] { init(&tId, &tL); });
    launch(blocks_for(N), TPB, [&] { analyzeClamped(&tL); });
    launch(blocks_for(N), TPB, [&] { reduce(&tId, &tL); });
    launch(blocks_for(N), TPB, [&] { analyzeUnclamped(&tL); });
}

/* convertFloatToGray16Kernel over a W x H height map (texture_save.cu:80-96). */
void ref_gray16(int W, int H, const float *h, float minv, float maxv, uint16_t *out)
{
    const size_t N = (size_t)W * H;
    std::vector<float> hc(h, h + N);
    CudaTexture<float> t(hc.data(), Vec2<int>(W, H));
    launch(blocks_for(N), TPB, [&] { texture_save_detail::convertFloatToGray16Kernel(&t, out, minv, maxv); });
}

/* convertGrayscaleToRgbKernel over a W x H plate-id map (texture_save.cu:10-78), every cell
 * (the reference's own launch, texture_save.cu:237, covers (W*H + 1) / 256 whole blocks only). */
void ref_ids_rgb(int W, int H, const uint8_t *ids, uint8_t *out)
{
    const size_t N = (size_t)W * H;
    std::vector<uint8_t> ic(ids, ids + N);
    CudaTexture<uint8_t> t(ic.data(), Vec2<int>(W, H));
    launch(blocks_for(N), TPB, [&] { texture_save_detail::convertGrayscaleToRgbKernel(&t, out); });
}

/* Plate dynamics, the reference's kernels on host arrays. */

/* processCollisions' CollisionVelocityChanges::frictionLoss per plate, with plate masses mass[255]
 * (plate_tectonics_kernel.cu:371-466); the other outputs of the step are discarded. */
void ref_collision_friction(int W, int H, const uint8_t *id_old, const float *h_old, const uint32_t *word,
                            const tecto_plate *plates, const float *mass, const uint8_t *type_bitmap,
                            const uint32_t *div_bitmap, int seed, unsigned iteration, float *friction)
{
    const size_t N = (size_t)W * H;
    std::vector<uint8_t> idc(id_old, id_old + N), idn(N), acc(N);
    std::vector<float> hc(h_old, h_old + N), hn(N);
    std::vector<uint32_t> wc(word, word + N), div(div_bitmap, div_bitmap + NUM_WORDS_TRIANGLE_SINGLE_BITS);
    std::vector<uint8_t> bm(type_bitmap, type_bitmap + NUM_TRIANGLE_ENTRIES);
    auto pd = make_plates(plates);
    for (unsigned k = 0; k < MAX_PLATE_COUNT; ++k) pd[k].mass = mass[k];
    std::vector<uint32_t> hasDiv(NUM_WORDS_TRIANGLE_SINGLE_BITS, 0);
    std::vector<UpliftData> up(N);
    std::vector<CollisionVelocityChanges> vchg(MAX_PLATE_COUNT);
    CudaTexture<uint8_t> tId(idc.data(), Vec2<int>(W, H)), tIdNew(idn.data(), Vec2<int>(W, H)),
        tAcc(acc.data(), Vec2<int>(W, H));
    CudaTexture<float> tH(hc.data(), Vec2<int>(W, H)), tHNew(hn.data(), Vec2<int>(W, H));
    CudaTexture<uint32_t> tWord(wc.data(), Vec2<int>(W, H));
    CudaTexture<UpliftData> tUp(up.data(), Vec2<int>(W, H));
    const PlateTexturesRead rd = {&tId, &tH, pd.data()};
    const PlateTexturesWrite wr = {&tIdNew, &tHNew};
    const NoiseParameters np = {seed, iteration};
    launch(blocks_for(N), TPB, [&] {
        processCollisions(rd, &tWord, div.data(), bm.data(), wr, hasDiv.data(), &tUp, &tAcc, vchg.data(), np);
    });
    for (unsigned k = 0; k < MAX_PLATE_COUNT; ++k) friction[k] = vchg[k].frictionLoss;
}

/* accumulatePlateAngularCoords + calculatePlateCenters (:2154-2226): centre_xy[2 * plate + axis];
 * plates without samples keep the value passed in. */
void ref_plate_centres(int W, int H, const uint8_t *ids, float *centre_xy)
{
    const size_t N = (size_t)W * H;
    std::vector<uint8_t> ic(ids, ids + N);
    std::vector<float4> sums(MAX_PLATE_COUNT, float4{0, 0, 0, 0});
    std::vector<int> counts(MAX_PLATE_COUNT, 0);
    std::vector<PlateData> pd(MAX_PLATE_COUNT);
    for (unsigned k = 0; k < MAX_PLATE_COUNT; ++k)
        pd[k].geometricCenter = Vec2<float>(centre_xy[2 * k], centre_xy[2 * k + 1]);
    CudaTexture<uint8_t> tId(ic.data(), Vec2<int>(W, H));
    CudaTexture<float4> tSums(sums.data(), Vec2<int>(MAX_PLATE_COUNT, 1));
    CudaTexture<int> tCounts(counts.data(), Vec2<int>(MAX_PLATE_COUNT, 1));
    launch(blocks_for(N), TPB, [&] { accumulatePlateAngularCoords(&tId, &tSums, &tCounts); });
    launch(MAX_PLATE_COUNT, 1, [&] { calculatePlateCenters(&tId, &tSums, &tCounts, pd.data()); });
    for (unsigned k = 0; k < MAX_PLATE_COUNT; ++k) {
        centre_xy[2 * k] = pd[k].geometricCenter.x;
        centre_xy[2 * k + 1] = pd[k].geometricCenter.y;
    }
}

/* computeCurl (:2788-2822): the W x H asthenosphere field (x, y per cell) of a pw x ph pressure
 * texture. */
void ref_curl(int pw, int ph, const float *pressure, int W, int H, float *curl_xy)
{
    std::vector<float> pc(pressure, pressure + (size_t)pw * ph);
    std::vector<Vec2<float>> out((size_t)W * H);
    CudaTexture<float> tP(pc.data(), Vec2<int>(pw, ph));
    CudaTexture<Vec2<float>> tC(out.data(), Vec2<int>(W, H));
    launch(blocks_for((size_t)W * H), TPB, [&] { computeCurl(&tP, &tC); });
    for (size_t i = 0; i < out.size(); ++i) {
        curl_xy[2 * i] = out[i].x;
        curl_xy[2 * i + 1] = out[i].y;
    }
}

/* applyPlateMovementChanges (:1863-1925) over the 255 plates: plates (velocity, direction,
 * pixelCenter) and dyn (velocitySmoothed, directionSmoothed, geometricCenter, mergeWaitTime) are
 * updated in place; friction[255] is CollisionVelocityChanges::frictionLoss; curl_xy the W x H
 * asthenosphere field. */
void ref_plate_motion(int W, int H, tecto_plate *plates, tecto_plate_dynamics *dyn, const float *friction,
                      const float *curl_xy)
{
    auto pd = make_plates(plates);
    std::vector<CollisionVelocityChanges> vchg(MAX_PLATE_COUNT);
    for (unsigned k = 0; k < MAX_PLATE_COUNT; ++k) {
        pd[k].velocitySmoothed = dyn[k].velocitySmoothed;
        pd[k].directionSmoothed = Vec2<float>(dyn[k].directionSmoothed_x, dyn[k].directionSmoothed_y);
        pd[k].geometricCenter = Vec2<float>(dyn[k].geometricCenter_x, dyn[k].geometricCenter_y);
        pd[k].mergeWaitTime = dyn[k].mergeWaitTime;
        vchg[k].frictionLoss = friction[k];
    }
    std::vector<Vec2<float>> curl((size_t)W * H);
    for (size_t i = 0; i < curl.size(); ++i) curl[i] = Vec2<float>(curl_xy[2 * i], curl_xy[2 * i + 1]);
    CudaTexture<Vec2<float>> tC(curl.data(), Vec2<int>(W, H));
    launch(1, 256, [&] { applyPlateMovementChanges(pd.data(), vchg.data(), &tC); });
    for (unsigned k = 0; k < MAX_PLATE_COUNT; ++k) {
        plates[k].velocity = pd[k].velocity;
        plates[k].direction_x = pd[k].direction.x;
        plates[k].direction_y = pd[k].direction.y;
        plates[k].pixelCenter_x = pd[k].pixelCenter.x;
        plates[k].pixelCenter_y = pd[k].pixelCenter.y;
        dyn[k].velocitySmoothed = pd[k].velocitySmoothed;
        dyn[k].directionSmoothed_x = pd[k].directionSmoothed.x;
        dyn[k].directionSmoothed_y = pd[k].directionSmoothed.y;
        dyn[k].mergeWaitTime = pd[k].mergeWaitTime;
    }
}

/* initPlateIDs + initHeightmap (plate_tectonics_kernel.cu:31-99) for the given seeds. */
void ref_init(int W, int H, int seed, const float *sx, const float *sy, const uint8_t *sid, int S, float *h,
              uint8_t *id)
{
    std::vector<VoronoiSeed> seeds((size_t)S);
    for (int k = 0; k < S; ++k) {
        seeds[(size_t)k].position = Vec2<float>(sx[k], sy[k]);
        seeds[(size_t)k].id = sid[k];
    }
    CudaTexture<uint8_t> tId(id, Vec2<int>(W, H));
    CudaTexture<float> tH(h, Vec2<int>(W, H));
    launch(blocks_for((size_t)W * H), TPB, [&] { initPlateIDs(&tId, seeds.data(), S); });
    launch(blocks_for((size_t)W * H), TPB, [&] { initHeightmap(&tH, seed, 4); });
}

/* mergePlates (plate_tectonic_sim.cu:470-494) with the reference's kernels: getNeighboringPlates,
 * getPlateMerges (its threads in ascending order; the device-side launch of clearCollisionTypes is
 * not compiled here, so clearCollisionTypes runs afterwards for each parent), then
 * mergeAndCountSizeMass for the id remap (its per-block sums, which need a real barrier, are
 * discarded).  merge_ids[255] receives getPlateMerges' table. */
void ref_merges(int W, int H, uint8_t *ids, const tecto_plate *plates, const tecto_plate_dynamics *dyn,
                uint8_t *type_bitmap, int *merge_ids)
{
    const size_t N = (size_t)W * H;
    auto pd = make_plates(plates);
    for (unsigned k = 0; k < MAX_PLATE_COUNT; ++k) {
        pd[k].velocitySmoothed = dyn[k].velocitySmoothed;
        pd[k].directionSmoothed = Vec2<float>(dyn[k].directionSmoothed_x, dyn[k].directionSmoothed_y);
        pd[k].mass = dyn[k].mass;
        pd[k].size = dyn[k].size;
        pd[k].mergeWaitTime = dyn[k].mergeWaitTime;
    }
    std::vector<uint8_t> nbm((size_t)MAX_PLATE_COUNT * MAX_PLATE_COUNT, 0);
    bool *nb = reinterpret_cast<bool *>(nbm.data());
    CudaTexture<uint8_t> tId(ids, Vec2<int>(W, H));
    CudaTexture<bool> tNb(nb, Vec2<int>(MAX_PLATE_COUNT, MAX_PLATE_COUNT));
    CudaTexture<uint8_t> tBm(type_bitmap, Vec2<int>(NUM_TRIANGLE_ENTRIES, 1));
    std::memset(merge_ids, 0, sizeof(int) * MAX_PLATE_COUNT);
    launch(blocks_for(N), TPB, [&] { getNeighboringPlates(&tId, &tNb); });
    launch(blocks_for((size_t)MAX_PLATE_COUNT * MAX_PLATE_COUNT), TPB,
           [&] { getPlateMerges(&tNb, pd.data(), merge_ids, &tBm); });
    for (unsigned k = 0; k < MAX_PLATE_COUNT; ++k)
        if (merge_ids[k] == -1) launch(1, TPB, [&] { clearCollisionTypes(tBm, (int)k); });
    std::vector<Vec2<float>> slope(N);
    CudaTexture<Vec2<float>> tSlope(slope.data(), Vec2<int>(W, H));
    std::vector<float> hz(N, 0.0f);
    CudaTexture<float> tH(hz.data(), Vec2<int>(W, H));
    auto scratch = pd;
    launch(blocks_for(N), TPB, [&] { mergeAndCountSizeMass(&tId, &tH, merge_ids, scratch.data(), &tSlope); });
}

} // extern "C"
