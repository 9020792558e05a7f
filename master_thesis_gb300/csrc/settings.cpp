// settings.cpp - reference defaults, the synthetic benchmark parameterisation and a config.json
// reader for tecto_settings.  Host code only.
#include <cctype>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/tecto.h"

namespace tecto {
void set_error(const std::string &msg);
}

extern "C" int tecto_settings_default(tecto_settings *out)
{
    if (!out) return TECTO_ERR_INVALID;
    std::memset(out, 0, sizeof(*out));
    tecto_kernel_settings &k = out->kernel;
    // KernelSettings initialisers, src/cuda_compute/kernel_settings.cuh:6-71
    k.inelasticCollisionMultiplierContinental = 1.f;
    k.inelasticCollisionMultiplierSubduction = 0.25f;
    k.inelasticCollisionMultiplierAccretion = 0.5f;
    k.frictionCoefficientContinental = 1.f;
    k.frictionCoefficientSubduction = 0.2f;
    k.frictionCoefficientAccretion = 0.5f;
    k.environmentalDragCoefficient = 0.25f;
    k.velocitySmoothingFactor = 0.9f;
    k.directionSmoothingFactor = 0.9f;
    k.breakScoreSmoothingFactor = 0.9f;
    k.mergeDotDirectionThreshold = .998f;
    k.mergeVelocityDiffThreshold = 0.01f;
    k.mergeMinVelocity = 0.05f;
    k.mergeWaitAfterSplit = 10;
    k.minPlateSize = 10;
    k.continentalCrustThreshold = 10000.f;
    k.divergence_height_target_min = 1000.f;
    k.divergence_height_target_max = 2000.f;
    k.divergence_interpolation_factor = 0.025f;
    k.collisionTypeUpdateCooldown = 4;
    k.minCollisionSize = 50;
    k.subductionOverUpliftMultiplier = 0.005f;
    k.subductionUnderUpliftMultiplier = 0.01f;
    k.continentalUpliftMultiplier = 0.01f;
    k.minUpliftClamp = 0.f;
    k.maxUpliftClamp = 20000.f;
    k.upliftRange = 50;
    k.subductionOverRange = 20;
    k.continentalPropMaxIters = 50;
    k.continentalPropThreshold = 13000;
    k.hydrationPipeCrossSection = 1000;
    k.hydrationPipeLength = 1000;
    k.hydrationRainfall = (float)0.101;
    k.hydrationEvaporation = (float)0.303;
    k.gravity = (float)9.81;
    k.sedimentCapacity = (float)0.9;
    k.sedimentErosionRate = (float)0.5;
    k.sedimentDepositionRate = (float)0.01;
    k.pressureAccumulation = 0.02f;
    k.pressureDecayRate = 0.8f;
    k.pressureBlurRange = 25;
    k.pressureMultiplier = 1.0f;
    k.curlNoiseMultiplier = 30.f;
    k.stressSplitThreshold = 30.0f;
    k.targetMinimumPlateArea = 100;
    k.targetMaximumPlateArea = 100000;
    k.thermalErosionStrength = 1.0f;
    k.thermalErosionAmplitude = 0.5f;
    k.thermalCellSize = 1000.0f;
    k.thermalThresholdAngle = 0.5f;
    // SimulationSettings initialisers, src/generation_settings.h:69-72
    out->sim.numStartingPlates = 16;
    out->sim.seed = 1000;
    out->sim.numVoronoiSeeds[0] = 200;
    out->sim.numVoronoiSeeds[1] = 500;
    out->sim.numVoronoiGenerations = 2;
    out->sim.iterationsForCCL = 10;
    // literal step constants of plate_tectonic_sim.cu:73, :336-363; CCL of ccl.cu
    out->step.hydraulicIterations = 10;
    out->step.hydraulicDt = 1.0f;
    out->step.thermalIterations = 1;
    out->step.upliftMode = TECTO_UPLIFT_GAUSSIAN;
    out->step.upliftAmount = 0.01f;
    out->step.upliftSigma = 1.5f;
    out->step.upliftRadius = 3;
    out->step.cclConnectivity = TECTO_CCL_REF8;
    out->step.sortRadixBits = 0;
    return TECTO_OK;
}

extern "C" int tecto_settings_baseline(tecto_settings *out)
{
    const int rc = tecto_settings_default(out);
    if (rc != TECTO_OK) return rc;
    tecto_kernel_settings &k = out->kernel;
    k.hydrationRainfall = 0.01f;
    k.hydrationEvaporation = 0.05f;
    k.sedimentCapacity = 0.1f;
    k.sedimentErosionRate = 0.3f;
    k.sedimentDepositionRate = 0.1f;
    k.thermalThresholdAngle = 0.01f;
    k.thermalCellSize = 1.0f;
    k.thermalErosionAmplitude = 0.5f;
    k.thermalErosionStrength = 1.0f;
    k.continentalCrustThreshold = 0.0f;
    out->step.hydraulicIterations = 20;
    out->step.hydraulicDt = 0.02f;
    out->step.thermalIterations = 10;
    out->step.upliftMode = TECTO_UPLIFT_GAUSSIAN;
    out->step.upliftAmount = 0.01f;
    out->step.upliftSigma = 1.5f;
    out->step.upliftRadius = 3;
    out->step.cclConnectivity = TECTO_CCL_4;
    out->sim.iterationsForCCL = 10;
    return TECTO_OK;
}

// ---- minimal JSON reader: objects, numbers, booleans, strings (skipped), arrays of numbers ----

namespace {

struct Field {
    const char *name;
    char type;  // 'f' float, 'i' int, 'u' uint32
    size_t offset;
};

#define KF(n) {#n, 'f', offsetof(tecto_kernel_settings, n)}
#define KI(n) {#n, 'i', offsetof(tecto_kernel_settings, n)}
const Field kKernelFields[] = {
    KF(inelasticCollisionMultiplierContinental), KF(inelasticCollisionMultiplierSubduction),
    KF(inelasticCollisionMultiplierAccretion), KF(frictionCoefficientContinental),
    KF(frictionCoefficientSubduction), KF(frictionCoefficientAccretion),
    KF(environmentalDragCoefficient), KF(velocitySmoothingFactor), KF(directionSmoothingFactor),
    KF(breakScoreSmoothingFactor), KF(mergeDotDirectionThreshold), KF(mergeVelocityDiffThreshold),
    KF(mergeMinVelocity), KI(mergeWaitAfterSplit), KI(minPlateSize), KF(continentalCrustThreshold),
    KF(divergence_height_target_min), KF(divergence_height_target_max),
    KF(divergence_interpolation_factor), KI(collisionTypeUpdateCooldown), KI(minCollisionSize),
    KF(subductionOverUpliftMultiplier), KF(subductionUnderUpliftMultiplier),
    KF(continentalUpliftMultiplier), KF(minUpliftClamp), KF(maxUpliftClamp), KI(upliftRange),
    KI(subductionOverRange), KI(continentalPropMaxIters), KF(continentalPropThreshold),
    KF(hydrationPipeCrossSection), KF(hydrationPipeLength), KF(hydrationRainfall),
    KF(hydrationEvaporation), KF(gravity), KF(sedimentCapacity), KF(sedimentErosionRate),
    KF(sedimentDepositionRate), KF(pressureAccumulation), KF(pressureDecayRate),
    KI(pressureBlurRange), KF(pressureMultiplier), KF(curlNoiseMultiplier),
    KF(stressSplitThreshold), KI(targetMinimumPlateArea), KI(targetMaximumPlateArea),
    KF(thermalErosionStrength), KF(thermalErosionAmplitude), KF(thermalCellSize),
    KF(thermalThresholdAngle)};
#undef KF
#undef KI
#define SF(n) {#n, 'f', offsetof(tecto_step_settings, n)}
#define SI(n) {#n, 'i', offsetof(tecto_step_settings, n)}
const Field kStepFields[] = {SI(hydraulicIterations), SF(hydraulicDt), SI(thermalIterations),
                             SI(upliftMode), SF(upliftAmount), SF(upliftSigma), SI(upliftRadius),
                             SI(cclConnectivity), SI(sortRadixBits), SI(hydraulicTile), SI(thermalTile),
                             SI(plateDynamics), SI(platePolicy)};
#undef SF
#undef SI
const Field kSimFields[] = {{"numStartingPlates", 'i', offsetof(tecto_simulation_settings, numStartingPlates)},
                            {"seed", 'u', offsetof(tecto_simulation_settings, seed)},
                            {"iterationsForCCL", 'i', offsetof(tecto_simulation_settings, iterationsForCCL)}};

struct Parser {
    const char *p;
    std::string err;
    void ws()
    {
        while (*p && std::isspace((unsigned char)*p)) ++p;
    }
    bool expect(char c)
    {
        ws();
        if (*p != c) {
            err = std::string("expected '") + c + "'";
            return false;
        }
        ++p;
        return true;
    }
    bool string(std::string *out)
    {
        ws();
        if (*p != '"') {
            err = "expected string";
            return false;
        }
        ++p;
        std::string s;
        while (*p && *p != '"') {
            if (*p == '\\' && p[1]) ++p;
            s.push_back(*p++);
        }
        if (*p != '"') {
            err = "unterminated string";
            return false;
        }
        ++p;
        if (out) *out = s;
        return true;
    }
    bool number(double *out)
    {
        ws();
        if (std::strncmp(p, "true", 4) == 0) { *out = 1; p += 4; return true; }
        if (std::strncmp(p, "false", 5) == 0) { *out = 0; p += 5; return true; }
        char *end = nullptr;
        const double v = std::strtod(p, &end);
        if (end == p) {
            err = "expected number";
            return false;
        }
        p = end;
        *out = v;
        return true;
    }
    bool skip_value()
    {
        ws();
        if (*p == '"') return string(nullptr);
        if (*p == '{') {
            ++p;
            ws();
            if (*p == '}') { ++p; return true; }
            while (true) {
                if (!string(nullptr) || !expect(':') || !skip_value()) return false;
                ws();
                if (*p == ',') { ++p; continue; }
                return expect('}');
            }
        }
        if (*p == '[') {
            ++p;
            ws();
            if (*p == ']') { ++p; return true; }
            while (true) {
                if (!skip_value()) return false;
                ws();
                if (*p == ',') { ++p; continue; }
                return expect(']');
            }
        }
        if (std::strncmp(p, "null", 4) == 0) { p += 4; return true; }
        double d;
        return number(&d);
    }
    template <size_t N>
    bool fields(const Field (&tab)[N], void *base)
    {
        if (!expect('{')) return false;
        ws();
        if (*p == '}') { ++p; return true; }
        while (true) {
            std::string key;
            if (!string(&key) || !expect(':')) return false;
            const Field *f = nullptr;
            for (const Field &c : tab)
                if (key == c.name) f = &c;
            if (f) {
                double v;
                if (!number(&v)) return false;
                char *dst = (char *)base + f->offset;
                if (f->type == 'f') *(float *)dst = (float)v;
                else if (f->type == 'i') *(int *)dst = (int)v;
                else *(uint32_t *)dst = (uint32_t)v;
            } else if (!skip_value()) {
                return false;
            }
            ws();
            if (*p == ',') { ++p; continue; }
            return expect('}');
        }
    }
};

}  // namespace

extern "C" int tecto_settings_from_json(const char *text, tecto_settings *inout, int *width,
                                        int *height)
{
    if (!text || !inout) return TECTO_ERR_INVALID;
    Parser ps{text, {}};
    tecto_settings s = *inout;
    if (!ps.expect('{')) goto fail;
    ps.ws();
    if (*ps.p == '}') return TECTO_OK;
    while (true) {
        std::string key;
        if (!ps.string(&key) || !ps.expect(':')) goto fail;
        if (key == "heightmap_dimensions") {  // src/config.h:29
            if (!ps.expect('{')) goto fail;
            while (true) {
                std::string k2;
                double v;
                if (!ps.string(&k2) || !ps.expect(':') || !ps.number(&v)) goto fail;
                if (k2 == "x" && width) *width = (int)v;
                if (k2 == "y" && height) *height = (int)v;
                ps.ws();
                if (*ps.p == ',') { ++ps.p; continue; }
                if (!ps.expect('}')) goto fail;
                break;
            }
        } else if (key == "kernel_settings") {
            if (!ps.fields(kKernelFields, &s.kernel)) goto fail;
        } else if (key == "simulation_settings") {
            ps.ws();
            // numVoronoiSeeds is an array; handle it inline
            if (!ps.expect('{')) goto fail;
            ps.ws();
            if (*ps.p != '}') {
                while (true) {
                    std::string k2;
                    if (!ps.string(&k2) || !ps.expect(':')) goto fail;
                    if (k2 == "numVoronoiSeeds") {
                        if (!ps.expect('[')) goto fail;
                        int n = 0;
                        ps.ws();
                        if (*ps.p == ']') {
                            ++ps.p;
                        } else {
                            while (true) {
                                double v;
                                if (!ps.number(&v)) goto fail;
                                if (n < TECTO_MAX_VORONOI_GENS) s.sim.numVoronoiSeeds[n++] = (int)v;
                                ps.ws();
                                if (*ps.p == ',') { ++ps.p; continue; }
                                if (!ps.expect(']')) goto fail;
                                break;
                            }
                        }
                        s.sim.numVoronoiGenerations = n;
                    } else {
                        const Field *f = nullptr;
                        for (const Field &c : kSimFields)
                            if (k2 == c.name) f = &c;
                        double v;
                        if (f) {
                            if (!ps.number(&v)) goto fail;
                            char *dst = (char *)&s.sim + f->offset;
                            if (f->type == 'u') *(uint32_t *)dst = (uint32_t)v;
                            else *(int *)dst = (int)v;
                        } else if (!ps.skip_value()) {
                            goto fail;
                        }
                    }
                    ps.ws();
                    if (*ps.p == ',') { ++ps.p; continue; }
                    if (!ps.expect('}')) goto fail;
                    break;
                }
            } else {
                ++ps.p;
            }
        } else if (key == "step_settings") {
            if (!ps.fields(kStepFields, &s.step)) goto fail;
        } else {
            if (!ps.skip_value()) goto fail;  // use_renderer and unknown keys
        }
        ps.ws();
        if (*ps.p == ',') { ++ps.p; continue; }
        if (!ps.expect('}')) goto fail;
        break;
    }
    *inout = s;
    return TECTO_OK;
fail:
    tecto::set_error("tecto_settings_from_json: " + ps.err);
    return TECTO_ERR_INVALID;
}
