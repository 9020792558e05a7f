// noise.cuh - the two noise functions on the hot path, written from their published methods:
//  - rain: cudaNoise's discreteNoise/randomGrid over Robert Jenkins' 32-bit integer hash
//    (src/cuda_compute/cuda_noise.cuh:44-54, :66-71, :108-111, :470-477);
//  - new crust: Gustavson's 3D simplex noise with hashed gradient selection
//    (cuda_noise.cuh:228-320), called by processDivergence (plate_tectonics_kernel.cu:345).
// Evaluated in IEEE single precision, no contraction (the library is built with -fmad=false).
#pragma once

#include <cstdint>

namespace tecto {

__device__ __forceinline__ uint32_t jenkins_hash(uint32_t a)
{
    a = (a + 0x7ed55d16u) + (a << 12);
    a = (a ^ 0xc761c23cu) ^ (a >> 19);
    a = (a + 0x165667b1u) + (a << 5);
    a = (a + 0xd3a2646cu) ^ (a << 9);
    a = (a + 0xfd7046c5u) + (a << 3);
    a = (a ^ 0xb55a4f09u) ^ (a >> 16);
    return a;
}

// discreteNoise(make_float3(x, 0, y), 1, seed): value in [-1, 1] per cell.
__device__ __forceinline__ float rain_noise(int x, int y, int seed)
{
    const int ix = (int)((float)x * 1.0f);
    const int iz = (int)((float)y * 1.0f);
    float v = (float)ix * 1723.0f;
    v = v + 0.0f * 93241.0f;
    v = v + (float)iz * 149812.0f;
    v = v + 3824.0f;
    v = v + (float)seed;
    const uint32_t hv = jenkins_hash(__float2uint_rz(v));  // saturating conversion
    const float r = (float)hv / 4294967296.0f;
    return r * 2.0f - 1.0f;
}

__device__ __forceinline__ float grad_dot(int g, float x, float y, float z)
{
    // Gustavson's twelve gradient directions (1,1,0), (-1,1,0), ... in cuda_noise.cuh:158-160 order
    const float gx = (g < 8) ? ((g & 1) ? -1.0f : 1.0f) : 0.0f;
    const float gy = (g < 4) ? ((g & 2) ? -1.0f : 1.0f) : (g < 8 ? 0.0f : ((g & 1) ? -1.0f : 1.0f));
    const float gz = (g < 4) ? 0.0f : (g < 8 ? ((g & 2) ? -1.0f : 1.0f) : ((g & 2) ? -1.0f : 1.0f));
    return (gx * x + gy * y) + gz * z;
}

__device__ __forceinline__ int perm12(uint32_t p) { return (int)(jenkins_hash(p) % 12u); }

__device__ __forceinline__ float simplex3(float px, float py, float pz, float scale, int seed)
{
    const float xin = px * scale, yin = py * scale, zin = pz * scale;
    const float F3 = 1.0f / 3.0f, G3 = 1.0f / 6.0f;
    const float s = ((xin + yin) + zin) * F3;
    const int i = (int)floorf(xin + s);
    const int j = (int)floorf(yin + s);
    const int k = (int)floorf(zin + s);
    const float t = (float)(i + j + k) * G3;
    const float x0 = xin - ((float)i - t), y0 = yin - ((float)j - t), z0 = zin - ((float)k - t);
    int i1, j1, k1, i2, j2, k2;
    if (x0 >= y0) {
        if (y0 >= z0) { i1 = 1; j1 = 0; k1 = 0; i2 = 1; j2 = 1; k2 = 0; }
        else if (x0 >= z0) { i1 = 1; j1 = 0; k1 = 0; i2 = 1; j2 = 0; k2 = 1; }
        else { i1 = 0; j1 = 0; k1 = 1; i2 = 1; j2 = 0; k2 = 1; }
    } else {
        if (y0 < z0) { i1 = 0; j1 = 0; k1 = 1; i2 = 0; j2 = 1; k2 = 1; }
        else if (x0 < z0) { i1 = 0; j1 = 1; k1 = 0; i2 = 0; j2 = 1; k2 = 1; }
        else { i1 = 0; j1 = 1; k1 = 0; i2 = 1; j2 = 1; k2 = 0; }
    }
    const float x1 = (x0 - (float)i1) + G3, y1 = (y0 - (float)j1) + G3, z1 = (z0 - (float)k1) + G3;
    const float x2 = (x0 - (float)i2) + 2.0f * G3, y2 = (y0 - (float)j2) + 2.0f * G3,
                z2 = (z0 - (float)k2) + 2.0f * G3;
    const float x3 = (x0 - 1.0f) + 3.0f * G3, y3 = (y0 - 1.0f) + 3.0f * G3,
                z3 = (z0 - 1.0f) + 3.0f * G3;
    const uint32_t us = (uint32_t)seed, ui = (uint32_t)i, uj = (uint32_t)j, uk = (uint32_t)k;
    const int g0 = perm12(us + ui * 607495u + uj * 359609u + uk * 654846u);
    const int g1 = perm12(us + (ui + (uint32_t)i1) * 607495u + (uj + (uint32_t)j1) * 359609u +
                          (uk + (uint32_t)k1) * 654846u);
    const int g2 = perm12(us + (ui + (uint32_t)i2) * 607495u + (uj + (uint32_t)j2) * 359609u +
                          (uk + (uint32_t)k2) * 654846u);
    const int g3 = perm12(us + (ui + 1u) * 607495u + (uj + 1u) * 359609u + (uk + 1u) * 654846u);
    float n0 = 0.0f, n1 = 0.0f, n2 = 0.0f, n3 = 0.0f;
    float t0 = ((0.6f - x0 * x0) - y0 * y0) - z0 * z0;
    if (!(t0 < 0.0f)) { t0 = t0 * t0; n0 = (t0 * t0) * grad_dot(g0, x0, y0, z0); }
    float t1 = ((0.6f - x1 * x1) - y1 * y1) - z1 * z1;
    if (!(t1 < 0.0f)) { t1 = t1 * t1; n1 = (t1 * t1) * grad_dot(g1, x1, y1, z1); }
    float t2 = ((0.6f - x2 * x2) - y2 * y2) - z2 * z2;
    if (!(t2 < 0.0f)) { t2 = t2 * t2; n2 = (t2 * t2) * grad_dot(g2, x2, y2, z2); }
    float t3 = ((0.6f - x3 * x3) - y3 * y3) - z3 * z3;
    if (!(t3 < 0.0f)) { t3 = t3 * t3; n3 = (t3 * t3) * grad_dot(g3, x3, y3, z3); }
    return 32.0f * (((n0 + n1) + n2) + n3);
}

// cuda::std::lerp (P0811R3 algorithm), processDivergence (plate_tectonics_kernel.cu:354)
__device__ __forceinline__ float lerp_p0811(float a, float b, float t)
{
    if ((a <= 0.0f && b >= 0.0f) || (a >= 0.0f && b <= 0.0f)) return t * b + (1.0f - t) * a;
    if (t == 1.0f) return b;
    const float x = a + t * (b - a);
    if ((t > 1.0f) == (b > a)) return b < x ? x : b;
    return x < b ? x : b;
}

}  // namespace tecto
