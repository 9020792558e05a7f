/*
 * tecto_math.h - the engine's definition of sin(x) in single precision.
 *
 * The reference's sediment capacity uses sinf (src/cuda_compute/plate_tectonics_kernel.cu:2546).
 * CUDA's sinf and the host libm's sinf are different approximations, and the erosion step has
 * thresholds (capacity > sediment, clamps), so a last-bit difference in sin can flip a branch.
 * The engine therefore fixes one sine, evaluated with the same IEEE operations in the same order
 * on the GPU and on the host, so that the CUDA kernels and the CPU oracle agree bit for bit.
 *
 * Method: Cody-Waite additive range reduction by pi/2 (W. J. Cody and W. Waite, "Software Manual
 * for the Elementary Functions", 1980) with a four-part split of pi/2 (8 + 8 + 8 + 24 significant
 * bits, exact products for |k| < 2^16), then the Taylor series of sin and cos about 0 on
 * [-pi/4, pi/4] to degree 11 / 10 (truncation error below 1e-11).  Accuracy (measured against the
 * correctly rounded sine): within 2 ulp for |x| < 6.5e4; beyond that the reduction loses bits
 * gracefully.
 *
 * Compile GPU code with -fmad=false and host code with -ffp-contract=off so that no multiply-add
 * is contracted; then both sides produce identical results.
 */
#ifndef TECTO_MATH_H
#define TECTO_MATH_H

#if defined(__CUDACC__)
#define TECTO_HD __host__ __device__ __forceinline__
#else
#define TECTO_HD static inline
#include <math.h>
#endif

TECTO_HD float tecto_sinf(float x)
{
    /* pi/2 = C1 + C2 + C3 + C4, C1..C3 with 8 significant bits each */
    const float C1 = 1.5703125f;
    const float C2 = 4.825592041015625e-4f;
    const float C3 = 1.2665987014770508e-6f;
    const float C4 = 9.92093629470503e-10f;
    const float TWO_OVER_PI = 0.6366197466850281f;
    /* Taylor coefficients 1/n! with alternating signs */
    const float S3 = -1.6666666666666666e-1f;
    const float S5 = 8.3333333333333332e-3f;
    const float S7 = -1.9841269841269841e-4f;
    const float S9 = 2.7557319223985893e-6f;
    const float S11 = -2.5052108385441720e-8f;
    const float K2 = -0.5f;
    const float K4 = 4.1666666666666664e-2f;
    const float K6 = -1.3888888888888889e-3f;
    const float K8 = 2.4801587301587302e-5f;
    const float K10 = -2.7557319223985888e-7f;

    const float kf = rintf(x * TWO_OVER_PI);
    float r = x - kf * C1;
    r = r - kf * C2;
    r = r - kf * C3;
    r = r - kf * C4;
    const float r2 = r * r;
    float ps = S11;
    ps = S9 + r2 * ps;
    ps = S7 + r2 * ps;
    ps = S5 + r2 * ps;
    ps = S3 + r2 * ps;
    const float s = r + (r * r2) * ps;
    float pc = K10;
    pc = K8 + r2 * pc;
    pc = K6 + r2 * pc;
    pc = K4 + r2 * pc;
    pc = K2 + r2 * pc;
    const float c = 1.0f + r2 * pc;
    const int q = ((int)kf) & 3;
    return q == 0 ? s : (q == 1 ? c : (q == 2 ? -s : -c));
}

#endif /* TECTO_MATH_H */
