/*
 * tecto_math.h - the engine's definitions of sin(x), cos(x), exp(x), log10(x) and atan2(y, x) in
 * single precision.
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
 * [-pi/4, pi/4] to degree 11 / 10 (truncation error below 1e-11), evaluated by Horner's rule with
 * explicit fused multiply-adds.  Accuracy (measured against the correctly rounded sine): within
 * 2 ulp for |x| < 6.5e4; beyond that the reduction loses bits gracefully.
 *
 * Compile GPU code with -fmad=false and host code with -ffp-contract=off so that no other
 * multiply-add is contracted; then both sides produce identical results.
 */
#ifndef TECTO_MATH_H
#define TECTO_MATH_H

#if defined(__CUDACC__)
#define TECTO_HD __host__ __device__ __forceinline__
#include <string.h>
#else
#define TECTO_HD static inline
#include <math.h>
#include <string.h>
#endif

/* 2/pi; rintf(x * TECTO_TWO_OVER_PI) is the quadrant of the reduction */
#define TECTO_TWO_OVER_PI 0.6366197466850281f

/* The sine series of the reduced argument r (Taylor coefficients 1/n! with alternating signs). */
TECTO_HD float tecto_sin_series(float r)
{
    const float S3 = -1.6666666666666666e-1f;
    const float S5 = 8.3333333333333332e-3f;
    const float S7 = -1.9841269841269841e-4f;
    const float S9 = 2.7557319223985893e-6f;
    const float S11 = -2.5052108385441720e-8f;
    const float r2 = r * r;
    float ps = fmaf(r2, S11, S9);
    ps = fmaf(r2, ps, S7);
    ps = fmaf(r2, ps, S5);
    ps = fmaf(r2, ps, S3);
    return fmaf(r * r2, ps, r);
}

/* The shared core of tecto_sinf and tecto_cosf: the quadrant q of x and the sine and cosine of the
 * reduced argument.  Every step is a fused multiply-add (one rounding), the same on the GPU (FFMA)
 * and on the host (C99 fmaf, correctly rounded), so both sides still agree bit for bit; the
 * products kf * C1..C3 are exact, so the first three reduction steps equal the unfused ones. */
TECTO_HD void tecto_sincos_core(float x, int *q, float *s, float *c)
{
    /* pi/2 = C1 + C2 + C3 + C4, C1..C3 with 8 significant bits each */
    const float C1 = 1.5703125f;
    const float C2 = 4.825592041015625e-4f;
    const float C3 = 1.2665987014770508e-6f;
    const float C4 = 9.92093629470503e-10f;
    const float TWO_OVER_PI = TECTO_TWO_OVER_PI;
    /* Taylor coefficients 1/n! with alternating signs */
    const float K2 = -0.5f;
    const float K4 = 4.1666666666666664e-2f;
    const float K6 = -1.3888888888888889e-3f;
    const float K8 = 2.4801587301587302e-5f;
    const float K10 = -2.7557319223985888e-7f;

    const float kf = rintf(x * TWO_OVER_PI);
    float r = fmaf(-kf, C1, x);
    r = fmaf(-kf, C2, r);
    r = fmaf(-kf, C3, r);
    r = fmaf(-kf, C4, r);
    const float r2 = r * r;
    *s = tecto_sin_series(r);
    float pc = fmaf(r2, K10, K8);
    pc = fmaf(r2, pc, K6);
    pc = fmaf(r2, pc, K4);
    pc = fmaf(r2, pc, K2);
    *c = fmaf(r2, pc, 1.0f);
    *q = ((int)kf) & 3;
}

TECTO_HD float tecto_sinf(float x)
{
    int q;
    float s, c;
    tecto_sincos_core(x, &q, &s, &c);
    return q == 0 ? s : (q == 1 ? c : (q == 2 ? -s : -c));
}

/* cos(x): the reduction and the two series of tecto_sinf, with the quadrant shifted by one.  Used by
 * plate dynamics' angular centre sums (cosf at src/cuda_compute/plate_tectonics_kernel.cu:2173-2175). */
TECTO_HD float tecto_cosf(float x)
{
    int q;
    float s, c;
    tecto_sincos_core(x, &q, &s, &c);
    return q == 0 ? c : (q == 1 ? -s : (q == 2 ? -c : s));
}

/* Bit pattern helpers (no type punning through unions, valid C and CUDA C++). */
TECTO_HD unsigned tecto_f2u(float f)
{
    unsigned u;
    memcpy(&u, &f, sizeof u);
    return u;
}

TECTO_HD float tecto_u2f(unsigned u)
{
    float f;
    memcpy(&f, &u, sizeof f);
    return f;
}

/*
 * exp(x) in single precision, for the reference uplift's distance profiles (expf at
 * src/cuda_compute/plate_tectonics_kernel.cu:1656-1659).  Method: Cody-Waite reduction
 * x = k ln2 + r with ln2 split in a 16-bit head (exact products for |k| < 2^8) and a tail, the
 * Taylor series of e^r to degree 8 on |r| <= ln2 / 2 (truncation below 2e-10), and the scale by 2^k
 * assembled from the exponent bits, with one final rounding for subnormal results.  Accuracy:
 * within 1.2 ulp of exp for |x| < 88 and in the subnormal range (measured on the host against
 * double precision over every 991st float).
 */
TECTO_HD float tecto_expf(float x)
{
    const float LOG2E = 1.44269502162933349609375f;
    const float LN2_HI = 0.693145751953125f;          /* 16 significant bits */
    const float LN2_LO = 1.428606765330187045037746429443359375e-6f;
    if (x != x) return x + x;                          /* NaN */
    if (x > 88.72283935546875f) return tecto_u2f(0x7f800000u);
    if (x < -103.97208404541015625f) return 0.0f;
    const float kf = rintf(x * LOG2E);
    float r = x - kf * LN2_HI;
    r = r - kf * LN2_LO;
    float p = 2.4801587301587302e-5f;                  /* 1/8! */
    p = 1.9841269841269841e-4f + r * p;                /* 1/7! */
    p = 1.3888888888888889e-3f + r * p;                /* 1/6! */
    p = 8.3333333333333332e-3f + r * p;                /* 1/5! */
    p = 4.1666666666666664e-2f + r * p;                /* 1/4! */
    p = 1.6666666666666666e-1f + r * p;                /* 1/3! */
    p = 0.5f + r * p;
    p = 1.0f + r * p;
    p = 1.0f + r * p;
    const int k = (int)kf;
    if (k > 127) return (p * tecto_u2f((unsigned)(127 + 127) << 23)) * 2.0f;
    if (k < -126) return (p * tecto_u2f((unsigned)(k + 64 + 127) << 23)) * tecto_u2f((unsigned)(127 - 64) << 23);
    return p * tecto_u2f((unsigned)(k + 127) << 23);
}

/*
 * log10(x) in single precision, for the reference uplift's subduction trench profile (log10 at
 * src/cuda_compute/plate_tectonics_kernel.cu:1649).  Method: x = m 2^e with m in [sqrt(2)/2,
 * sqrt(2)); ln m = 2 atanh(s), s = (m - 1) / (m + 1), |s| < 0.1716, summed as the odd series of
 * atanh to s^13; then log10 x = e log10(2) + ln(m) log10(e) with log10(2) split in a 16-bit head
 * and a tail.  Zero gives -inf, negative arguments and NaN give NaN.  Accuracy: within 3.5 ulp of
 * log10 (measured on the host against double precision over every 991st positive float).
 */
TECTO_HD float tecto_log10f(float x)
{
    const float LG2_HI = 0.30102539062500000000f;       /* 16 significant bits */
    const float LG2_LO = 4.6050389811952137388947244930267681898814621085413e-6f;
    const float INV_LN10 = 0.43429448190325182765f;
    unsigned u = tecto_f2u(x);
    if (x != x) return x + x;
    if (x < 0.0f) return tecto_u2f(0x7fc00000u);
    if (x == 0.0f) return tecto_u2f(0xff800000u);
    if (u >= 0x7f800000u) return x;                    /* +inf */
    int e = 0;
    if (u < 0x00800000u) {                             /* subnormal: scale by 2^25 */
        u = tecto_f2u(x * 33554432.0f);
        e = -25;
    }
    e += (int)(u >> 23) - 127;
    float m = tecto_u2f((u & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421353816986083984375f) {
        m = m * 0.5f;
        e += 1;
    }
    const float f = m - 1.0f;
    const float s = f / (2.0f + f);
    const float z = s * s;
    float q = 0.15384615384615385f;                    /* 2/13 */
    q = 0.18181818181818182f + z * q;                  /* 2/11 */
    q = 0.22222222222222221f + z * q;                  /* 2/9 */
    q = 0.2857142857142857f + z * q;                   /* 2/7 */
    q = 0.4f + z * q;                                  /* 2/5 */
    q = 0.66666666666666663f + z * q;                  /* 2/3 */
    const float lnm = 2.0f * s + (s * z) * q;
    const float ef = (float)e;
    return ef * LG2_HI + (ef * LG2_LO + lnm * INV_LN10);
}

/* v x scale rounded to the nearest 64-bit integer (ties to even), v first limited to [-lim, lim]
 * (NaN counts as 0): the fixed-point terms of plate dynamics' sums, whose integer additions give
 * the same result in any order. */
TECTO_HD long long tecto_fix(float v, float scale, float lim)
{
    v = (v == v) ? v : 0.0f;
    v = v < -lim ? -lim : (v > lim ? lim : v);
#if defined(__CUDA_ARCH__)
    return __float2ll_rn(v * scale);
#else
    return llrintf(v * scale);
#endif
}

/* A fixed-point sum back to float: (float)(sum x inv_scale), through double. */
TECTO_HD float tecto_unfix(long long sum, double inv_scale) { return (float)((double)sum * inv_scale); }

/*
 * atan2(y, x) in single precision, for plate dynamics' geometric centres (atan2f at
 * src/cuda_compute/plate_tectonics_kernel.cu:2216-2217).  Method (Cody and Waite, 1980, chapter
 * on the arctangent): t = min(|x|, |y|) / max(|x|, |y|) in [0, 1]; for t > 2 - sqrt(3) the
 * identity atan t = pi/6 + atan(((sqrt(3) - 1) t - 1/2 - 1/2 + t) / (sqrt(3) + t)) brings the
 * argument to |f| <= 2 - sqrt(3); there the Taylor series of atan to f^13 (truncation below 2e-9);
 * then the octant and the signs of x and y place the angle in (-pi, pi].  Signed zeros and
 * infinities follow C's atan2; NaN gives NaN.  Accuracy: within 3 ulp of atan2 (measured on the
 * host against double precision on a grid of 2^20 argument pairs).
 */
TECTO_HD float tecto_atan2f(float y, float x)
{
    const float PI_HI = 3.1415927410125732f;            /* float(pi) */
    const float PI_LO = -8.7422776573475858e-8f;         /* pi - PI_HI */
    const float PIO2_HI = 1.5707963705062866f;
    const float PIO2_LO = -4.3711388286737929e-8f;
    const float PIO6 = 0.52359877559829893f;
    const float SQRT3 = 1.7320508075688772f;
    const float SQRT3_M1 = 0.73205080756887719f;
    const float TWO_M_SQRT3 = 0.26794919243112270f;
    if (x != x || y != y) return x + y;
    const float ax = fabsf(x), ay = fabsf(y);
    const unsigned xneg = tecto_f2u(x) >> 31, yneg = tecto_f2u(y) >> 31;
    float a;
    if (ax == ay && ax == tecto_u2f(0x7f800000u)) {
        a = 0.78539816339744831f;                        /* both infinite: pi/4 */
    } else if (ay == 0.0f && ax == 0.0f) {
        a = 0.0f;
    } else {
        const int swap = ay > ax;
        const float t = swap ? ax / ay : ay / ax;        /* in [0, 1] */
        float f = t, base = 0.0f;
        if (t > TWO_M_SQRT3) {
            f = (((SQRT3_M1 * t - 0.5f) - 0.5f) + t) / (SQRT3 + t);
            base = PIO6;
        }
        const float z = f * f;
        float p = 1.0f / 13.0f;
        p = -1.0f / 11.0f + z * p;
        p = 1.0f / 9.0f + z * p;
        p = -1.0f / 7.0f + z * p;
        p = 1.0f / 5.0f + z * p;
        p = -1.0f / 3.0f + z * p;
        a = base + (f + (f * z) * p);
        if (swap) a = (PIO2_HI - a) + PIO2_LO;
    }
    if (xneg) a = (PI_HI - a) + PI_LO;
    return yneg ? -a : a;
}

#endif /* TECTO_MATH_H */
