// Arithmetic contract of the path tracer: one definition of every operation whose result
// GLSL leaves to the implementation, shared by the CUDA kernels and the CPU oracle.
//
// GLSL 3.30 fixes the formulas of min/max/clamp/mix/reflect/refract/dot/cross but not the
// precision of sin/cos/tan/acos/atan/exp/log/pow, nor how `inverse()` or texture filtering
// round. The reference path tracer (shaders/common/*.glsl) depends on all of them, so
// bit-identical CPU/GPU results need a fixed definition:
//  - min/max/clamp/mix/reflect/refract/dot/cross/normalize: the GLSL specification
//    formulas, evaluated left to right in IEEE single precision, no fused multiply-add
//    (device code is compiled with --fmad=false, host code with -ffp-contract=off);
//  - sqrt and division: IEEE correctly rounded on both sides;
//  - sin/cos/tan: Cody-Waite reduction by pi/2 (three-part constant) and Taylor
//    polynomials on [-pi/4, pi/4] (sin to x^9, cos to x^10);
//  - atan/atan2/acos: reduction to |s| <= tan(pi/8) via atan(t) = pi/4 + atan((t-1)/(t+1))
//    and the arctangent series to s^17; acos(x) = atan2(sqrt((1-x)(1+x)), x);
//  - exp: k = rint(x log2 e), two-part ln 2, degree-7 Taylor polynomial, exact scaling;
//  - log: m in [sqrt(1/2), sqrt(2)), log m = 2 atanh((m-1)/(m+1)) series to s^11;
//  - pow(x, y) = exp(y log x) with the IEEE special cases for 0, 1 and infinity;
//  - matrix inverses (instance transforms, normal matrices) are computed once on the
//    host in double precision by cofactor expansion and rounded to float.
// Accuracy is about 1-2 ulp on the ranges the tracer uses; what matters is that host and
// device evaluate exactly the same sequence of IEEE operations.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

// The transcendental functions (LF_HD_CALL) stay out of line on the device: the shading kernel
// calls them from many places and inlining every copy costs more in instruction fetch than the
// calls do.
#if defined(__CUDACC__)
#define LF_HD __host__ __device__ __forceinline__
#define LF_HD_CALL [[maybe_unused]] static __host__ __device__ __noinline__
#else
#define LF_HD inline
#define LF_HD_CALL inline
#endif

namespace lfc
{
LF_HD float as_float(uint32_t u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

LF_HD uint32_t as_uint(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

// GLSL min(x, y): y if y < x, otherwise x. max(x, y): y if x < y, otherwise x.
LF_HD float fmin_g(float x, float y) { return (y < x) ? y : x; }
LF_HD float fmax_g(float x, float y) { return (x < y) ? y : x; }
LF_HD float clamp_g(float x, float lo, float hi) { return fmin_g(fmax_g(x, lo), hi); }
LF_HD float mix_g(float x, float y, float a) { return x * (1.0f - a) + y * a; }

LF_HD float round_even(float x)
{
#if defined(__CUDA_ARCH__)
    return rintf(x);
#else
    return nearbyintf(x);
#endif
}

// x * 2^k for integer k in [-252, 254], exact (two-step power-of-two scaling).
LF_HD float scale2(float x, int k)
{
    int k1 = k / 2;
    int k2 = k - k1;
    float s1 = as_float((uint32_t)(k1 + 127) << 23);
    float s2 = as_float((uint32_t)(k2 + 127) << 23);
    return (x * s1) * s2;
}

constexpr float kPi = 3.14159265358979323846f;
constexpr float kPiO2 = 1.57079632679489661923f;
constexpr float kPiO4 = 0.785398163397448309616f;

// ------------------------------------------------------------------ sin / cos / tan
LF_HD float sin_poly(float r)
{
    float z = r * r;
    float p = 2.75573192e-6f;                   // 1/9!
    p = p * z + -1.98412698e-4f;                // -1/7!
    p = p * z + 8.33333333e-3f;                 // 1/5!
    p = p * z + -1.66666667e-1f;                // -1/3!
    return r + (r * z) * p;
}

LF_HD float cos_poly(float r)
{
    float z = r * r;
    float p = -2.75573192e-7f;                  // -1/10!
    p = p * z + 2.48015873e-5f;                 // 1/8!
    p = p * z + -1.38888889e-3f;                // -1/6!
    p = p * z + 4.16666667e-2f;                 // 1/4!
    p = p * z + -0.5f;
    return 1.0f + z * p;
}

// r = x - q*pi/2 with pi/2 = C1 + C2 + C3 (C1, C2 hold 12 significant bits).
LF_HD float reduce_pio2(float x, int* q)
{
    float k = round_even(x * 0.636619772f);
    *q = (int)k;
    const float C1 = 1.57080078125f;
    const float C2 = -4.45358455181121826e-06f;
    const float C3 = -8.70551630782756500e-10f;
    return ((x - k * C1) - k * C2) - k * C3;
}

LF_HD_CALL void sincos_c(float x, float* s, float* c)
{
    int q;
    float r = reduce_pio2(x, &q);
    float sr = sin_poly(r), cr = cos_poly(r);
    switch (q & 3)
    {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = -sr; break;
    case 2: *s = -sr; *c = -cr; break;
    default: *s = -cr; *c = sr; break;
    }
}

LF_HD_CALL float sin_c(float x)
{
    float s, c;
    sincos_c(x, &s, &c);
    return s;
}

LF_HD_CALL float cos_c(float x)
{
    float s, c;
    sincos_c(x, &s, &c);
    return c;
}

LF_HD_CALL float tan_c(float x)
{
    float s, c;
    sincos_c(x, &s, &c);
    return s / c;
}

// ------------------------------------------------------------------ atan / atan2 / acos
// atan on [0, 1].
LF_HD float atan_unit(float t)
{
    float base = 0.0f;
    if (t > 0.414213568f)
    {
        t = (t - 1.0f) / (t + 1.0f);
        base = kPiO4;
    }
    float z = t * t;
    float p = 1.0f / 17.0f;
    p = p * z + -1.0f / 15.0f;
    p = p * z + 1.0f / 13.0f;
    p = p * z + -1.0f / 11.0f;
    p = p * z + 1.0f / 9.0f;
    p = p * z + -1.0f / 7.0f;
    p = p * z + 1.0f / 5.0f;
    p = p * z + -1.0f / 3.0f;
    return base + (t + (t * z) * p);
}

LF_HD_CALL float atan2_c(float y, float x)
{
    if (x != x || y != y) return x + y;
    float ax = fabsf(x), ay = fabsf(y);
    bool xneg = (as_uint(x) >> 31) != 0;
    float a;
    if (ay == 0.0f)
        a = xneg ? kPi : 0.0f;
    else if (ax == 0.0f)
        a = kPiO2;
    else if (ax == ay)
        a = xneg ? 3.0f * kPiO4 : kPiO4;   // also covers both infinite
    else
    {
        if (ay <= ax)
            a = atan_unit(ay / ax);
        else
            a = kPiO2 - atan_unit(ax / ay);
        if (xneg) a = kPi - a;
    }
    return (as_uint(y) >> 31) ? -a : a;
}

LF_HD_CALL float acos_c(float x) { return atan2_c(sqrtf((1.0f - x) * (1.0f + x)), x); }

// ------------------------------------------------------------------ exp / log / pow
LF_HD_CALL float exp_c(float x)
{
    if (x != x) return x;
    if (x > 88.7228394f) return as_float(0x7f800000u);
    if (x < -103.972076f) return 0.0f;
    float k = round_even(x * 1.44269502f);
    const float L1 = 0.693115234375f;
    const float L2 = 3.19461832987144589e-05f;
    float r = (x - k * L1) - k * L2;
    float p = 1.0f / 5040.0f;
    p = p * r + 1.0f / 720.0f;
    p = p * r + 1.0f / 120.0f;
    p = p * r + 1.0f / 24.0f;
    p = p * r + 1.0f / 6.0f;
    p = p * r + 0.5f;
    p = p * r + 1.0f;
    p = p * r + 1.0f;
    return scale2(p, (int)k);
}

LF_HD_CALL float log_c(float x)
{
    if (x != x || x < 0.0f) return as_float(0x7fc00000u);
    if (x == 0.0f) return -as_float(0x7f800000u);
    if (x == as_float(0x7f800000u)) return x;
    int e = 0;
    uint32_t u = as_uint(x);
    if ((u >> 23) == 0)
    {   // subnormal
        x = x * 8388608.0f;
        u = as_uint(x);
        e = -23;
    }
    e += (int)(u >> 23) - 127;
    float m = as_float((u & 0x007fffffu) | 0x3f800000u);   // [1, 2)
    if (m > 1.41421354f)
    {
        m = m * 0.5f;
        e += 1;
    }
    float s = (m - 1.0f) / (m + 1.0f);
    float z = s * s;
    float p = 1.0f / 11.0f;
    p = p * z + 1.0f / 9.0f;
    p = p * z + 1.0f / 7.0f;
    p = p * z + 1.0f / 5.0f;
    p = p * z + 1.0f / 3.0f;
    float lm = (2.0f * s) + (2.0f * s) * (z * p);
    const float L1 = 0.693115234375f;
    const float L2 = 3.19461832987144589e-05f;
    float fe = (float)e;
    return fe * L1 + (fe * L2 + lm);
}

LF_HD_CALL float pow_c(float x, float y)
{
    if (y == 0.0f || x == 1.0f) return 1.0f;
    if (x != x || y != y) return x + y;
    if (x < 0.0f) return as_float(0x7fc00000u);
    const float inf = as_float(0x7f800000u);
    if (x == 0.0f) return y > 0.0f ? 0.0f : inf;
    if (x == inf) return y > 0.0f ? inf : 0.0f;
    return exp_c(y * log_c(x));
}

// ------------------------------------------------------------------ matrix inverses
// Inverse of a 4x4 matrix given as 16 floats in LavaFrame's Mat4 order (m[i*4+j] =
// data[i][j], i.e. GLSL column i, row j). Output uses the same order. Returns false for
// a singular matrix (output then holds zeros). Cofactor expansion in double precision.
inline bool inverse4(const float* m, float* out)
{
    double a[16], inv[16];
    for (int i = 0; i < 16; ++i) a[i] = (double)m[i];
    inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    double det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
    if (det == 0.0)
    {
        for (int i = 0; i < 16; ++i) out[i] = 0.0f;
        return false;
    }
    double id = 1.0 / det;
    for (int i = 0; i < 16; ++i) out[i] = (float)(inv[i] * id);
    return true;
}

// Normal matrix transpose(inverse(mat3(M))) of a LavaFrame Mat4, as 9 floats in GLSL
// column-major order (n[c*3+r] = column c, row r).
inline bool normal_matrix(const float* m, float* n)
{
    // GLSL mat3(M)[c][r] = m[c*4+r]
    double a00 = m[0], a01 = m[4], a02 = m[8];    // row 0: columns 0..2
    double a10 = m[1], a11 = m[5], a12 = m[9];
    double a20 = m[2], a21 = m[6], a22 = m[10];
    double c00 = a11 * a22 - a12 * a21, c01 = -(a10 * a22 - a12 * a20), c02 = a10 * a21 - a11 * a20;
    double c10 = -(a01 * a22 - a02 * a21), c11 = a00 * a22 - a02 * a20, c12 = -(a00 * a21 - a01 * a20);
    double c20 = a01 * a12 - a02 * a11, c21 = -(a00 * a12 - a02 * a10), c22 = a00 * a11 - a01 * a10;
    double det = a00 * c00 + a01 * c01 + a02 * c02;
    if (det == 0.0)
    {
        for (int i = 0; i < 9; ++i) n[i] = 0.0f;
        return false;
    }
    double id = 1.0 / det;
    // inverse(A)[r][c] = cof(c, r)/det; transpose(inverse(A))[r][c] = cof(r, c)/det.
    // Column-major storage of B = transpose(inverse(A)): n[c*3 + r] = B[r][c] = cof(r,c)/det.
    const double cof[3][3] = {{c00, c01, c02}, {c10, c11, c12}, {c20, c21, c22}};
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r)
            n[c * 3 + r] = (float)(cof[r][c] * id);
    return true;
}
}
