// Small vector types with the GLSL 3.30 built-in semantics the path tracer relies on.
// Formulas are the ones the GLSL specification states (dot, cross, normalize = x/length,
// reflect, refract, mix, clamp, min, max), evaluated left to right in IEEE single
// precision; transcendental functions come from lf_contract.h. Shared by the CUDA kernels
// and the CPU oracle so that both run the same operation sequence.
#pragma once

#include "lf_contract.h"

namespace lfc
{
struct v2
{
    float x, y;
    LF_HD v2() : x(0.f), y(0.f) {}
    LF_HD v2(float a, float b) : x(a), y(b) {}
};

struct v3
{
    float x, y, z;
    LF_HD v3() : x(0.f), y(0.f), z(0.f) {}
    LF_HD explicit v3(float a) : x(a), y(a), z(a) {}
    LF_HD v3(float a, float b, float c) : x(a), y(b), z(c) {}
    LF_HD float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

LF_HD v3 operator+(v3 a, v3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
LF_HD v3 operator-(v3 a, v3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
LF_HD v3 operator*(v3 a, v3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
LF_HD v3 operator/(v3 a, v3 b) { return v3(a.x / b.x, a.y / b.y, a.z / b.z); }
LF_HD v3 operator*(v3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
LF_HD v3 operator*(float s, v3 a) { return v3(s * a.x, s * a.y, s * a.z); }
LF_HD v3 operator/(v3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
LF_HD v3 operator/(float s, v3 a) { return v3(s / a.x, s / a.y, s / a.z); }
LF_HD v3 operator+(v3 a, float s) { return v3(a.x + s, a.y + s, a.z + s); }
LF_HD v3 operator-(v3 a, float s) { return v3(a.x - s, a.y - s, a.z - s); }
LF_HD v3 operator-(v3 a) { return v3(-a.x, -a.y, -a.z); }
LF_HD v2 operator+(v2 a, v2 b) { return v2(a.x + b.x, a.y + b.y); }
LF_HD v2 operator*(v2 a, float s) { return v2(a.x * s, a.y * s); }

LF_HD float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
LF_HD v3 cross(v3 a, v3 b)
{
    return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
LF_HD float length(v3 a) { return sqrtf(dot(a, a)); }
LF_HD v3 normalize(v3 a)
{
    float l = length(a);
    return v3(a.x / l, a.y / l, a.z / l);
}
LF_HD v3 vmin(v3 a, v3 b) { return v3(fmin_g(a.x, b.x), fmin_g(a.y, b.y), fmin_g(a.z, b.z)); }
LF_HD v3 vmax(v3 a, v3 b) { return v3(fmax_g(a.x, b.x), fmax_g(a.y, b.y), fmax_g(a.z, b.z)); }
LF_HD v3 vabs(v3 a) { return v3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
LF_HD v3 vsqrt(v3 a) { return v3(sqrtf(a.x), sqrtf(a.y), sqrtf(a.z)); }
LF_HD v3 vexp(v3 a) { return v3(exp_c(a.x), exp_c(a.y), exp_c(a.z)); }
LF_HD v3 vlog(v3 a) { return v3(log_c(a.x), log_c(a.y), log_c(a.z)); }
LF_HD v3 vpow(v3 a, v3 b) { return v3(pow_c(a.x, b.x), pow_c(a.y, b.y), pow_c(a.z, b.z)); }
// GLSL mix(x, y, a) = x*(1-a) + y*a
LF_HD v3 mix(v3 x, v3 y, float a)
{
    float ia = 1.0f - a;
    return v3(x.x * ia + y.x * a, x.y * ia + y.y * a, x.z * ia + y.z * a);
}
LF_HD float mix(float x, float y, float a) { return mix_g(x, y, a); }
// GLSL reflect(I, N) = I - 2*dot(N, I)*N
LF_HD v3 reflect(v3 I, v3 N)
{
    float d = 2.0f * dot(N, I);
    return I - d * N;
}
// GLSL refract(I, N, eta): k = 1 - eta*eta*(1 - dot(N,I)*dot(N,I));
// k < 0 -> 0, else eta*I - (eta*dot(N,I) + sqrt(k))*N
LF_HD v3 refract(v3 I, v3 N, float eta)
{
    float d = dot(N, I);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return v3(0.f, 0.f, 0.f);
    return eta * I - (eta * d + sqrtf(k)) * N;
}

// Column-major 3x3 (c[col*3+row]) times vector: ((c0*v.x + c1*v.y) + c2*v.z).
LF_HD v3 mul3(const float* c, v3 v)
{
    return v3(c[0] * v.x + c[3] * v.y + c[6] * v.z,
              c[1] * v.x + c[4] * v.y + c[7] * v.z,
              c[2] * v.x + c[5] * v.y + c[8] * v.z);
}

// GLSL mat4 * vec4(p, w) keeping xyz: column c = (m[c*4+0], m[c*4+1], m[c*4+2]).
LF_HD v3 mul4_point(const float* m, v3 p, float w)
{
    return v3(m[0] * p.x + m[4] * p.y + m[8] * p.z + m[12] * w,
              m[1] * p.x + m[5] * p.y + m[9] * p.z + m[13] * w,
              m[2] * p.x + m[6] * p.y + m[10] * p.z + m[14] * w);
}
}
