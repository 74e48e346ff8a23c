// GLSL 3.30 semantics for C++ (test infrastructure): lets oracle/ref_shader_gen.py compile
// the reference's own fragment shaders (shaders/renderer.glsl + shaders/common/*.glsl) for
// the CPU, to produce golden vectors that pin the oracle and the CUDA path.
//
// Types follow the GLSL specification: vec2/3/4, ivec2/3/4, uvec4, bvec4, mat3/mat4
// (column-major), swizzles as proxy members (read and write), component-wise operators.
// Operations the specification leaves to the implementation take the project's arithmetic
// contract (csrc/lf_contract.h): transcendentals, inverse() (double-precision cofactors),
// texture filtering (GL_REPEAT, nearest = floor(u*size), linear with texel centres at +0.5).
// Float literals of the shader become float literals (the generator adds the suffix), so all
// arithmetic is single precision, evaluated left to right without contraction.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "lf_contract.h"

namespace glsl
{
typedef unsigned int uint;

struct vec2;
struct vec3;
struct vec4;

template <int A, int B>
struct Swz2
{
    float v[4];
    operator vec2() const;
    Swz2& operator=(const vec2& o);
};
template <int A, int B, int C>
struct Swz3
{
    float v[4];
    operator vec3() const;
    Swz3& operator=(const vec3& o);
};

struct vec2
{
    union
    {
        struct { float x, y; };
        struct { float r, g; };
    };
    vec2() : x(0.f), y(0.f) {}
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    vec2(const vec2& o) : x(o.x), y(o.y) {}
    vec2& operator=(const vec2& o) { x = o.x; y = o.y; return *this; }
};

struct vec3
{
    union
    {
        struct { float x, y, z; };
        struct { float r, g, b; };
        Swz2<0, 1> xy;
    };
    vec3() : x(0.f), y(0.f), z(0.f) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(const vec2& a, float c) : x(a.x), y(a.y), z(c) {}
    explicit vec3(const vec4& a);
    vec3(const vec3& o) : x(o.x), y(o.y), z(o.z) {}
    vec3& operator=(const vec3& o) { x = o.x; y = o.y; z = o.z; return *this; }
};

struct vec4
{
    union
    {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        Swz3<0, 1, 2> xyz;
        Swz3<0, 1, 2> rgb;
        Swz3<3, 0, 1> wxy;
        Swz2<0, 1> xy;
    };
    vec4() : x(0.f), y(0.f), z(0.f), w(0.f) {}
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec4(const vec4& o) : x(o.x), y(o.y), z(o.z), w(o.w) {}
    vec4& operator=(const vec4& o) { x = o.x; y = o.y; z = o.z; w = o.w; return *this; }
    // GLSL: vec4 xyzw swizzle of a texel fetch is the vector itself
    struct Self
    {
    };
};

inline vec3::vec3(const vec4& a) : x(a.x), y(a.y), z(a.z) {}

template <int A, int B>
Swz2<A, B>::operator vec2() const { return vec2(v[A], v[B]); }
template <int A, int B>
Swz2<A, B>& Swz2<A, B>::operator=(const vec2& o)
{
    v[A] = o.x;
    v[B] = o.y;
    return *this;
}
template <int A, int B, int C>
Swz3<A, B, C>::operator vec3() const { return vec3(v[A], v[B], v[C]); }
template <int A, int B, int C>
Swz3<A, B, C>& Swz3<A, B, C>::operator=(const vec3& o)
{
    v[A] = o.x;
    v[B] = o.y;
    v[C] = o.z;
    return *this;
}

struct ivec2
{
    int x, y;
    ivec2() : x(0), y(0) {}
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(const vec2& v) : x((int)v.x), y((int)v.y) {}
};
struct ivec3
{
    int x, y, z;
    ivec3() : x(0), y(0), z(0) {}
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    explicit ivec3(const vec3& v) : x((int)v.x), y((int)v.y), z((int)v.z) {}
};
struct ivec4
{
    union
    {
        struct { int x, y, z, w; };
        struct { int ix3[3]; int pad; };
    };
    ivec4() : x(0), y(0), z(0), w(0) {}
    ivec4(int a, int b, int c, int d) : x(a), y(b), z(c), w(d) {}
    // `.xyz` of an integer texel, used only as ivec3(texelFetch(...).xyz)
    struct XYZ
    {
        int a, b, c;
        operator ivec3() const { return ivec3(a, b, c); }
    };
};

struct uvec4
{
    uint x, y, z, w;
    uvec4() : x(0), y(0), z(0), w(0) {}
    uvec4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {}
    uvec4(const vec2& p, uint c, uint d) : x((uint)p.x), y((uint)p.y), z(c), w(d) {}
};
inline uvec4 operator*(const uvec4& a, uint s) { return uvec4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline uvec4 operator+(const uvec4& a, uint s) { return uvec4(a.x + s, a.y + s, a.z + s, a.w + s); }
inline uvec4 operator>>(const uvec4& a, uint s) { return uvec4(a.x >> s, a.y >> s, a.z >> s, a.w >> s); }
inline uvec4 operator^(const uvec4& a, const uvec4& b) { return uvec4(a.x ^ b.x, a.y ^ b.y, a.z ^ b.z, a.w ^ b.w); }

struct bvec4
{
    bool x, y, z, w;
};

// ---------------------------------------------------------------- vector operators
#define GLSL_V2OP(op)                                                                          \
    inline vec2 operator op(const vec2& a, const vec2& b) { return vec2(a.x op b.x, a.y op b.y); } \
    inline vec2 operator op(const vec2& a, float s) { return vec2(a.x op s, a.y op s); }           \
    inline vec2 operator op(float s, const vec2& a) { return vec2(s op a.x, s op a.y); }
GLSL_V2OP(+) GLSL_V2OP(-) GLSL_V2OP(*) GLSL_V2OP(/)
#define GLSL_V3OP(op)                                                                                        \
    inline vec3 operator op(const vec3& a, const vec3& b) { return vec3(a.x op b.x, a.y op b.y, a.z op b.z); } \
    inline vec3 operator op(const vec3& a, float s) { return vec3(a.x op s, a.y op s, a.z op s); }             \
    inline vec3 operator op(float s, const vec3& a) { return vec3(s op a.x, s op a.y, s op a.z); }
GLSL_V3OP(+) GLSL_V3OP(-) GLSL_V3OP(*) GLSL_V3OP(/)
#define GLSL_V4OP(op)                                                                                     \
    inline vec4 operator op(const vec4& a, const vec4& b)                                                 \
    {                                                                                                     \
        return vec4(a.x op b.x, a.y op b.y, a.z op b.z, a.w op b.w);                                      \
    }                                                                                                     \
    inline vec4 operator op(const vec4& a, float s) { return vec4(a.x op s, a.y op s, a.z op s, a.w op s); } \
    inline vec4 operator op(float s, const vec4& a) { return vec4(s op a.x, s op a.y, s op a.z, s op a.w); }
GLSL_V4OP(+) GLSL_V4OP(-) GLSL_V4OP(*) GLSL_V4OP(/)
#undef GLSL_V2OP
#undef GLSL_V3OP
#undef GLSL_V4OP
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec2 operator-(const vec2& a) { return vec2(-a.x, -a.y); }
inline vec4 operator-(const vec4& a) { return vec4(-a.x, -a.y, -a.z, -a.w); }
inline vec2& operator*=(vec2& a, const vec2& b) { return a = a * b; }
inline vec2& operator/=(vec2& a, const vec2& b) { return a = a / b; }
inline vec3& operator+=(vec3& a, const vec3& b) { return a = a + b; }
inline vec3& operator-=(vec3& a, const vec3& b) { return a = a - b; }
inline vec3& operator*=(vec3& a, const vec3& b) { return a = a * b; }
inline vec3& operator*=(vec3& a, float s) { return a = a * s; }
inline vec3& operator/=(vec3& a, float s) { return a = a / s; }
inline vec4& operator*=(vec4& a, float s) { return a = a * s; }

// ---------------------------------------------------------------- built-ins
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(const vec3& a, const vec3& b)
{
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length(const vec3& a) { return ::sqrtf(dot(a, a)); }
inline vec3 normalize(const vec3& a)
{
    float l = length(a);
    return vec3(a.x / l, a.y / l, a.z / l);
}
inline float min(float x, float y) { return lfc::fmin_g(x, y); }
inline float max(float x, float y) { return lfc::fmax_g(x, y); }
inline vec3 min(const vec3& a, const vec3& b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(const vec3& a, const vec3& b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline vec4 clamp(const vec4& x, float lo, float hi)
{
    return vec4(clamp(x.x, lo, hi), clamp(x.y, lo, hi), clamp(x.z, lo, hi), clamp(x.w, lo, hi));
}
inline vec4 max(const vec4& a, const vec4& b) { return vec4(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z), max(a.w, b.w)); }
// distance(a, b) = length(a - b): differences, squares and sum in component order, IEEE sqrt
inline float distance(const vec2& a, const vec2& b)
{
    float dx = a.x - b.x, dy = a.y - b.y;
    return ::sqrtf(dx * dx + dy * dy);
}
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(const vec3& x, const vec3& y, float a)
{
    float ia = 1.0f - a;
    return vec3(x.x * ia + y.x * a, x.y * ia + y.y * a, x.z * ia + y.z * a);
}
inline float abs(float x) { return ::fabsf(x); }
inline float sqrt(float x) { return ::sqrtf(x); }
inline vec3 sqrt(const vec3& a) { return vec3(sqrt(a.x), sqrt(a.y), sqrt(a.z)); }
inline float sin(float x) { return lfc::sin_c(x); }
inline float cos(float x) { return lfc::cos_c(x); }
inline float tan(float x) { return lfc::tan_c(x); }
inline float acos(float x) { return lfc::acos_c(x); }
inline float atan(float y, float x) { return lfc::atan2_c(y, x); }
inline float exp(float x) { return lfc::exp_c(x); }
inline float log(float x) { return lfc::log_c(x); }
inline float pow(float x, float y) { return lfc::pow_c(x, y); }
inline vec3 exp(const vec3& a) { return vec3(exp(a.x), exp(a.y), exp(a.z)); }
inline vec3 log(const vec3& a) { return vec3(log(a.x), log(a.y), log(a.z)); }
inline vec3 pow(const vec3& a, const vec3& b) { return vec3(pow(a.x, b.x), pow(a.y, b.y), pow(a.z, b.z)); }
inline vec4 pow(const vec4& a, const vec4& b) { return vec4(pow(a.x, b.x), pow(a.y, b.y), pow(a.z, b.z), pow(a.w, b.w)); }
inline vec3 reflect(const vec3& I, const vec3& N)
{
    float d = 2.0f * dot(N, I);
    return I - d * N;
}
inline vec3 refract(const vec3& I, const vec3& N, float eta)
{
    float d = dot(N, I);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return vec3(0.f, 0.f, 0.f);
    return eta * I - (eta * d + sqrt(k)) * N;
}
inline bvec4 greaterThanEqual(const vec4& a, const vec4& b) { return bvec4{a.x >= b.x, a.y >= b.y, a.z >= b.z, a.w >= b.w}; }
inline bool all(const bvec4& b) { return b.x && b.y && b.z && b.w; }

// ---------------------------------------------------------------- matrices (column-major)
struct mat3
{
    float m[9];   // m[c*3 + r]
    mat3() { std::memset(m, 0, sizeof m); }
};
struct mat4
{
    float m[16];  // m[c*4 + r]
    mat4() { std::memset(m, 0, sizeof m); }
    mat4(const vec4& c0, const vec4& c1, const vec4& c2, const vec4& c3)
    {
        const vec4* c[4] = {&c0, &c1, &c2, &c3};
        for (int i = 0; i < 4; ++i)
        {
            m[i * 4 + 0] = c[i]->x;
            m[i * 4 + 1] = c[i]->y;
            m[i * 4 + 2] = c[i]->z;
            m[i * 4 + 3] = c[i]->w;
        }
    }
};
inline mat3 mat3_of(const mat4& a)
{
    mat3 r;
    for (int c = 0; c < 3; ++c)
        for (int k = 0; k < 3; ++k) r.m[c * 3 + k] = a.m[c * 4 + k];
    return r;
}
inline vec4 operator*(const mat4& M, const vec4& v)
{
    const float* m = M.m;
    return vec4(m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * v.w, m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * v.w,
                m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w, m[3] * v.x + m[7] * v.y + m[11] * v.z + m[15] * v.w);
}
inline vec3 operator*(const mat3& M, const vec3& v)
{
    const float* m = M.m;
    return vec3(m[0] * v.x + m[3] * v.y + m[6] * v.z, m[1] * v.x + m[4] * v.y + m[7] * v.z, m[2] * v.x + m[5] * v.y + m[8] * v.z);
}
inline mat4 inverse(const mat4& a)
{
    mat4 r;
    lfc::inverse4(a.m, r.m);
    return r;
}
// transpose(inverse(mat3(M))) is what the shader forms; the contract defines it in one
// double-precision step (lfc::normal_matrix). inverse() marks the matrix, transpose()
// evaluates the pair.
struct mat3_inv
{
    mat3 src;
};
inline mat3_inv inverse(const mat3& a) { return mat3_inv{a}; }
inline mat3 transpose(const mat3_inv& x)
{
    float m4[16] = {0};
    for (int c = 0; c < 3; ++c)
        for (int k = 0; k < 3; ++k) m4[c * 4 + k] = x.src.m[c * 3 + k];
    m4[15] = 1.0f;
    mat3 r;
    lfc::normal_matrix(m4, r.m);
    return r;
}

// ---------------------------------------------------------------- samplers
struct samplerBuffer
{
    const float* data = nullptr;
    int comps = 3;
    long long n = 0;
};
struct isamplerBuffer
{
    const int* data = nullptr;
    int comps = 3;
    long long n = 0;
};
struct sampler2D
{
    const float* data = nullptr;
    int w = 0, h = 0, comps = 4;
    bool linear = false;
};
struct sampler2DArray
{
    const unsigned char* data = nullptr;
    int w = 0, h = 0, layers = 0;
};

inline vec4 texelFetch(const samplerBuffer& s, int i)
{
    const float* p = s.data + (long long)i * s.comps;
    return vec4(p[0], s.comps > 1 ? p[1] : 0.f, s.comps > 2 ? p[2] : 0.f, s.comps > 3 ? p[3] : 1.f);
}
struct ivec4fetch
{
    int x, y, z, w;
    ivec4::XYZ xyz;
};
inline ivec4fetch texelFetch(const isamplerBuffer& s, int i)
{
    const int* p = s.data + (long long)i * s.comps;
    ivec4fetch r{p[0], p[1], p[2], 1, {p[0], p[1], p[2]}};
    return r;
}
inline vec4 texel2D(const sampler2D& s, int x, int y)
{
    const float* p = s.data + ((long long)y * s.w + x) * s.comps;
    return vec4(p[0], s.comps > 1 ? p[1] : 0.f, s.comps > 2 ? p[2] : 0.f, s.comps > 3 ? p[3] : 1.f);
}
inline vec4 texelFetch(const sampler2D& s, const ivec2& c, int) { return texel2D(s, c.x, c.y); }
inline int wrap(int i, int n)
{
    int r = i % n;
    return r < 0 ? r + n : r;
}
inline vec4 texture(const sampler2D& s, const vec2& uv)
{
    if (!s.data) return vec4(0.f);
    if (!s.linear)
        return texel2D(s, wrap((int)::floorf(uv.x * (float)s.w), s.w), wrap((int)::floorf(uv.y * (float)s.h), s.h));
    float xf = uv.x * (float)s.w - 0.5f, yf = uv.y * (float)s.h - 0.5f;
    float x0f = ::floorf(xf), y0f = ::floorf(yf);
    float a = xf - x0f, b = yf - y0f;
    int x0 = wrap((int)x0f, s.w), x1 = wrap((int)x0f + 1, s.w), y0 = wrap((int)y0f, s.h), y1 = wrap((int)y0f + 1, s.h);
    vec4 t00 = texel2D(s, x0, y0), t10 = texel2D(s, x1, y0), t01 = texel2D(s, x0, y1), t11 = texel2D(s, x1, y1);
    float ia = 1.0f - a, ib = 1.0f - b;
    float c[4];
    const float* p00 = &t00.x;
    const float* p10 = &t10.x;
    const float* p01 = &t01.x;
    const float* p11 = &t11.x;
    for (int k = 0; k < 4; ++k)
    {
        float top = p00[k] * ia + p10[k] * a;
        float bot = p01[k] * ia + p11[k] * a;
        c[k] = top * ib + bot * b;
    }
    return vec4(c[0], c[1], c[2], c[3]);
}
inline vec4 texture(const sampler2DArray& s, const vec3& uvl)
{
    int l = (int)::floorf(uvl.z + 0.5f);
    l = l < 0 ? 0 : (l >= s.layers ? s.layers - 1 : l);
    const unsigned char* base = s.data + (long long)l * s.w * s.h * 4;
    float xf = uvl.x * (float)s.w - 0.5f, yf = uvl.y * (float)s.h - 0.5f;
    float x0f = ::floorf(xf), y0f = ::floorf(yf);
    float a = xf - x0f, b = yf - y0f;
    int x0 = wrap((int)x0f, s.w), x1 = wrap((int)x0f + 1, s.w), y0 = wrap((int)y0f, s.h), y1 = wrap((int)y0f + 1, s.h);
    float c[4];
    for (int k = 0; k < 4; ++k)
    {
        float t00 = base[((long long)y0 * s.w + x0) * 4 + k] / 255.0f, t10 = base[((long long)y0 * s.w + x1) * 4 + k] / 255.0f;
        float t01 = base[((long long)y1 * s.w + x0) * 4 + k] / 255.0f, t11 = base[((long long)y1 * s.w + x1) * 4 + k] / 255.0f;
        float top = t00 * (1.0f - a) + t10 * a;
        float bot = t01 * (1.0f - a) + t11 * a;
        c[k] = top * (1.0f - b) + bot * b;
    }
    return vec4(c[0], c[1], c[2], c[3]);
}
}
