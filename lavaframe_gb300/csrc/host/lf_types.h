// Host value types of the LavaFrame scene API: Vec2/iVec2/Vec3/Vec4/Mat4.
//
// Layouts follow the reference (LavaFrame/Vec2.h:9-24, Vec3.h:13-38, Vec4.h:11-19,
// Mat4.h:12-27) because the flat scene arrays built from them are uploaded byte-for-byte:
// Vec3 is 12 bytes, Vec4 16 bytes, Mat4 64 bytes stored as data[row][col] where row i is
// GL column i (translation lives in data[3][0..2]).
//
// Min/Max deliberately keep std::min/std::max semantics ((b < a) ? b : a and
// (a < b) ? b : a): with signed zeros and NaNs the result depends on argument order,
// and the BVH node bytes must come out identical to the reference build.
// Everything here must be compiled without floating-point contraction
// (-ffp-contract=off): the BVH build is order- and rounding-sensitive.
#pragma once

#include <cmath>
#include <cstdint>

#define LF_PI 3.14159265358979323846f

namespace LavaFrame
{
    struct Math
    {
        static inline float Degrees(float radians) { return radians * (180.f / LF_PI); }
        static inline float Radians(float degrees) { return degrees * (LF_PI / 180.f); }
        static inline float Clamp(float x, float lo, float hi)
        {
            float m = (x < lo) ? lo : x;   // std::max(x, lo)
            return (m < hi) ? m : hi;      // std::min(hi, m)
        }
    };

    struct iVec2
    {
        iVec2() : x(0), y(0) {}
        iVec2(int x_, int y_) : x(x_), y(y_) {}
        int x, y;
    };

    struct Vec2
    {
        Vec2() : x(0), y(0) {}
        Vec2(float x_, float y_) : x(x_), y(y_) {}
        float x, y;
    };

    struct Vec4
    {
        Vec4() : x(0), y(0), z(0), w(0) {}
        Vec4(float x_, float y_, float z_, float w_) : x(x_), y(y_), z(z_), w(w_) {}
        float operator[](int i) const { return i == 0 ? x : i == 1 ? y : i == 2 ? z : w; }
        float x, y, z, w;
    };

    struct Vec3
    {
        Vec3() : x(0), y(0), z(0) {}
        Vec3(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}
        explicit Vec3(const Vec4& b) : x(b.x), y(b.y), z(b.z) {}

        Vec3 operator*(const Vec3& b) const { return Vec3(x * b.x, y * b.y, z * b.z); }
        Vec3 operator+(const Vec3& b) const { return Vec3(x + b.x, y + b.y, z + b.z); }
        Vec3 operator-(const Vec3& b) const { return Vec3(x - b.x, y - b.y, z - b.z); }
        Vec3 operator*(float b) const { return Vec3(x * b, y * b, z * b); }

        float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
        float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }

        static Vec3 Min(const Vec3& a, const Vec3& b)
        {
            return Vec3(b.x < a.x ? b.x : a.x, b.y < a.y ? b.y : a.y, b.z < a.z ? b.z : a.z);
        }
        static Vec3 Max(const Vec3& a, const Vec3& b)
        {
            return Vec3(a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y, a.z < b.z ? b.z : a.z);
        }
        static Vec3 Cross(const Vec3& a, const Vec3& b)
        {
            return Vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
        }
        static float Dot(const Vec3& a, const Vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
        static float Length(const Vec3& a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
        static float Distance(const Vec3& a, const Vec3& b) { return Length(a - b); }
        static Vec3 Clamp(const Vec3& a, const Vec3& lo, const Vec3& hi)
        {
            return Vec3(Math::Clamp(a.x, lo.x, hi.x), Math::Clamp(a.y, lo.y, hi.y), Math::Clamp(a.z, lo.z, hi.z));
        }
        static Vec3 Normalize(const Vec3& a)
        {
            float l = Length(a);
            return Vec3(a.x / l, a.y / l, a.z / l);
        }

        float x, y, z;
    };

    struct Mat4
    {
        Mat4()
        {
            for (int r = 0; r < 4; ++r)
                for (int c = 0; c < 4; ++c)
                    data[r][c] = (r == c) ? 1.f : 0.f;
        }
        float (&operator[](int i))[4] { return data[i]; }
        const float (&operator[](int i) const)[4] { return data[i]; }

        // Same expansion order as the reference product (Mat4.h:47-72): out[i][j] =
        // ((a[i][0]*b[0][j] + a[i][1]*b[1][j]) + a[i][2]*b[2][j]) + a[i][3]*b[3][j].
        Mat4 operator*(const Mat4& b) const
        {
            Mat4 out;
            for (int i = 0; i < 4; ++i)
                for (int j = 0; j < 4; ++j)
                    out.data[i][j] = data[i][0] * b.data[0][j] + data[i][1] * b.data[1][j] +
                                     data[i][2] * b.data[2][j] + data[i][3] * b.data[3][j];
            return out;
        }
        static Mat4 Translate(const Vec3& a)
        {
            Mat4 out;
            out[3][0] = a.x; out[3][1] = a.y; out[3][2] = a.z;
            return out;
        }
        static Mat4 Scale(const Vec3& a)
        {
            Mat4 out;
            out[0][0] = a.x; out[1][1] = a.y; out[2][2] = a.z;
            return out;
        }

        float data[4][4];
    };

    static_assert(sizeof(Vec3) == 12, "Vec3 layout");
    static_assert(sizeof(Vec4) == 16, "Vec4 layout");
    static_assert(sizeof(Mat4) == 64, "Mat4 layout");
}
