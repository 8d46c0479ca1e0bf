// Oracle (test infrastructure only): GLSL-style vector maths for the CPU restatement of Lumen's shaders.
//
// Every helper follows the GLSL 4.60 definition of the built-in it stands for (dot, cross, length,
// normalize, mix, clamp, reflect, sign), evaluated left to right in the element type T, so that a
// float instantiation performs the same IEEE operation sequence as the shader source it restates.
// The oracle is built with -ffp-contract=off: no multiply-add is fused behind the source's back.
// A double instantiation gives the FP64 reference renders.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>

namespace orc {

template <class T> struct V2 {
    T x, y;
    V2() : x(0), y(0) {}
    V2(T a, T b) : x(a), y(b) {}
};

template <class T> struct V3 {
    T x, y, z;
    V3() : x(0), y(0), z(0) {}
    explicit V3(T a) : x(a), y(a), z(a) {}
    V3(T a, T b, T c) : x(a), y(b), z(c) {}
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    V3& operator+=(const V3& o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
    V3& operator-=(const V3& o) { x = x - o.x; y = y - o.y; z = z - o.z; return *this; }
    V3& operator*=(const V3& o) { x = x * o.x; y = y * o.y; z = z * o.z; return *this; }
    V3& operator*=(T s) { x = x * s; y = y * s; z = z * s; return *this; }
    V3& operator/=(T s) { x = x / s; y = y / s; z = z / s; return *this; }
};

template <class T> struct V4 {
    T x, y, z, w;
    V4() : x(0), y(0), z(0), w(0) {}
    V4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    V3<T> xyz() const { return V3<T>(x, y, z); }
};

template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return V3<T>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return V3<T>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class T> inline V3<T> operator*(V3<T> a, V3<T> b) { return V3<T>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <class T> inline V3<T> operator/(V3<T> a, V3<T> b) { return V3<T>(a.x / b.x, a.y / b.y, a.z / b.z); }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return V3<T>(a.x * s, a.y * s, a.z * s); }
template <class T> inline V3<T> operator*(T s, V3<T> a) { return V3<T>(s * a.x, s * a.y, s * a.z); }
template <class T> inline V3<T> operator/(V3<T> a, T s) { return V3<T>(a.x / s, a.y / s, a.z / s); }
template <class T> inline V3<T> operator+(V3<T> a, T s) { return V3<T>(a.x + s, a.y + s, a.z + s); }
template <class T> inline V3<T> operator-(V3<T> a, T s) { return V3<T>(a.x - s, a.y - s, a.z - s); }
template <class T> inline V3<T> operator-(T s, V3<T> a) { return V3<T>(s - a.x, s - a.y, s - a.z); }
template <class T> inline V3<T> operator-(V3<T> a) { return V3<T>(-a.x, -a.y, -a.z); }
template <class T> inline bool operator==(V3<T> a, V3<T> b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

template <class T> inline V2<T> operator+(V2<T> a, V2<T> b) { return V2<T>(a.x + b.x, a.y + b.y); }
template <class T> inline V2<T> operator-(V2<T> a, V2<T> b) { return V2<T>(a.x - b.x, a.y - b.y); }
template <class T> inline V2<T> operator*(V2<T> a, T s) { return V2<T>(a.x * s, a.y * s); }
template <class T> inline V2<T> operator*(T s, V2<T> a) { return V2<T>(s * a.x, s * a.y); }
template <class T> inline V2<T> operator-(V2<T> a, T s) { return V2<T>(a.x - s, a.y - s); }

// GLSL dot: x*x' + y*y' + z*z', summed left to right.
template <class T> inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline T dot(V2<T> a, V2<T> b) { return a.x * b.x + a.y * b.y; }
template <class T> inline V3<T> cross(V3<T> a, V3<T> b) {
    return V3<T>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
template <class T> inline T length(V3<T> a) { return std::sqrt(dot(a, a)); }
// normalize(v) = v / length(v), three IEEE divisions.
template <class T> inline V3<T> normalize(V3<T> a) {
    T l = length(a);
    return V3<T>(a.x / l, a.y / l, a.z / l);
}
template <class T> inline V4<T> normalize(V4<T> a) {
    T l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z + a.w * a.w);
    return V4<T>(a.x / l, a.y / l, a.z / l, a.w / l);
}
// GLSL mix(x, y, a) = x * (1 - a) + y * a
template <class T> inline T mix(T x, T y, T a) { return x * (T(1) - a) + y * a; }
template <class T> inline V3<T> mix(V3<T> x, V3<T> y, T a) {
    return V3<T>(mix(x.x, y.x, a), mix(x.y, y.y, a), mix(x.z, y.z, a));
}
template <class T> inline T gmin(T a, T b) { return std::fmin(a, b); }
template <class T> inline T gmax(T a, T b) { return std::fmax(a, b); }
template <class T> inline T clamp(T x, T lo, T hi) { return gmin(gmax(x, lo), hi); }
template <class T> inline V3<T> vmax(V3<T> a, T s) { return V3<T>(gmax(a.x, s), gmax(a.y, s), gmax(a.z, s)); }
template <class T> inline V3<T> vsqrt(V3<T> a) { return V3<T>(std::sqrt(a.x), std::sqrt(a.y), std::sqrt(a.z)); }
// GLSL reflect(I, N) = I - 2 * dot(N, I) * N
template <class T> inline V3<T> reflect(V3<T> I, V3<T> N) { return I - (T(2) * dot(N, I)) * N; }
template <class T> inline T sign(T x) { return x > T(0) ? T(1) : (x < T(0) ? T(-1) : T(0)); }

// float <-> bit casts (GLSL floatBitsToInt / intBitsToFloat / uintBitsToFloat)
inline int32_t f2i(float f) { int32_t i; std::memcpy(&i, &f, 4); return i; }
inline float i2f(int32_t i) { float f; std::memcpy(&f, &i, 4); return f; }
inline float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

// Column-major 4x4 matrix as in GLSL/glm: m[col][row].
template <class T> struct M4 {
    T m[4][4];
    V4<T> operator*(V4<T> v) const {
        // GLSL: result[row] = sum_col m[col][row] * v[col], summed col 0..3 left to right.
        T r[4];
        for (int row = 0; row < 4; row++)
            r[row] = m[0][row] * v.x + m[1][row] * v.y + m[2][row] * v.z + m[3][row] * v.w;
        return V4<T>(r[0], r[1], r[2], r[3]);
    }
};

template <class T> inline V3<T> cvt3(V3<float> v) { return V3<T>(T(v.x), T(v.y), T(v.z)); }

}  // namespace orc
