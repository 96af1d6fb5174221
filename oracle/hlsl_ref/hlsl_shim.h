// HLSL-in-C++ shim: the types, swizzles, intrinsics and resource objects that the reference's
// compute shaders use, so that their own source (mechanically rewritten by translate.py) compiles
// with g++ and runs on the CPU.  Test infrastructure only: it exists to pin the oracle against the
// reference's shader code.
//
// Intrinsic semantics are fixed here once (the reference does not define them beyond HLSL's
// loose rules) and are the same ones the oracle restatement and the CUDA kernels use:
//   dot = left-to-right sum of products; length = sqrt(dot); normalize(v) = v * (1 / length(v));
//   mul(v, M)[c] = ((v.x*M[0][c] + v.y*M[1][c]) + v.z*M[2][c]) + v.w*M[3][c];
//   min / max = IEEE minNum / maxNum; exp / sqrt / sin / cos = the C library's float versions;
//   integer min / max as usual.  Build with -ffp-contract=off (no FMA contraction).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

typedef unsigned int uint;

struct float3;
struct float4;

// A three-component view (.xyz) over the first three floats of a float3 or float4.
template <int N>
struct SwzXYZ {
    float e[N];
    inline operator float3() const;
    inline SwzXYZ& operator=(const float3& v);
    inline SwzXYZ& operator=(const SwzXYZ& v);
    inline SwzXYZ& operator+=(const float3& v);
    inline SwzXYZ& operator-=(const float3& v);
    inline SwzXYZ& operator*=(float s);
};

// A two-component view (.xy) over the first two floats of a float2 or float4.
template <int N>
struct SwzXY {
    float e[N];
    inline operator struct float2() const;
};

struct float2 {
    union {
        struct { float x, y; };
        SwzXY<2> xy;
    };
    float2() : x(0), y(0) {}
    float2(float a, float b) : x(a), y(b) {}
    float2(const float2& o) : x(o.x), y(o.y) {}
    template <int N> float2(const SwzXY<N>& s) : x(s.e[0]), y(s.e[1]) {}
    float2& operator=(const float2& o) { x = o.x; y = o.y; return *this; }
    float& operator[](int i) { return (&x)[i]; }
    float operator[](int i) const { return (&x)[i]; }
};
template <int N> inline SwzXY<N>::operator float2() const { return float2(e[0], e[1]); }

struct float3 {
    union {
        struct { float x, y, z; };
        SwzXYZ<3> xyz;
    };
    float3() : x(0), y(0), z(0) {}
    float3(float a, float b, float c) : x(a), y(b), z(c) {}
    float3(const float3& o) : x(o.x), y(o.y), z(o.z) {}
    inline float3(const float4& o);   // HLSL truncation float4 -> float3
    template <int N> float3(const SwzXYZ<N>& s) : x(s.e[0]), y(s.e[1]), z(s.e[2]) {}
    float3& operator=(const float3& o) { x = o.x; y = o.y; z = o.z; return *this; }
    float& operator[](int i) { return (&x)[i]; }
    float operator[](int i) const { return (&x)[i]; }
};

struct float4 {
    union {
        struct { float x, y, z, w; };
        SwzXYZ<4> xyz;
        SwzXY<4> xy;
    };
    float4() : x(0), y(0), z(0), w(0) {}
    float4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    float4(const float3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    float4(const float2& v, float c, float d) : x(v.x), y(v.y), z(c), w(d) {}
    float4(const float2& a, const float2& b) : x(a.x), y(a.y), z(b.x), w(b.y) {}
    float4(const float4& o) : x(o.x), y(o.y), z(o.z), w(o.w) {}
    float4& operator=(const float4& o) { x = o.x; y = o.y; z = o.z; w = o.w; return *this; }
    float& operator[](int i) { return (&x)[i]; }
    float operator[](int i) const { return (&x)[i]; }
    float4& operator*=(float s) { x = x * s; y = y * s; z = z * s; w = w * s; return *this; }
};

inline float3::float3(const float4& o) : x(o.x), y(o.y), z(o.z) {}

template <int N> inline SwzXYZ<N>::operator float3() const { return float3(e[0], e[1], e[2]); }
template <int N> inline SwzXYZ<N>& SwzXYZ<N>::operator=(const float3& v) { e[0] = v.x; e[1] = v.y; e[2] = v.z; return *this; }
template <int N> inline SwzXYZ<N>& SwzXYZ<N>::operator=(const SwzXYZ& v) { float3 t(v); return *this = t; }
template <int N> inline SwzXYZ<N>& SwzXYZ<N>::operator+=(const float3& v) { e[0] = e[0] + v.x; e[1] = e[1] + v.y; e[2] = e[2] + v.z; return *this; }
template <int N> inline SwzXYZ<N>& SwzXYZ<N>::operator-=(const float3& v) { e[0] = e[0] - v.x; e[1] = e[1] - v.y; e[2] = e[2] - v.z; return *this; }
template <int N> inline SwzXYZ<N>& SwzXYZ<N>::operator*=(float s) { e[0] = e[0] * s; e[1] = e[1] * s; e[2] = e[2] * s; return *this; }

// float3 arithmetic (non-template, so swizzle views and float4 convert implicitly)
inline float3 operator+(const float3& a, const float3& b) { return float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(const float3& a, const float3& b) { return float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator*(const float3& a, const float3& b) { return float3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float3 operator/(const float3& a, const float3& b) { return float3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline float3 operator*(const float3& a, float s) { return float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator*(float s, const float3& a) { return float3(s * a.x, s * a.y, s * a.z); }
inline float3 operator/(const float3& a, float s) { return float3(a.x / s, a.y / s, a.z / s); }
inline float3 operator-(const float3& a) { return float3(-a.x, -a.y, -a.z); }
inline float3& operator+=(float3& a, const float3& b) { a = a + b; return a; }
inline float3& operator-=(float3& a, const float3& b) { a = a - b; return a; }
inline float3& operator*=(float3& a, float s) { a = a * s; return a; }
inline float3& operator/=(float3& a, float s) { a = a / s; return a; }

inline float4 operator+(const float4& a, const float4& b) { return float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline float4 operator-(const float4& a, const float4& b) { return float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline float4 operator*(const float4& a, float s) { return float4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline float4 operator*(float s, const float4& a) { return float4(s * a.x, s * a.y, s * a.z, s * a.w); }
inline float4 operator/(const float4& a, float s) { return float4(a.x / s, a.y / s, a.z / s, a.w / s); }

struct int3 {
    int x, y, z;
    int3() : x(0), y(0), z(0) {}
    int3(int a, int b, int c) : x(a), y(b), z(c) {}
};
inline int3 operator-(const int3& a, const int3& b) { return int3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline int3 operator+(const int3& a, const int3& b) { return int3(a.x + b.x, a.y + b.y, a.z + b.z); }

struct int2 {
    int x, y;
};

struct uint3 {
    uint x, y, z;
    uint3() : x(0), y(0), z(0) {}
    uint3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
};

struct int4 {
    int x, y, z, w;
    int& operator[](int i) { return (&x)[i]; }
};

// float4x4: m[r][c] = row r, column c (HLSL logical indexing, independent of the packing qualifier)
struct float4x4 {
    union {
        float m[4][4];
        struct { float _m00, _m01, _m02, _m03, _m10, _m11, _m12, _m13, _m20, _m21, _m22, _m23, _m30, _m31, _m32, _m33; };
    };
    float4x4() { std::memset(m, 0, sizeof(m)); }
    float4x4(const float4x4& o) { std::memcpy(m, o.m, sizeof(m)); }
    float4x4& operator=(const float4x4& o) { std::memcpy(m, o.m, sizeof(m)); return *this; }
    float4& operator[](int r) { return *reinterpret_cast<float4*>(m[r]); }
    const float4& operator[](int r) const { return *reinterpret_cast<const float4*>(m[r]); }
    float4x4& operator+=(const float4x4& o) {
        for (int r = 0; r < 4; ++r) for (int c = 0; c < 4; ++c) m[r][c] = m[r][c] + o.m[r][c];
        return *this;
    }
    float4x4& operator/=(float s) {
        for (int r = 0; r < 4; ++r) for (int c = 0; c < 4; ++c) m[r][c] = m[r][c] / s;
        return *this;
    }
};
inline float4x4 operator*(const float4x4& a, float s) {
    float4x4 o;
    for (int r = 0; r < 4; ++r) for (int c = 0; c < 4; ++c) o.m[r][c] = a.m[r][c] * s;
    return o;
}
// mul(M, v) (column vector): r[i] = ((M[i][0]*v.x + M[i][1]*v.y) + M[i][2]*v.z) + M[i][3]*v.w
inline float4 mul(const float4x4& M, const float4& v) {
    float o[4];
    for (int r = 0; r < 4; ++r) o[r] = ((M.m[r][0] * v.x + M.m[r][1] * v.y) + M.m[r][2] * v.z) + M.m[r][3] * v.w;
    return float4(o[0], o[1], o[2], o[3]);
}
inline float4 mul(const float4& v, const float4x4& M) {
    float o[4];
    for (int c = 0; c < 4; ++c) o[c] = ((v.x * M.m[0][c] + v.y * M.m[1][c]) + v.z * M.m[2][c]) + v.w * M.m[3][c];
    return float4(o[0], o[1], o[2], o[3]);
}

// ------------------------------------------------------------------------------------ intrinsics
inline float2 operator*(const float2& a, float s) { return float2(a.x * s, a.y * s); }
inline float2 operator/(const float2& a, float s) { return float2(a.x / s, a.y / s); }
inline float length(const float2& a) { return std::sqrt(a.x * a.x + a.y * a.y); }
inline float3& operator*=(float3& a, const float3& b) { a = a * b; return a; }
inline float4 operator*(const float4& a, const float4& b) { return float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
// rcp: the IEEE reciprocal; lerp(x, y, s) = x + s * (y - x)
inline float rcp(float a) { return 1.0f / a; }
inline float lerp(float x, float y, float s) { return x + s * (y - x); }
inline float3 lerp(const float3& x, const float3& y, float s) { return x + (y - x) * s; }
struct SamplerState {};
// Texture sampling is a graphics operation; here every texture is white.
template <class T> struct Texture2D {
    T SampleLevel(const SamplerState&, const float2&, float) const { return T(1.0f, 1.0f, 1.0f, 1.0f); }
};
inline float dot(const float3& a, const float3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float3 cross(const float3& a, const float3& b) {
    return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(const float3& a) { return std::sqrt(dot(a, a)); }
inline float length(const float4& a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z + a.w * a.w); }
inline float3 normalize(const float3& a) { float inv = 1.0f / std::sqrt(dot(a, a)); return a * inv; }
inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline float3 min(const float3& a, const float3& b) { return float3(std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)); }
inline float3 max(const float3& a, const float3& b) { return float3(std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)); }
inline float abs(float a) { return std::fabs(a); }
inline float sqrt(float a) { return std::sqrt(a); }
inline float exp(float a) { return std::exp(a); }
inline float sin(float a) { return std::sin(a); }
inline float cos(float a) { return std::cos(a); }
inline float floor(float a) { return std::floor(a); }
inline uint asuint(float f) { uint u; std::memcpy(&u, &f, 4); return u; }
inline float asfloat(uint u) { float f; std::memcpy(&f, &u, 4); return f; }

// ------------------------------------------------------------------------------------ resources
// RWStructuredBuffer / StructuredBuffer with D3D out-of-bounds rules: reads return zero, writes
// are discarded.
template <class T>
struct RWStructuredBuffer {
    T* data = nullptr;
    int64_t count = 0;
    T dummy;
    template <class I> T& operator[](I i) {
        int64_t k = (int64_t)i;
        if (k >= 0 && k < count) return data[k];
        std::memset((void*)&dummy, 0, sizeof(T));
        return dummy;
    }
    void GetDimensions(uint& n, uint& stride) { n = (uint)count; stride = (uint)sizeof(T); }
    void bind(void* p, int64_t n) { data = (T*)p; count = n; }
};
template <class T> using StructuredBuffer = RWStructuredBuffer<T>;

// constant-buffer arrays may be indexed with a float (converted to uint)
template <class T, int N>
struct HArray {
    T a[N];
    template <class I> T& operator[](I i) { return a[(int64_t)i]; }
};

inline void InterlockedMin(uint& dest, uint value) { if (value < dest) dest = value; }
// InterlockedAdd(dest, value, original): threads of a dispatch run one at a time here.
template <class D, class V, class O> inline void InterlockedAdd(D& dest, V value, O& original) {
    original = (O)dest;
    dest = (D)(dest + value);
}

// Group barrier: provided by the fiber scheduler of the dispatch emulator.
void GroupMemoryBarrierWithGroupSync();
