// Types and constants shared by the C++ host classes (the reference's TressFXCommon.h, AMD_Types.h,
// AMD_TressFX.h and Math/Vector3D.h, reduced to what the simulation / SDF host code uses).
// The host classes sit on the C ABI of tressfx_gb300.h; link with libtressfx_host.so.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "../tressfx_gb300.h"

#define AMD_TRESSFX_VERSION_MAJOR 4                 /* AMD_TressFX.h:33 */
#define AMD_TRESSFX_MAX_NUM_BONES TFX_MAX_BONES     /* AMD_TressFX.h:45-47 */
#define TRESSFX_SIM_THREAD_GROUP_SIZE TFX_THREAD_GROUP_SIZE
#define TRESSFX_MAX_INFLUENTIAL_BONE_COUNT 4         /* TressFXAsset.h:37 */

namespace AMD {
typedef int32_t int32;
typedef uint32_t uint32;
typedef uint8_t uint8;
typedef float real32;
struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; };
// 16 floats, row-major, row-vector convention (p' = [p 1] * M), as the simulation shaders read the
// bone matrices (row_major float4x4 g_BoneSkinningMatrix[], TressFXSimulation.hlsl:70).
struct float4x4 { float m[16]; };
}  // namespace AMD

// A 16-byte (x, y, z, w) vector with the float arithmetic of the reference's Vector3
// (Math/Vector3D.cpp): component-wise x, y, z; w carried by copies only.  Vectors built from three
// components get w = 0 here (the reference leaves it unset).
struct Vector3 {
    float x = 0.0f, y = 0.0f, z = 0.0f, w = 0.0f;
    Vector3() = default;
    Vector3(float x_, float y_, float z_) : x(x_), y(y_), z(z_), w(0.0f) {}
    Vector3(float x_, float y_, float z_, float w_) : x(x_), y(y_), z(z_), w(w_) {}
    void Set(float x_, float y_, float z_) { x = x_; y = y_; z = z_; }
    float& operator[](int i) { return (&x)[i]; }
    float operator[](int i) const { return (&x)[i]; }
    Vector3 operator-(const Vector3& o) const { return Vector3(x - o.x, y - o.y, z - o.z); }
    Vector3 operator+(const Vector3& o) const { return Vector3(x + o.x, y + o.y, z + o.z); }
    Vector3 operator*(float s) const { Vector3 v(*this); v.x *= s; v.y *= s; v.z *= s; return v; }
    Vector3& operator-=(const Vector3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    Vector3& operator+=(const Vector3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    Vector3& operator=(float s) { x = s; y = s; z = s; return *this; }
    float Length() const { return std::sqrt(x * x + y * y + z * z); }
    // Vector3::Normalize (Math/Vector3D.cpp:48-62): divide by the length unless it is zero.
    Vector3& Normalize() {
        const float d = std::sqrt(x * x + y * y + z * z);
        if (d == 0) return *this;
        x = x / d; y = y / d; z = z / d;
        return *this;
    }
};
inline Vector3 operator*(float s, const Vector3& v) { return v * s; }

// The reference's TressFXNonCopyable (TressFXCommon.h).
class TressFXNonCopyable {
protected:
    TressFXNonCopyable() = default;
    ~TressFXNonCopyable() = default;
public:
    TressFXNonCopyable(const TressFXNonCopyable&) = delete;
    TressFXNonCopyable& operator=(const TressFXNonCopyable&) = delete;
};

// Thrown by the host classes where the reference asserts: carries the tfx_status of the failing
// C-ABI call and its message.
class TressFXError : public std::runtime_error {
public:
    TressFXError(int status, const std::string& what) : std::runtime_error(what), m_status(status) {}
    int status() const { return m_status; }
private:
    int m_status;
};
