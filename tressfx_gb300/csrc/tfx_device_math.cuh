// Device-side vector / quaternion helpers shared by the simulation and SDF kernels.
//
// Every helper evaluates component-wise, left to right, in FP32.  The library is compiled with
// -fmad=false (no FMA contraction) and IEEE division / square root, so each helper produces the
// same bits as the oracle's restatement of the reference HLSL (dot = x*x' + y*y' + z*z';
// normalize(v) = v * (1 / sqrt(dot(v,v))); HLSL float literals stay float).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tfx {

struct Q4 { float x, y, z, w; };

__device__ __forceinline__ float3 mk3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 xyz(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float4 with_xyz(float4 a, float3 v) { return make_float4(v.x, v.y, v.z, a.w); }
__device__ __forceinline__ float3 add(float3 a, float3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 sub(float3 a, float3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 neg(float3 a) { return mk3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 mul(float s, float3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 mul(float3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 divs(float3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float length(float3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ float3 normalize(float3 a) {
    float inv = 1.0f / sqrtf(dot(a, a));
    return mul(a, inv);
}
__device__ __forceinline__ float3 vmin(float3 a, float3 b) { return mk3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
__device__ __forceinline__ float3 vmax(float3 a, float3 b) { return mk3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }

// D3D ftoi: truncation toward zero, saturating, NaN -> 0 (cvt.rzi.s32.f32 has exactly these rules).
__device__ __forceinline__ int ftoi(float f) { return __float2int_rz(f); }

// MultQuaternionAndVector, TressFXSimulation.hlsl:305-315
__device__ __forceinline__ float3 qrot(Q4 q, float3 v) {
    float3 qv = mk3(q.x, q.y, q.z);
    float3 uv = cross(qv, v);
    float3 uuv = cross(qv, uv);
    uv = mul(uv, 2.0f * q.w);
    uuv = mul(uuv, 2.0f);
    return add(add(v, uv), uuv);
}

// NormalizeQuaternion, TressFXSimulation.hlsl:329-342
__device__ __forceinline__ Q4 qnormalize(Q4 q) {
    float n = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
    if (n < 1e-10f) { q.w = 1.0f; return q; }
    float s = 1.0f / sqrtf(n);
    return Q4{q.x * s, q.y * s, q.z * s, q.w * s};
}

// QuatFromTwoUnitVectors, TressFXSimulation.hlsl:345-363
__device__ __forceinline__ Q4 qfrom2(float3 u, float3 v) {
    float r = 1.0f + dot(u, v);
    float3 n;
    if (r < 1e-7f) {
        r = 0.0f;
        n = fabsf(u.x) > fabsf(u.z) ? mk3(-u.y, u.x, 0.0f) : mk3(0.0f, -u.z, u.y);
    } else {
        n = cross(u, v);
    }
    return qnormalize(Q4{n.x, n.y, n.z, r});
}

// MakeQuaternion(float4x4), TressFXSimulation.hlsl:247-288; m[r][c] = row r, column c.
__device__ __forceinline__ Q4 quat_from_matrix(const float (&m)[4][4]) {
    Q4 q;
    float trace = m[0][0] + m[1][1] + m[2][2];
    if (trace > 0.0f) {
        float r = sqrtf(trace + 1.0f);
        q.w = 0.5f * r;
        r = 0.5f / r;
        q.x = (m[1][2] - m[2][1]) * r;
        q.y = (m[2][0] - m[0][2]) * r;
        q.z = (m[0][1] - m[1][0]) * r;
    } else {
        // (i,j,k) = (0,1,2), (1,2,0) or (2,0,1); unrolled selects keep m in registers.
        int i = 0;
        if (m[1][1] > m[0][0]) i = 1;
        float mii = (i == 0) ? m[0][0] : m[1][1];
        if (m[2][2] > mii) i = 2;
        float r, qi, qj, qk, w;
        if (i == 0) {
            r = sqrtf(m[0][0] - m[1][1] - m[2][2] + 1.0f);
            qi = 0.5f * r; r = 0.5f / r;
            w = (m[1][2] - m[2][1]) * r; qj = (m[1][0] + m[0][1]) * r; qk = (m[2][0] + m[0][2]) * r;
            q = Q4{qi, qj, qk, w};
        } else if (i == 1) {
            r = sqrtf(m[1][1] - m[2][2] - m[0][0] + 1.0f);
            qi = 0.5f * r; r = 0.5f / r;
            w = (m[2][0] - m[0][2]) * r; qj = (m[2][1] + m[1][2]) * r; qk = (m[0][1] + m[1][0]) * r;
            q = Q4{qk, qi, qj, w};
        } else {
            r = sqrtf(m[2][2] - m[0][0] - m[1][1] + 1.0f);
            qi = 0.5f * r; r = 0.5f / r;
            w = (m[0][1] - m[1][0]) * r; qj = (m[0][2] + m[2][0]) * r; qk = (m[1][2] + m[2][1]) * r;
            q = Q4{qj, qk, qi, w};
        }
    }
    return q;
}

// Weighted bone blend of ApplyVertexBoneSkinning (matrix path), TressFXSimulation.hlsl:550-566;
// the same blend is the first half of BoneSkinning, TressFXBoneSkinning.hlsl:67-84.
// bones: row-major 4x4 matrices, 16 floats each. skin = {boneIndex.xyzw, boneWeight.xyzw}.
__device__ __forceinline__ void blend_bones(const float4* __restrict__ bones, float4 idx, float4 wgt,
                                            float (&m)[4][4]) {
    const float wv[4] = {wgt.x, wgt.y, wgt.z, wgt.w};
    const float iv[4] = {idx.x, idx.y, idx.z, idx.w};
    {
        const float4* M = bones + 4 * ftoi(iv[0]);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            float4 row = __ldg(M + r);
            m[r][0] = row.x * wv[0]; m[r][1] = row.y * wv[0]; m[r][2] = row.z * wv[0]; m[r][3] = row.w * wv[0];
        }
    }
    float wsum = wv[0];
#pragma unroll
    for (int i = 1; i < 4; ++i) {
        if (wv[i] > 0.0f) {
            const float4* M = bones + 4 * ftoi(iv[i]);
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                float4 row = __ldg(M + r);
                m[r][0] = m[r][0] + row.x * wv[i]; m[r][1] = m[r][1] + row.y * wv[i];
                m[r][2] = m[r][2] + row.z * wv[i]; m[r][3] = m[r][3] + row.w * wv[i];
            }
            wsum = wsum + wv[i];
        }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) m[r][c] = m[r][c] / wsum;
}

// mul(float4(p, w), M).xyz for a row-major M (row-vector convention).
__device__ __forceinline__ float3 xform_row(float3 p, float w, const float (&m)[4][4]) {
    return mk3(((p.x * m[0][0] + p.y * m[1][0]) + p.z * m[2][0]) + w * m[3][0],
               ((p.x * m[0][1] + p.y * m[1][1]) + p.z * m[2][1]) + w * m[3][1],
               ((p.x * m[0][2] + p.y * m[1][2]) + p.z * m[2][2]) + w * m[3][2]);
}

struct DC { float4 p0, p1; };

// ApplyDistanceConstraint + ConstraintMultiplier, TressFXSimulation.hlsl:214-230, :377-387 (stiffness 1).
__device__ __forceinline__ DC distance_constraint(float4 p0, float4 p1, float target) {
    float3 delta = sub(xyz(p1), xyz(p0));
    const float distance = fmaxf(length(delta), 1e-7f);
    const float stretching = 1.0f - target / distance;
    delta = mul(stretching, delta);
    float m0, m1;
    if (p0.w > 0.0f) { if (p1.w > 0.0f) { m0 = 0.5f; m1 = 0.5f; } else { m0 = 1.0f; m1 = 0.0f; } }
    else { if (p1.w > 0.0f) { m0 = 0.0f; m1 = 1.0f; } else { m0 = 0.0f; m1 = 0.0f; } }
    const float3 a = mul(mul(m0, delta), 1.0f);
    const float3 b = mul(mul(m1, delta), 1.0f);
    p0.x = p0.x + a.x; p0.y = p0.y + a.y; p0.z = p0.z + a.z;
    p1.x = p1.x - b.x; p1.y = p1.y - b.y; p1.z = p1.z - b.z;
    return DC{p0, p1};
}

static constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ float4 shfl4(float4 v, int src) {
    return make_float4(__shfl_sync(FULL, v.x, src), __shfl_sync(FULL, v.y, src), __shfl_sync(FULL, v.z, src),
                       __shfl_sync(FULL, v.w, src));
}
__device__ __forceinline__ float4 shfl4_down(float4 v, int d) {
    return make_float4(__shfl_down_sync(FULL, v.x, d), __shfl_down_sync(FULL, v.y, d), __shfl_down_sync(FULL, v.z, d),
                       __shfl_down_sync(FULL, v.w, d));
}
__device__ __forceinline__ float4 shfl4_up(float4 v, int d) {
    return make_float4(__shfl_up_sync(FULL, v.x, d), __shfl_up_sync(FULL, v.y, d), __shfl_up_sync(FULL, v.z, d),
                       __shfl_up_sync(FULL, v.w, d));
}

}  // namespace tfx
