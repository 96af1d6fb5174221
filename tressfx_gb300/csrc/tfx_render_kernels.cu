// Rendering-side kernels on the simulated buffers, headless: the strand quad expansion of the hair
// vertex shader (TressFXStrands.hlsl) into a device vertex buffer.
#include "tfx_device_math.cuh"
#include "tfx_internal.h"

namespace tfx {
namespace {

// Safe_normalize (TressFXUtilities.hlsl:104-119): v * rcp(|v|) when |v| >= 1e-7, else 0 (rcp = the
// IEEE reciprocal).
__device__ __forceinline__ float3 safe_normalize3(float3 v) {
    const float len = sqrtf(dot(v, v));
    if (!(len >= 1e-7f)) return mk3(0.f, 0.f, 0.f);
    return mul(v, 1.0f / len);
}
__device__ __forceinline__ float2 safe_normalize2(float2 v) {
    const float len = sqrtf(v.x * v.x + v.y * v.y);
    if (!(len >= 1e-7f)) return make_float2(0.f, 0.f);
    const float r = 1.0f / len;
    return make_float2(v.x * r, v.y * r);
}
// mul(M, v) for a row-major M: r[i] = ((M[i][0] v.x + M[i][1] v.y) + M[i][2] v.z) + M[i][3] v.w
__device__ __forceinline__ float4 mul_mv(const ExpandParams& P, float4 v) {
    float o[4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
        o[r] = ((P.viewProj[4 * r] * v.x + P.viewProj[4 * r + 1] * v.y) + P.viewProj[4 * r + 2] * v.z) +
               P.viewProj[4 * r + 3] * v.w;
    return make_float4(o[0], o[1], o[2], o[3]);
}

// GetExpandedTressFXVert / GetExpandedTressFXShadowVert for one vertex id: out[id] = {Position,
// Tangent, p0p1, StrandColor}; the shadow form writes the position and zeros.  lerp(x, y, s) =
// x + s (y - x); the albedo texture is white.
__global__ void __launch_bounds__(256) k_expand_strands(const float4* __restrict__ pos, const float4* __restrict__ tan,
                                                        int64_t vtot, ExpandParams P, float4* __restrict__ out) {
    const int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (id >= 2 * vtot) return;
    const uint32_t vid = (uint32_t)id;
    const int64_t index = vid / 2;
    const float3 v = xyz(pos[index]);
    const float3 t = xyz(tan[index]);
    const uint32_t inStrand = (uint32_t)(index % P.n);
    const float fraction = (float)inStrand / (float)(P.n - 1);
    const float ratio = P.enableThinTip > 0 ? 1.0f + fraction * (P.fiberRatio - 1.0f) : 1.0f;
    const float3 right = safe_normalize3(cross(t, safe_normalize3(sub(v, mk3(P.eye[0], P.eye[1], P.eye[2])))));
    const float4 pr = mul_mv(P, make_float4(right.x, right.y, right.z, 0.0f));
    const float2 projRight = safe_normalize2(make_float2(pr.x, pr.y));
    const float expandPixels = P.shadow ? 1.0f : 0.71f;
    const float3 p0 = add(v, mul(mul(mul(right, -1.0f), ratio), P.fiberRadius));
    const float3 p1 = add(v, mul(mul(mul(right, 1.0f), ratio), P.fiberRadius));
    const float4 e0 = mul_mv(P, make_float4(p0.x, p0.y, p0.z, 1.0f));
    const float4 e1 = mul_mv(P, make_float4(p1.x, p1.y, p1.z, 1.0f));
    const bool odd = (vid & 1u) != 0;
    const float fDir = odd ? -1.0f : 1.0f;
    const float4 sel = odd ? e0 : e1;
    const float ox = (projRight.x * expandPixels) / P.winH, oy = (projRight.y * expandPixels) / P.winH;
    float4* o = out + 4 * id;
    o[0] = make_float4(sel.x + (fDir * ox) * sel.w, sel.y + (fDir * oy) * sel.w, sel.z + (fDir * 0.0f) * sel.w,
                       sel.w + (fDir * 0.0f) * sel.w);
    if (P.shadow) {
        o[1] = o[2] = o[3] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    o[1] = make_float4(t.x, t.y, t.z, odd ? 0.0f : 1.0f);
    const float w0 = fmaxf(e0.w, 1e-7f), w1 = fmaxf(e1.w, 1e-7f);
    o[2] = make_float4(e0.x / w0, e0.y / w0, e1.x / w1, e1.y / w1);
    const float3 root = mk3(1.0f * P.baseColor[0], 1.0f * P.baseColor[1], 1.0f * P.baseColor[2]);
    const float3 tip = mk3(P.tipColor[0], P.tipColor[1], P.tipColor[2]);
    const float3 col = fraction > 1.0f - P.tipPercentage ? add(root, mul(sub(tip, root), fraction)) : root;
    o[3] = make_float4(col.x, col.y, col.z, fraction);
}

}  // namespace

cudaError_t launch_expand_strands(const float4* pos, const float4* tan, int64_t vtot, const ExpandParams& P, float4* out,
                                  cudaStream_t s) {
    if (vtot <= 0) return cudaSuccess;
    k_expand_strands<<<(unsigned)((2 * vtot + 255) / 256), 256, 0, s>>>(pos, tan, vtot, P, out);
    return cudaGetLastError();
}

}  // namespace tfx
