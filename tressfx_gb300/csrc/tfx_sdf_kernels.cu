// Signed-distance-field kernels of the plain path (src/Shaders/TressFXSDFCollision.hlsl) and the
// collision-mesh bone skinning kernel (src/Shaders/TressFXBoneSkinning.hlsl:57-94).
//
// The SDF grid is uint32[X*Y*Z] holding FloatFlip3-encoded distances while it is built (atomicMin
// over the encoding = min |d|, ties to the positive value) and plain floats after Finalize.
// atomicMin is order independent, and the distance arithmetic below is the reference's in the
// same order with no FMA contraction, so the finished grid matches the oracle bit for bit.
#include <atomic>

#include "tfx_sdf_math.cuh"

namespace tfx {

// --------------------------------------------------------------------------------------------
// InitializeSignedDistanceField, :301-312 (vectorised: 4 cells per 16 B store)
__global__ void __launch_bounds__(256) k_sdf_initialize(uint32_t* __restrict__ sdf, long long cells) {
    const uint32_t v = float_flip3(1e10f);
    const long long n4 = cells >> 2;
    const long long stride = (long long)gridDim.x * blockDim.x;
    uint4* s4 = reinterpret_cast<uint4*>(sdf);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += stride) s4[i] = make_uint4(v, v, v, v);
    for (long long i = (n4 << 2) + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cells; i += stride) sdf[i] = v;
}

// ConstructSignedDistanceField, :329-397.  Each warp takes chunks of `per` (<= 32) consecutive
// triangles (sdf_construct_chunk_warp: STAGED, lane k makes the job of the chunk's k-th triangle), then
// runs the triangles' cell loops in turn; the warps stride over the chunks.
template <bool STAGED>
__global__ void __launch_bounds__(128) k_sdf_construct(uint32_t* __restrict__ sdf, SdfGrid g,
                                                       const float4* __restrict__ mesh,
                                                       const uint32_t* __restrict__ idx, int ntri, int per) {
    __shared__ TriJob jobs[STAGED ? 4 : 1][STAGED ? kTriJobsPerWarp : 1];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int warpsTotal = gridDim.x * (blockDim.x >> 5);
    const int chunks = (ntri + per - 1) / per;
    for (int k = blockIdx.x * (blockDim.x >> 5) + warp; k < chunks; k += warpsTotal) {
        const int first = k * per;
        sdf_construct_chunk_warp<STAGED>(jobs[STAGED ? warp : 0], first, min(per, ntri - first), lane, [&](int t) {
            const float3 x0 = xyz(__ldg(mesh + 2 * (size_t)__ldg(idx + 3 * t + 0)));
            const float3 x1 = xyz(__ldg(mesh + 2 * (size_t)__ldg(idx + 3 * t + 1)));
            const float3 x2 = xyz(__ldg(mesh + 2 * (size_t)__ldg(idx + 3 * t + 2)));
            return tri_job(g, sdf, x0, x1, x2);
        });
    }
}

// FinalizeSignedDistanceField, :400-412 (vectorised)
__global__ void __launch_bounds__(256) k_sdf_finalize(uint32_t* __restrict__ sdf, long long cells) {
    const long long n4 = cells >> 2;
    const long long stride = (long long)gridDim.x * blockDim.x;
    uint4* s4 = reinterpret_cast<uint4*>(sdf);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += stride) {
        uint4 u = s4[i];
        s4[i] = make_uint4(ifloat_flip3(u.x), ifloat_flip3(u.y), ifloat_flip3(u.z), ifloat_flip3(u.w));
    }
    for (long long i = (n4 << 2) + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cells; i += stride)
        sdf[i] = ifloat_flip3(sdf[i]);
}

// CollideHairVerticesWithSdf_forward, :531-595.  One thread per hair vertex (guides and follows).
__global__ void __launch_bounds__(256) k_sdf_collide(const float* __restrict__ sdf, SdfGrid g, float margin,
                                                     float4* __restrict__ pos, float4* __restrict__ prev,
                                                     int n, long long vtot) {
    const long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (v >= vtot) return;
    const int local = (int)(v % n);
    if (local == 0 || local == 1) return;
    const float4 hv = pos[v];
    const float3 p = xyz(hv);
    const float distance = sdf_lookup(sdf, g, p);
    if (distance > margin) return;
    const float h = 0.1f * g.cell;
    const float fx = sdf_lookup(sdf, g, add(p, mul(mk3(1.0f, 0.0f, 0.0f), h)));
    const float fy = sdf_lookup(sdf, g, add(p, mul(mk3(0.0f, 1.0f, 0.0f), h)));
    const float fz = sdf_lookup(sdf, g, add(p, mul(mk3(0.0f, 0.0f, 1.0f), h)));
    const float3 grad = mk3((fx - distance) / h, (fy - distance) / h, (fz - distance) / h);
    const float3 nrm = normalize(grad);
    if (distance < margin) {
        const float3 proj = add(p, mul(nrm, margin - distance));
        pos[v] = with_xyz(hv, proj);
        const float4 pv = prev[v];
        prev[v] = with_xyz(pv, proj);
    }
}

// BoneSkinning, src/Shaders/TressFXBoneSkinning.hlsl:57-94.  One thread per mesh vertex.
// in/out: {float4 position, float4 normal}; skin: {float4 boneIndex, float4 boneWeight}.
// CollideHairVerticesWithSdf (TressFXSDFCollision.hlsl:599-715), the mixed-difference variant: one
// thread per vertex (roots included), one 8-corner fetch, the gradient by forward or backward
// differences within the same cell (h = 0.1 * cellSize added to the cell-normalised coordinates,
// as the shader writes it).
__global__ void __launch_bounds__(256) k_sdf_collide_mixed(const float* __restrict__ sdf, SdfGrid g, float margin,
                                                           float4* __restrict__ pos, float4* __restrict__ prev,
                                                           int64_t vtot) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= vtot) return;
    const float4 hv = pos[v];
    const float3 p = xyz(hv);
    const int3 gc = sdf_coords(g, p);
    if (!(0 <= gc.x && gc.x < g.nx - 2) || !(0 <= gc.y && gc.y < g.ny - 2) || !(0 <= gc.z && gc.z < g.nz - 2)) return;
    const long long X = 1, Y = g.nx, Z = (long long)g.ny * g.nx;
    const long long base = Z * gc.z + Y * gc.y + gc.x;
    const long long off[8] = {0, X, Y, Y + X, Z, Z + X, Z + Y, Z + Y + X};
    float d[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        d[j] = __ldg(sdf + base + off[j]);
        if (d[j] == 1e10f) return;
    }
    auto tri = [&](float x, float y, float z) {
        const float b0 = lerp_ref(lerp_ref(d[0], d[1], x), lerp_ref(d[2], d[3], x), y);
        const float b1 = lerp_ref(lerp_ref(d[4], d[5], x), lerp_ref(d[6], d[7], x), y);
        return lerp_ref(b0, b1, z);
    };
    const float3 cp = sdf_cell_pos(g, gc.x, gc.y, gc.z);
    const float3 ip = divs(sub(p, cp), g.cell);
    const float dist = tri(ip.x, ip.y, ip.z);
    const float h = 0.1f * g.cell;
    const float3 dir = mk3((ip.x + h < 1.0f) ? 1.0f : -1.0f, (ip.y + h < 1.0f) ? 1.0f : -1.0f, (ip.z + h < 1.0f) ? 1.0f : -1.0f);
    const float3 nd = mk3(tri(ip.x + h * dir.x, ip.y, ip.z), tri(ip.x, ip.y + h * dir.y, ip.z), tri(ip.x, ip.y, ip.z + h * dir.z));
    const float3 grad = mk3((dir.x * (nd.x - dist)) / h, (dir.y * (nd.y - dist)) / h, (dir.z * (nd.z - dist)) / h);
    const float3 nrm = normalize(grad);
    if (dist < margin) {
        const float3 proj = add(p, mul(nrm, margin - dist));
        pos[v] = with_xyz(hv, proj);
        prev[v] = with_xyz(prev[v], proj);
    }
}

__global__ void __launch_bounds__(256) k_mesh_skin(float4* __restrict__ out, const float4* __restrict__ in,
                                                   const float4* __restrict__ skin, const float4* __restrict__ bones,
                                                   int nverts) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nverts) return;
    const float4 p = __ldg(in + 2 * v), nr = __ldg(in + 2 * v + 1);
    float m[4][4];
    blend_bones(bones, __ldg(skin + 2 * v), __ldg(skin + 2 * v + 1), m);
    out[2 * v] = with_xyz(p, xform_row(xyz(p), 1.0f, m));
    out[2 * v + 1] = with_xyz(nr, xform_row(xyz(nr), 0.0f, m));
}

// --------------------------------------------------------------------------------------------
int sm_count() {
    constexpr int kMaxDevices = 64;
    static std::atomic<int> cache[kMaxDevices];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 1;
    int v = cache[dev].load(std::memory_order_relaxed);
    if (v <= 0) {
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) return 1;
        cache[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

static inline unsigned grid_for(long long work, int threads, unsigned cap) {
    long long b = (work + threads - 1) / threads;
    if (b < 1) b = 1;
    return (unsigned)(b > cap ? cap : b);
}

cudaError_t launch_sdf_initialize(uint32_t* sdf, int64_t cells, cudaStream_t s) {
    if (cells <= 0) return cudaSuccess;
    k_sdf_initialize<<<grid_for((cells + 3) / 4, 256, sm_count() * 16), 256, 0, s>>>(sdf, cells);
    return cudaGetLastError();
}

cudaError_t launch_sdf_construct(uint32_t* sdf, const SdfGrid& g, const float4* mesh, const uint32_t* idx, int ntri,
                                 cudaStream_t s) {
    if (ntri <= 0) return cudaSuccess;
    const int per = sdf_construct_chunk(ntri, sm_count());
    const long long chunks = ((long long)ntri + per - 1) / per;
    const unsigned blocks = (unsigned)std::min<long long>((chunks + 3) / 4, (long long)sm_count() * 64);
    if (per >= kTriJobsStagedFrom)
        k_sdf_construct<true><<<blocks, 128, 0, s>>>(sdf, g, mesh, idx, ntri, per);
    else
        k_sdf_construct<false><<<blocks, 128, 0, s>>>(sdf, g, mesh, idx, ntri, per);
    return cudaGetLastError();
}

cudaError_t launch_sdf_finalize(uint32_t* sdf, int64_t cells, cudaStream_t s) {
    if (cells <= 0) return cudaSuccess;
    k_sdf_finalize<<<grid_for((cells + 3) / 4, 256, sm_count() * 16), 256, 0, s>>>(sdf, cells);
    return cudaGetLastError();
}

cudaError_t launch_sdf_collide(const uint32_t* sdf, const SdfGrid& g, float margin, float4* pos, float4* prev, int n,
                               int64_t vtot, cudaStream_t s) {
    if (vtot <= 0) return cudaSuccess;
    k_sdf_collide<<<(unsigned)((vtot + 255) / 256), 256, 0, s>>>(reinterpret_cast<const float*>(sdf), g, margin, pos,
                                                                 prev, n, vtot);
    return cudaGetLastError();
}

cudaError_t launch_sdf_collide_mixed(const uint32_t* sdf, const SdfGrid& g, float margin, float4* pos, float4* prev,
                                     int64_t vtot, cudaStream_t s) {
    if (vtot <= 0) return cudaSuccess;
    k_sdf_collide_mixed<<<(unsigned)((vtot + 255) / 256), 256, 0, s>>>(reinterpret_cast<const float*>(sdf), g, margin, pos,
                                                                       prev, vtot);
    return cudaGetLastError();
}

cudaError_t launch_mesh_skin(float4* out, const float4* in, const float4* skin, const float4* bones, int nverts,
                             cudaStream_t s) {
    if (nverts <= 0) return cudaSuccess;
    k_mesh_skin<<<(nverts + 255) / 256, 256, 0, s>>>(out, in, skin, bones, nverts);
    return cudaGetLastError();
}

}  // namespace tfx
