// Device-side SDF helpers shared by the plain SDF kernels and the batched (tiled) build / fused
// collide: FloatFlip3 encoding, grid coordinates, signed point-triangle distance and the
// trilinear lookup of src/Shaders/TressFXSDFCollision.hlsl, evaluated in the reference's order.
#pragma once
#include "tfx_device_math.cuh"
#include "tfx_internal.h"

namespace tfx {

// FloatFlip3 / IFloatFlip3, TressFXSDFCollision.hlsl:92-100
__device__ __forceinline__ uint32_t float_flip3(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u << 1) | (u >> 31);
}
__device__ __forceinline__ uint32_t ifloat_flip3(uint32_t u) { return (u >> 1) | (u << 31); }

// True when p certainly fails the lookup's bounds test 0 <= ftoi((p - origin) / cell) < dims - 2 on
// some axis, decided without the division.  d = p - origin is the reference's own first operation;
// d <= -2 cell (exact product) gives a quotient <= -2, and d >= RN(dims * cell) >= dims * cell *
// (1 - 2^-24) gives a quotient that truncates to dims - 1 or more (division is monotonic, dims is far
// below 2^22).  Infinite d goes the same way as the reference (its quotient saturates); NaN and the
// points near the range's faces take the exact path.
__device__ __forceinline__ bool sdf_surely_outside(const SdfGrid& g, float3 p) {
    const float dx = p.x - g.ox, dy = p.y - g.oy, dz = p.z - g.oz;
    const float lo = -2.0f * g.cell;
    return dx <= lo || dy <= lo || dz <= lo || dx >= (float)g.nx * g.cell || dy >= (float)g.ny * g.cell ||
           dz >= (float)g.nz * g.cell;
}

// GetSdfCoordinates, :103-113
__device__ __forceinline__ int3 sdf_coords(const SdfGrid& g, float3 p) {
    const float sx = (p.x - g.ox) / g.cell, sy = (p.y - g.oy) / g.cell, sz = (p.z - g.oz) / g.cell;
    return make_int3(ftoi(sx), ftoi(sy), ftoi(sz));
}
// GetSdfCellPosition, :115-121
__device__ __forceinline__ float3 sdf_cell_pos(const SdfGrid& g, int x, int y, int z) {
    const float3 c = mk3((float)x * g.cell, (float)y * g.cell, (float)z * g.cell);
    return add(c, mk3(g.ox, g.oy, g.oz));
}

// SignedDistancePointToTriangle (:163-215) and DistancePointToEdge (:147-159) split in two: the
// triangle-only terms, computed once per triangle, and signed_dist_pre(p, T), the per-cell part.
// Every term is the shader's expression on the same inputs in the same order, so the distance is
// bit-identical to evaluating the two functions per cell.
struct TriPre {
    float3 x0, x1, x2;
    float3 x02n, x12n;   // normalised edge frame
    float l0, l1, l2;
    float3 nTri;
    float3 e01, e12, e02; // x1-x0, x2-x1, x2-x0 (the x10 of the three edge calls)
    float d01, d12, d02;  // dot(x10, x10) of the three edge calls
};

__device__ __forceinline__ TriPre tri_pre(float3 x0, float3 x1, float3 x2) {
    TriPre T;
    T.x0 = x0; T.x1 = x1; T.x2 = x2;
    float3 x02 = sub(x0, x2);
    T.l0 = length(x02) + 1e-30f;
    T.x02n = divs(x02, T.l0);
    float3 x12 = sub(x1, x2);
    T.l1 = dot(x12, T.x02n);
    x12 = sub(x12, mul(T.l1, T.x02n));
    T.l2 = length(x12) + 1e-30f;
    T.x12n = divs(x12, T.l2);
    T.nTri = cross(sub(x1, x0), sub(x2, x0));
    T.e01 = sub(x1, x0); T.d01 = dot(T.e01, T.e01);
    T.e12 = sub(x2, x1); T.d12 = dot(T.e12, T.e12);
    T.e02 = sub(x2, x0); T.d02 = dot(T.e02, T.e02);
    return T;
}

// Squared DistancePointToEdge(p, a, b) with x10 = b - a and dot(x10, x10) precomputed: the value
// whose sqrtf the reference takes.
__device__ __forceinline__ float edge_dist2_pre(float3 p, float3 a, float3 b, float3 x10, float dd) {
    float t = dot(sub(b, p), x10) / dd;
    t = fmaxf(0.0f, fminf(t, 1.0f));
    const float3 q = sub(p, add(mul(t, a), mul(1.0f - t, b)));
    return dot(q, q);
}

// SignedDistancePointToTriangle with one square root: the reference takes sqrtf of the face
// distance, or of each edge distance and then the minimum; sqrtf is correctly rounded and so
// monotone, hence min(sqrtf(u), sqrtf(v)) == sqrtf(min(u, v)) and the result is the same float.
__device__ __forceinline__ float signed_dist_pre(float3 p, const TriPre& T) {
    const float3 px2 = sub(p, T.x2);
    const float b = dot(T.x12n, px2) / T.l2;
    const float a = (dot(T.x02n, px2) - T.l1 * b) / T.l0;
    const float c = (1.0f - a) - b;
    const float tol = 1e-8f;
    float d2;
    if (a >= -tol && b >= -tol && c >= -tol) {
        const float3 nn = sub(p, add(add(mul(a, T.x0), mul(b, T.x1)), mul(c, T.x2)));
        d2 = dot(nn, nn);
    } else {
        const float u01 = edge_dist2_pre(p, T.x0, T.x1, T.e01, T.d01);
        const float u12 = edge_dist2_pre(p, T.x1, T.x2, T.e12, T.d12);
        const float u02 = edge_dist2_pre(p, T.x0, T.x2, T.e02, T.d02);
        d2 = fminf(fminf(u01, u12), u02);
    }
    float d = sqrtf(d2);
    d = (dot(sub(p, T.x0), T.nTri) < 0.0f) ? -d : d;
    return d;
}

// The cell box ConstructSignedDistanceField visits for a triangle (:351-363): AABB +- one cell,
// grid coordinates -+ GRID_MARGIN, clamped to the grid.
__device__ __forceinline__ void tri_cell_box(const SdfGrid& g, float3 t0, float3 t1, float3 t2, int3& lo, int3& hi) {
    const float3 m = mk3(g.cell, g.cell, g.cell);
    const float3 aabbMin = sub(vmin(t0, vmin(t1, t2)), m);
    const float3 aabbMax = add(vmax(t0, vmax(t1, t2)), m);
    lo = sdf_coords(g, aabbMin);
    hi = sdf_coords(g, aabbMax);
    lo.x = max(0, min(lo.x - 1, g.nx - 1)); lo.y = max(0, min(lo.y - 1, g.ny - 1)); lo.z = max(0, min(lo.z - 1, g.nz - 1));
    hi.x = max(0, min(hi.x + 1, g.nx - 1)); hi.y = max(0, min(hi.y + 1, g.ny - 1)); hi.z = max(0, min(hi.z + 1, g.nz - 1));
}

// What ConstructSignedDistanceField (:329-397) computes once per triangle: its invariants, the
// reference's cell box and the grid that box indexes.  In the warp constructs lane k of a warp makes
// the job of the k-th of 32 consecutive triangles, and the warp then runs the 32 cell loops one after
// another, reading each job from shared memory.  So the per-triangle work (the vertex loads, six
// divisions for the box, two square roots and six divisions for the invariants) is done once per
// triangle instead of once per lane; every value is the same expression on the same inputs, so the
// results do not change.  48 words, 16-byte aligned: a job moves as twelve 16-byte loads.
struct alignas(16) TriJob {
    TriPre P;                  // 33 words
    float ox, oy, oz, cell;    // the grid
    int gnx, gny;
    int lox, loy, loz;         // the box: first cell, row length, slice size, cells
    int nx, nxy, vol;
    float inxy;                // 1 / nxy
    uint32_t* words;
};
static_assert(sizeof(TriJob) == 192, "a triangle job is 48 words");

// Warps of a construct block keep up to 32 jobs each in shared memory.
constexpr int kTriJobsPerWarp = 32;

// Triangles per warp chunk for a launch over `tris` triangles: 32 where there are enough of them for
// four chunks per resident warp (about 24 warps per SM), fewer down to one per chunk for small meshes,
// so that a launch still spreads over every SM.
inline int sdf_construct_chunk(long long tris, int sms) {
    const long long per = tris / ((long long)sms * 96);
    return (int)(per < 1 ? 1 : per > kTriJobsPerWarp ? kTriJobsPerWarp : per);
}
// Chunks this small make their jobs in every lane instead (no shared memory, fewer registers): staging
// a job through shared memory costs more than the few lanes it would spare.
constexpr int kTriJobsStagedFrom = 4;

__device__ __forceinline__ TriJob tri_job(const SdfGrid& g, uint32_t* words, float3 x0, float3 x1, float3 x2) {
    TriJob J;
    int3 lo, hi;
    tri_cell_box(g, x0, x1, x2, lo, hi);
    J.P = tri_pre(x0, x1, x2);
    J.ox = g.ox; J.oy = g.oy; J.oz = g.oz; J.cell = g.cell;
    J.gnx = g.nx; J.gny = g.ny;
    J.lox = lo.x; J.loy = lo.y; J.loz = lo.z;
    J.nx = hi.x - lo.x + 1;
    J.nxy = J.nx * (hi.y - lo.y + 1);
    J.vol = J.nxy * (hi.z - lo.z + 1);
    J.inxy = 1.0f / (float)J.nxy;
    J.words = words;
    return J;
}

// The cell loop of one job by one warp: the lanes over the box, each with the reference's distance and
// the same atomicMin on the FloatFlip3 word.  Box coordinates of cell c: (c + 0.5) / m lies at least
// 0.5 / m from an integer, and the float product (c + 0.5) * (1 / m) is within (c / m) * 2^-23 of it,
// so its truncation is the integer quotient while c < 2^22; larger boxes use integer division.
__device__ __forceinline__ void sdf_construct_job_warp(const TriJob& J, int lane) {
    SdfGrid g;
    g.ox = J.ox; g.oy = J.oy; g.oz = J.oz; g.cell = J.cell;
    g.nx = J.gnx; g.ny = J.gny; g.nz = 0; g.reserved = 0;
    const int nx = J.nx, nxy = J.nxy, vol = J.vol;
    const bool floatIdx = vol < (1 << 22);
    const float inxy = J.inxy, inx = 1.0f / (float)nx;
    for (int c = lane; c < vol; c += 32) {
        int cz, r, cy;
        if (floatIdx) {
            cz = (int)(((float)c + 0.5f) * inxy);
            r = c - cz * nxy;
            cy = (int)(((float)r + 0.5f) * inx);
        } else {
            cz = c / nxy;
            r = c - cz * nxy;
            cy = r / nx;
        }
        const int x = J.lox + (r - cy * nx), y = J.loy + cy, z = J.loz + cz;
        const float d = signed_dist_pre(sdf_cell_pos(g, x, y, z), J.P);
        atomicMin(J.words + ((long long)z * g.ny + y) * g.nx + x, float_flip3(d));
    }
}

// One warp's chunk of `count` (<= 32) consecutive triangles starting at `first`.  STAGED: lane k makes
// the job of triangle first + k with make(t) into `jobs`, the warp's own 32-job area, then the warp runs
// the cell loops; the chunk ends with the warp synchronised, so the area can take the next chunk.
// Otherwise every lane makes each job itself and `jobs` is not used.
template <bool STAGED, class MakeJob>
__device__ __forceinline__ void sdf_construct_chunk_warp(TriJob* __restrict__ jobs, int first, int count, int lane,
                                                         MakeJob make) {
    if (!STAGED) {
        for (int j = 0; j < count; ++j) sdf_construct_job_warp(make(first + j), lane);
        return;
    }
    if (lane < count) jobs[lane] = make(first + lane);
    __syncwarp();
    for (int j = 0; j < count; ++j) {
        const TriJob J = jobs[j];
        sdf_construct_job_warp(J, lane);
    }
    __syncwarp();
}

// GetSignedDistance + TrilinearInterpolate, :414-527
__device__ __forceinline__ float lerp_ref(float a, float b, float t) { return a * (1.0f - t) + b * t; }

__device__ __forceinline__ float sdf_lookup(const float* __restrict__ sdf, const SdfGrid& g, float3 p) {
    if (sdf_surely_outside(g, p)) return 1e10f;
    const int3 gc = sdf_coords(g, p);
    if (!(0 <= gc.x && gc.x < g.nx - 2) || !(0 <= gc.y && gc.y < g.ny - 2) || !(0 <= gc.z && gc.z < g.nz - 2))
        return 1e10f;
    const long long X = 1, Y = g.nx, Z = (long long)g.ny * g.nx;
    const long long base = Z * gc.z + Y * gc.y + gc.x;
    float d[8];
    d[0] = __ldg(sdf + base);
    d[1] = __ldg(sdf + base + X);
    d[2] = __ldg(sdf + base + Y);
    d[3] = __ldg(sdf + base + Y + X);
    d[4] = __ldg(sdf + base + Z);
    d[5] = __ldg(sdf + base + Z + X);
    d[6] = __ldg(sdf + base + Z + Y);
    d[7] = __ldg(sdf + base + Z + Y + X);
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if (d[j] == 1e10f) return 1e10f;
    const float3 cp = sdf_cell_pos(g, gc.x, gc.y, gc.z);
    const float3 ip = divs(sub(p, cp), g.cell);
    const float b0 = lerp_ref(lerp_ref(d[0], d[1], ip.x), lerp_ref(d[2], d[3], ip.x), ip.y);
    const float b1 = lerp_ref(lerp_ref(d[4], d[5], ip.x), lerp_ref(d[6], d[7], ip.x), ip.y);
    return lerp_ref(b0, b1, ip.z);
}

// CollideHairVerticesWithSdf_forward for one vertex (j >= 2): returns true and the projected
// position when the vertex is pushed out (then Pos.xyz and Prev.xyz both take it).
// The part after the first lookup: `distance` = sdf_lookup(sdf, g, p).
__device__ __forceinline__ bool sdf_collide_from(const float* __restrict__ sdf, const SdfGrid& g, float margin, float3 p,
                                                 float distance, float3& proj) {
    if (distance > margin) return false;
    const float h = 0.1f * g.cell;
    const float fx = sdf_lookup(sdf, g, add(p, mul(mk3(1.0f, 0.0f, 0.0f), h)));
    const float fy = sdf_lookup(sdf, g, add(p, mul(mk3(0.0f, 1.0f, 0.0f), h)));
    const float fz = sdf_lookup(sdf, g, add(p, mul(mk3(0.0f, 0.0f, 1.0f), h)));
    const float3 grad = mk3((fx - distance) / h, (fy - distance) / h, (fz - distance) / h);
    const float3 nrm = normalize(grad);
    if (distance < margin) {
        proj = add(p, mul(nrm, margin - distance));
        return true;
    }
    return false;
}

__device__ __forceinline__ bool sdf_collide_point(const float* __restrict__ sdf, const SdfGrid& g, float margin, float3 p,
                                                  float3& proj) {
    const float distance = sdf_lookup(sdf, g, p);
    if (distance > margin) return false;
    const float h = 0.1f * g.cell;
    const float fx = sdf_lookup(sdf, g, add(p, mul(mk3(1.0f, 0.0f, 0.0f), h)));
    const float fy = sdf_lookup(sdf, g, add(p, mul(mk3(0.0f, 1.0f, 0.0f), h)));
    const float fz = sdf_lookup(sdf, g, add(p, mul(mk3(0.0f, 0.0f, 1.0f), h)));
    const float3 grad = mk3((fx - distance) / h, (fy - distance) / h, (fz - distance) / h);
    const float3 nrm = normalize(grad);
    if (distance < margin) {
        proj = add(p, mul(nrm, margin - distance));
        return true;
    }
    return false;
}

}  // namespace tfx
