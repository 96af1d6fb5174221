// Batched path kernels: many hair objects (uneven strand counts, vertices per strand, settings) and
// their SDFs advance one frame in a handful of launches.
//
//  * k_batch_mesh_skin    - BoneSkinning (TressFXBoneSkinning.hlsl:57-94) over every vertex of every
//                           collision mesh.
//  * k_batch_sdf_init / k_batch_sdf_construct / k_batch_sdf_finalize
//                         - InitializeSignedDistanceField / ConstructSignedDistanceField /
//                           FinalizeSignedDistanceField (TressFXSDFCollision.hlsl:301-412) of every
//                           SDF.  The construct runs one warp per triangle: the lanes share the
//                           triangle's cell box (the reference's AABB +- one cell, -+ one grid cell),
//                           the triangle-only terms of the distance are computed once, and each
//                           (triangle, cell) pair does the reference's distance and an atomicMin on the
//                           FloatFlip3 word.  The pairs and the encoding are the reference's, so the grid
//                           is bit-identical.
//  * k_fused_strands      - the six simulation stages of the guide strands (TressFXSimulation.hlsl:
//                           609-975) for a group of 32 guide strands in one pass.  Phase 0: bulk
//                           asynchronous copies (cp.async.bulk on an mbarrier) bring the group's Pos
//                           rows (and below n = 64 its InitialPos rows) into shared memory while warp 0
//                           blends each strand's bone matrix.  Phase 1a
//                           (one lane per strand): strand-level data.  Phase 1b (one thread per
//                           vertex): integration + global shape, VSP, bind pose.  Phase 2 (one lane
//                           per strand, one warp per iteration): the local-shape sweeps as a
//                           wavefront (iteration k runs two vertices behind iteration k-1, which is
//                           exactly the order in which the sequential sweeps read and write).
//                           Phase 3a (n/VPL lanes per strand): wind, length constraints (warp
//                           shuffles), tangents, velocity clamp.  Phase 3c: the guides' state is
//                           written once.  Blocks are persistent over the strand groups of every
//                           object of one vertices-per-strand class.  Needs no SDF, so it runs
//                           while the frame's SDFs are being built.
//  * k_follow_collide     - UpdateFollowHairVertices (TressFXSimulation.hlsl:978-1001) and the SDF
//                           collision (TressFXSDFCollision.hlsl:531-595) of every guide and follow
//                           vertex, after both.
//  * k_collide_level      - the same collision with an object's further SDFs, one level (every object's
//                           k-th further SDF) per launch, after k_follow_collide.
// All per-vertex arithmetic is the reference's, in the same order, so every buffer matches the
// plain path and the oracle bit for bit.
#include "tfx_batch.h"
#include "tfx_bulk.cuh"
#include "tfx_sdf_math.cuh"

namespace tfx {

// ============================================================================================
// collision-mesh skinning over all meshes
__global__ void __launch_bounds__(256) k_batch_mesh_skin(const BatchMesh* __restrict__ meshes, int nmeshes,
                                                         int totalVerts) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= totalVerts) return;
    int lo = 0, hi = nmeshes - 1;
    while (lo < hi) {  // last mesh with firstVertex <= t
        const int mid = (lo + hi + 1) >> 1;
        if (meshes[mid].firstVertex <= t) lo = mid; else hi = mid - 1;
    }
    const BatchMesh& m = meshes[lo];
    const int v = t - m.firstVertex;
    const float4 p = __ldg(m.bind + 2 * v), nr = __ldg(m.bind + 2 * v + 1);
    float mm[4][4];
    blend_bones(m.bones, __ldg(m.skin + 2 * v), __ldg(m.skin + 2 * v + 1), mm);
    m.skinned[2 * v] = with_xyz(p, xform_row(xyz(p), 1.0f, mm));
    m.skinned[2 * v + 1] = with_xyz(nr, xform_row(xyz(nr), 0.0f, mm));
}

// ============================================================================================
// SDF rebuild of every SDF
__device__ __forceinline__ int find_by_prefix_tri(const BatchSdf* __restrict__ sdfs, int nsdf, long long t) {
    int lo = 0, hi = nsdf - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sdfs[mid].firstTriangle <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int find_by_prefix_quad(const BatchSdf* __restrict__ sdfs, int nsdf, long long q) {
    int lo = 0, hi = nsdf - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sdfs[mid].firstQuad <= q) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// InitializeSignedDistanceField, :301-312: every cell of every SDF, 4 cells per thread (the last
// quad of an SDF may be partial).
__global__ void __launch_bounds__(256) k_batch_sdf_init(const BatchSdf* __restrict__ sdfs, int nsdf, long long totalQuads) {
    const uint32_t v = float_flip3(1e10f);
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < totalQuads; q += stride) {
        const BatchSdf& s = sdfs[find_by_prefix_quad(sdfs, nsdf, q)];
        const long long c = 4 * (q - s.firstQuad);
        const long long cells = s.numCells;
        uint32_t* g = s.words;
        if (c + 4 <= cells) {
            *reinterpret_cast<uint4*>(g + c) = make_uint4(v, v, v, v);
        } else {
            for (long long i = c; i < cells; ++i) g[i] = v;
        }
    }
}

// FinalizeSignedDistanceField, :400-412
__global__ void __launch_bounds__(256) k_batch_sdf_finalize(const BatchSdf* __restrict__ sdfs, int nsdf,
                                                            long long totalQuads) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < totalQuads; q += stride) {
        const BatchSdf& s = sdfs[find_by_prefix_quad(sdfs, nsdf, q)];
        const long long c = 4 * (q - s.firstQuad);
        const long long cells = s.numCells;
        uint32_t* g = s.words;
        if (c + 4 <= cells) {
            uint4 u = *reinterpret_cast<uint4*>(g + c);
            *reinterpret_cast<uint4*>(g + c) = make_uint4(ifloat_flip3(u.x), ifloat_flip3(u.y), ifloat_flip3(u.z),
                                                          ifloat_flip3(u.w));
        } else {
            for (long long i = c; i < cells; ++i) g[i] = ifloat_flip3(g[i]);
        }
    }
}

// Corner-expanded copy of a finalized grid: record c holds the eight corners a trilinear lookup in
// cell c reads, in TrilinearInterpolate's order ((x,y,z), (x+1,y,z), (x,y+1,z), (x+1,y+1,z), then the
// same at z+1), so a lookup reads one 32-byte record instead of eight scattered words.  Only the
// cells a lookup can use (x < nx-1, y < ny-1, z < nz-1) are written.  The threads run over the cells
// of the SDFs that keep a copy (expSdf, with expFirst the prefix of their cell counts) and no others.
__global__ void __launch_bounds__(256) k_batch_sdf_expand(const BatchSdf* __restrict__ sdfs,
                                                          const int* __restrict__ expSdf,
                                                          const long long* __restrict__ expFirst, int nexp,
                                                          long long expCells) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < expCells; t += stride) {
        int lo = 0, hi = nexp - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(expFirst + mid) <= t) lo = mid; else hi = mid - 1;
        }
        const BatchSdf& s = sdfs[__ldg(expSdf + lo)];
        const long long c = t - __ldg(expFirst + lo);
        const SdfGrid g = s.frame->grid;
        const long long nxy = (long long)g.nx * g.ny;
        const int z = (int)(c / nxy);
        const long long r = c - (long long)z * nxy;
        const int y = (int)(r / g.nx), x = (int)(r - (long long)y * g.nx);
        if (x >= g.nx - 1 || y >= g.ny - 1 || z >= g.nz - 1) continue;
        const float* f = reinterpret_cast<const float*>(s.words);
        const long long Y = g.nx, Z = nxy;
        float4* o = s.expanded + 2 * c;
        o[0] = make_float4(f[c], f[c + 1], f[c + Y], f[c + Y + 1]);
        o[1] = make_float4(f[c + Z], f[c + Z + 1], f[c + Z + Y], f[c + Z + Y + 1]);
    }
}

// ConstructSignedDistanceField, :329-397.  Each warp takes chunks of `per` (<= 32) consecutive
// triangles of the batch's triangle list (which may span SDFs): lane k finds the SDF of the chunk's
// k-th triangle and makes its job, then the warp runs the triangles' cell loops in turn.
// WARPS = warps per block; STAGED as in sdf_construct_chunk_warp.
template <int WARPS, bool STAGED>
__global__ void __launch_bounds__(WARPS * 32) k_batch_sdf_construct(const BatchSdf* __restrict__ sdfs, int nsdf,
                                                                     int totalTris, int per) {
    __shared__ TriJob jobs[STAGED ? WARPS : 1][STAGED ? kTriJobsPerWarp : 1];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int chunks = (totalTris + per - 1) / per;
    for (int k = blockIdx.x * WARPS + warp; k < chunks; k += gridDim.x * WARPS) {
        const int first = k * per;
        sdf_construct_chunk_warp<STAGED>(jobs[STAGED ? warp : 0], first, min(per, totalTris - first), lane, [&](int t) {
            const BatchSdf& s = sdfs[find_by_prefix_tri(sdfs, nsdf, t)];
            const int tri = t - s.firstTriangle;
            const float3 x0 = xyz(__ldg(s.mesh + 2 * (size_t)__ldg(s.indices + 3 * tri + 0)));
            const float3 x1 = xyz(__ldg(s.mesh + 2 * (size_t)__ldg(s.indices + 3 * tri + 1)));
            const float3 x2 = xyz(__ldg(s.mesh + 2 * (size_t)__ldg(s.indices + 3 * tri + 2)));
            return tri_job(s.frame->grid, s.words, x0, x1, x2);
        });
    }
}

// ============================================================================================
// fused strand kernel
//
// One block runs one group of GS = fused_group_strands(N) guide strands of one object at a time.
// Shared memory, strand-major rows of N vertices padded to N+1 float4, so that both the one-lane-per-
// strand sweep and the one-lane-per-vertex passes are free of bank conflicts:
//   TP[GS][N+1] positions   TI[GS][N+1] InitialPos, then the bind pose (below N = 64 only)
//   SK[GS][4] blended bone matrix rows   SL[GS][3] StrandLevelData
//   one mbarrier, on which the bulk copies that bring a group's rows in complete.
// Prev, Tangent and RestLength never enter shared memory: each thread reads (and writes) its own
// vertices' words in global memory (coalesced), which keeps a block small enough for six to fit per
// SM at n = 32 and 64, and the serial local-shape sweeps of that many groups to run side by side.
// Below 64 vertices a strand's local-shape sweeps (as many as the settings ask, TressFXHairObject.cpp:
// 402-411) read the bind pose from a second tile; at 64 a strand has one sweep a frame, which computes
// the bind pose from InitialPos in global memory instead, so a group holds 32 strands in about the
// shared memory 16 took with the tile, and twice as many strands sweep at once per SM.
__host__ __device__ constexpr bool fused_init_tile(int n) { return n < 64; }
__host__ __device__ constexpr int fused_group_strands(int) { return 32; }
__host__ __device__ constexpr int fused_smem_for(int n) {
    return (fused_init_tile(n) ? 2 : 1) * fused_group_strands(n) * (n + 1) * 16 + fused_group_strands(n) * 7 * 16 + 16;
}
// k_fused_strands modes: the whole frame of the group, or its part before the local-shape sweeps
// (integration, strand-level data, VSP; the state goes to global memory for k_local_sweep), or its
// part after them (wind, length constraints, tangents, velocity clamp)
constexpr int kFusedFull = 0, kFusedPre = 1, kFusedPost = 2;

// IntegrationAndGlobalShapeConstraints (TressFXSimulation.hlsl:609-666) for vertex j: returns the new
// position (after the global shape constraint) and, in `cur`, the position that becomes Prev.
__device__ __forceinline__ float4 integrate_vertex(const DevSimConsts* __restrict__ c, const float (&m)[4][4], float4 ip,
                                                   float4& cur, float4 old, int j, int n) {
    float4 initialPos = ip;
    const float3 sk = xform_row(xyz(initialPos), 1.0f, m);
    initialPos.x = sk.x; initialPos.y = sk.y; initialPos.z = sk.z;
    float4 currentPos = cur;
    float4 shared = currentPos;
    float4 oldPos = old;
    if (c->reset != 0.0f) { currentPos = initialPos; oldPos = initialPos; }
    if (currentPos.w > 0.0f) {
        const float dt = c->timeStep;
        const float gx = c->gravity * 0.0f, gy = c->gravity * -1.0f;
        const float3 cu = xyz(currentPos), ol = xyz(oldPos);
        const float3 force = mk3(gx, gy, gx);
        const float3 r = add(add(cu, mul(c->decay, sub(cu, ol))), mul(mul(force, dt), dt));
        shared.x = r.x; shared.y = r.y; shared.z = r.z;
    } else {
        shared = initialPos;
    }
    const float kG = c->globalStiffness, range = c->globalRange;
    if (kG > 0.0f && range != 0.0f) {
        if (shared.w > 0.0f) {
            if ((float)j < range * (float)n) {
                const float3 del = mul(kG, sub(xyz(initialPos), xyz(shared)));
                shared.x = shared.x + del.x; shared.y = shared.y + del.y; shared.z = shared.z + del.z;
            }
        }
    }
    cur = currentPos;
    return shared;
}

// One step of LocalShapeConstraints (TressFXSimulation.hlsl:794-825) for vertex j: pm1/pos are the
// strand's vertices j-1 and j as this sweep has left them, pp1 vertex j+1 as the previous sweep left
// it, bm1/b0/bp1 the bind-pose positions.  Updates pos (final for j) and pp1.
__device__ __forceinline__ void local_shape_step(float4 pm1, float4& pos, float4& pp1, float3 bm1, float3 b0, float3 bp1,
                                                 float stiff) {
    const float3 lastVec = sub(xyz(pos), xyz(pm1));
    const float3 vecBindPose = sub(bp1, b0);
    const float3 lastVecBindPose = sub(b0, bm1);
    const Q4 rg = qfrom2(normalize(lastVecBindPose), normalize(lastVec));
    const float3 org = add(qrot(rg, vecBindPose), xyz(pos));
    const float3 del = mul(stiff, sub(org, xyz(pp1)));
    if (pos.w > 0.0f) { pos.x = pos.x - del.x; pos.y = pos.y - del.y; pos.z = pos.z - del.z; }
    if (pp1.w > 0.0f) { pp1.x = pp1.x + del.x; pp1.y = pp1.y + del.y; pp1.z = pp1.z + del.z; }
}

// Barrier among the first `threads` threads of the block (named barrier 1; all of them must call it).
__device__ __forceinline__ void bar_sync_first(int threads) {
    asm volatile("bar.sync 1, %0;" ::"r"(threads) : "memory");
}

// KW consecutive local-shape sweeps of the group's strands, as a wavefront over warps: warp k
// (k < KW) runs sweep k, lane s is strand s, and at time step t warp k works on vertex
// j = t - 2k + 1.  Sweep k needs vertex j+1 as sweep k-1 left it, which warp k-1 stored at step t-1;
// within one step no two warps touch the same element, and a barrier of the KW warps separates the
// steps, so every read sees exactly the value the sequential sweeps give it.  Element (s, j) of a
// tile is at s*RS + j.
template <int N>
__device__ __forceinline__ void sweep_wavefront(float4* __restrict__ SP, const float4* __restrict__ SB, int s, bool active,
                                                int k, int KW, float stiff) {
    constexpr int RS = N + 1;
    float4* P = SP + s * RS;
    const float4* B = SB + s * RS;
    if (KW == 1) {
        // A single sweep: no other warp reads this warp's stores, so the steps need no barrier, and
        // row element j + 2 (read once, at step j + 1, and written only after that) loads a step early.
        if (!active) return;
        float4 pm1 = P[0], pos = P[1], next = P[2];
        float3 bm1 = xyz(B[0]), b0 = xyz(B[1]), bnext = xyz(B[2]);
        for (int j = 1; j <= N - 2; ++j) {
            float4 pp1 = next;
            const float3 bp1 = bnext;
            if (j + 2 <= N - 1) { next = P[j + 2]; bnext = xyz(B[j + 2]); }
            local_shape_step(pm1, pos, pp1, bm1, b0, bp1, stiff);
            P[j] = pos;
            pm1 = pos; pos = pp1; bm1 = b0; b0 = bp1;
        }
        P[N - 1] = pos;
        return;
    }
    float4 pm1 = make_float4(0.f, 0.f, 0.f, 0.f), pos = pm1;
    float3 bm1 = mk3(0.f, 0.f, 0.f), b0 = bm1;
    const int T = (N - 2) + 2 * (KW - 1);
    for (int t = 0; t < T; ++t) {
        const int j = t - 2 * k + 1;
        if (active && j >= 1 && j <= N - 2) {
            if (j == 1) {
                pm1 = P[0]; pos = P[1];
                bm1 = xyz(B[0]); b0 = xyz(B[1]);
            }
            float4 pp1 = P[j + 1];
            const float3 bp1 = xyz(B[j + 1]);
            local_shape_step(pm1, pos, pp1, bm1, b0, bp1, stiff);
            P[j] = pos;
            if (j == N - 2) P[N - 1] = pp1;
            pm1 = pos; pos = pp1; bm1 = b0; b0 = bp1;
        }
        bar_sync_first(KW * 32);
    }
}

// The one sweep of a strand at N = 64 (the shader's single sweep; more when the caller asks for more
// dispatches, one after the other): as the single-sweep case of sweep_wavefront, with the bind pose of
// vertex j computed here as qrot(skinning quaternion, InitialPos_j), exactly as phase 1b computes it
// for the tile, and InitialPos loaded two steps ahead.
template <int N>
__device__ __forceinline__ void sweep_single_global(float4* __restrict__ P, const float4* __restrict__ init, Q4 bq,
                                                    float stiff) {
    auto bind = [&](float4 ip) { return qrot(bq, xyz(ip)); };
    float4 pm1 = P[0], pos = P[1], next = P[2];
    float3 bm1 = bind(__ldg(init + 0)), b0 = bind(__ldg(init + 1)), bnext = bind(__ldg(init + 2));
    float4 ahead = __ldg(init + 3);
    for (int j = 1; j <= N - 2; ++j) {
        float4 pp1 = next;
        const float3 bp1 = bnext;
        if (j + 2 <= N - 1) {
            next = P[j + 2];
            bnext = bind(ahead);
            if (j + 3 <= N - 1) ahead = __ldg(init + j + 3);
        }
        local_shape_step(pm1, pos, pp1, bm1, b0, bp1, stiff);
        P[j] = pos;
        pm1 = pos; pos = pp1; bm1 = b0; b0 = bp1;
    }
    P[N - 1] = pos;
}

// Register bounds: at n <= 16 the tiles are small (21 KB a block) and registers decide residency, so
// 64 a thread (eight 4-warp blocks per SM; a few words spill) beat 80 (six blocks).
template <int N, int VPL>
__global__ void __launch_bounds__(256, N <= 16 ? 4 : (VPL <= 2 ? 3 : 2)) k_fused_strands(const BatchObject* __restrict__ objs,
                                                                        const WorkItem* __restrict__ items, int numItems,
                                                                        int* err, int mode, int waitPolls) {
    constexpr int GS = fused_group_strands(N);
    constexpr int RS = N + 1;       // tile row stride, float4
    constexpr int L = N / VPL;      // lanes per strand in the per-strand passes
    constexpr int SPW = 32 / L;     // strands per warp pass
    constexpr bool KI = fused_init_tile(N);   // InitialPos / bind-pose tile
    extern __shared__ float4 smem_f4[];
    float4* TP = smem_f4;
    float4* TI = TP + GS * RS;      // used only when KI
    float4* SK = TP + (KI ? 2 : 1) * GS * RS;
    float4* SL = SK + GS * 4;
    const uint32_t bar = smem_u32(SL + GS * 3);

    const int tid = threadIdx.x, nthreads = blockDim.x;
    const int warp = tid >> 5, nwarps = nthreads >> 5;
    const int lane = tid & 31;
    const int q = lane % L;         // lane within the strand
    const int slot = lane / L;      // strand slot within the warp pass

    if (tid == 0) mbar_init(bar, 1);
    __syncthreads();

    uint32_t parity = 0;
    for (int it = blockIdx.x; it < numItems; it += gridDim.x, parity ^= 1u) {
        const WorkItem wi = items[it];
        const BatchObject& ob = objs[wi.obj];
        const HairView h = ob.hair;
        const DevSimConsts* __restrict__ c = ob.consts;
        const int F = h.F;
        const int count = wi.count;
        const int gs0 = wi.firstGuide * (F + 1);   // strand index of the group's first guide

        // ------------------------------------------------------------ phase 0: bring the group in
        float4 bq4 = make_float4(0.f, 0.f, 0.f, 0.f);
        const bool pre = mode != kFusedPost, post = mode != kFusedPre;   // phases 0-2 / phase 3 run
        if (warp == 0) {
            // rows: Pos always; InitialPos for phases 0-2 when it has a tile
            const uint32_t rowBytes = N * 16 + (pre && KI ? N * 16 : 0);
            if (lane == 0) mbar_arrive_expect_tx(bar, (uint32_t)count * rowBytes);
            __syncwarp();
            if (lane < count) {
                const size_t vo = (size_t)(gs0 + lane * (F + 1)) * N;
                bulk_g2s(smem_u32(TP + lane * RS), h.pos + vo, N * 16, bar);
                if (pre && KI) bulk_g2s(smem_u32(TI + lane * RS), h.init + vo, N * 16, bar);
            }
            if (pre && lane < count) {
                // strand level, while the rows are in flight: the blended bone matrix and its quaternion
                const int gs = gs0 + lane * (F + 1);
                float m[4][4];
                blend_bones(c->bones, __ldg(h.skin + 2 * gs), __ldg(h.skin + 2 * gs + 1), m);
#pragma unroll
                for (int r = 0; r < 4; ++r) SK[lane * 4 + r] = make_float4(m[r][0], m[r][1], m[r][2], m[r][3]);
                const Q4 bq = quat_from_matrix(m);
                bq4 = make_float4(bq.x, bq.y, bq.z, bq.w);
            }
        }
        // waitPolls is kFusedWaitPollsDefault except in tests of this path (0: give up at once).  On
        // giving up, the block waits again with the full limit for its copies in flight to land before
        // it returns; if that wait gives up too, the block returns regardless (the frame is reported
        // as failed, and a bounded wait is preferred over one that could hang the device).
        const bool arrived = mbar_wait_bounded(bar, parity, waitPolls);
        if (__syncthreads_or(!arrived)) {
            if (tid == 0) atomicOr(err, 1);
            mbar_wait_bounded(bar, parity, kFusedWaitPollsDefault);
            return;
        }

        // ------------------------------------------------------------ phase 1a: CalculateStrandLevelData
        if (pre && warp == 0 && lane < count) {
            const int s = lane, gs = gs0 + s * (F + 1);
            float m[4][4];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const float4 row = SK[s * 4 + r];
                m[r][0] = row.x; m[r][1] = row.y; m[r][2] = row.z; m[r][3] = row.w;
            }
            float4 o0 = TP[s * RS], o1 = TP[s * RS + 1];
            const size_t vo = (size_t)gs * N;
            const float4 oo1 = h.prev[vo + 1];
            const float4 i0 = KI ? TI[s * RS] : __ldg(h.init + vo), i1 = KI ? TI[s * RS + 1] : __ldg(h.init + vo + 1);
            const float4 n0 = integrate_vertex(c, m, i0, o0, h.prev[vo], 0, N);
            const float4 n1 = integrate_vertex(c, m, i1, o1, oo1, 1, N);
            const float3 u = normalize(sub(xyz(o1), xyz(o0)));
            const float3 v = normalize(sub(xyz(n1), xyz(n0)));
            const Q4 rot = qfrom2(u, v);
            const float3 trans = sub(xyz(n0), qrot(rot, xyz(o0)));
            float vspCoeff = c->vspCoeff;
            {
                const float ax = (n1.x - 2.0f * o1.x) + oo1.x;
                const float ay = (n1.y - 2.0f * o1.y) + oo1.y;
                const float az = (n1.z - 2.0f * o1.z) + oo1.z;
                const float aw = (n1.w - 2.0f * o1.w) + oo1.w;
                const float accel = sqrtf(ax * ax + ay * ay + az * az + aw * aw);
                if (accel > c->vspAccelThreshold) vspCoeff = 1.0f;
            }
            const float4 r4 = make_float4(rot.x, rot.y, rot.z, rot.w);
            const float4 t4 = make_float4(trans.x, trans.y, trans.z, vspCoeff);
            SL[s * 3 + 0] = bq4; SL[s * 3 + 1] = r4; SL[s * 3 + 2] = t4;
            h.sld[3 * gs + 0] = bq4; h.sld[3 * gs + 1] = r4; h.sld[3 * gs + 2] = t4;
        }
        __syncthreads();

        // ------------------------------------------------------------ phase 1b: integration, VSP, bind pose
        for (int e = tid; pre && e < count * N; e += nthreads) {
            const int s = e / N, j = e % N;
            const int x = s * RS + j;
            float m[4][4];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const float4 row = SK[s * 4 + r];
                m[r][0] = row.x; m[r][1] = row.y; m[r][2] = row.z; m[r][3] = row.w;
            }
            const size_t v = (size_t)(gs0 + s * (F + 1)) * N + j;
            const float4 ip = KI ? TI[x] : __ldg(h.init + v), old = h.prev[v];
            float4 pv = TP[x];
            float4 p = integrate_vertex(c, m, ip, pv, old, j, N);
            h.prevprev[v] = old;
            if (j >= 2) {
                const float4 r4 = SL[s * 3 + 1], t4 = SL[s * 3 + 2];
                const Q4 rot{r4.x, r4.y, r4.z, r4.w};
                const float3 trans = xyz(t4);
                const float vspCoeff = t4.w;
                const float3 a = add(mul(1.0f - vspCoeff, xyz(p)), mul(vspCoeff, add(qrot(rot, xyz(p)), trans)));
                const float3 b = add(mul(1.0f - vspCoeff, xyz(pv)), mul(vspCoeff, add(qrot(rot, xyz(pv)), trans)));
                p = with_xyz(p, a);
                pv = with_xyz(pv, b);
            }
            TP[x] = p;
            h.prev[v] = pv;   // read back by phase 3 (after a block barrier)
            if (KI && mode == kFusedFull) {   // the bind pose, for the sweeps below
                const float4 b4 = SL[s * 3 + 0];
                const float3 bp = qrot(Q4{b4.x, b4.y, b4.z, b4.w}, xyz(ip));
                TI[x] = make_float4(bp.x, bp.y, bp.z, 0.0f);
            }
        }
        __syncthreads();
        if (mode == kFusedPre) {
            // the constrained-to-be state goes out; k_local_sweep and the kFusedPost pass take over
            for (int e = tid; e < count * N; e += nthreads) {
                const int s = e / N, j = e % N;
                const int x = s * RS + j;
                const size_t v = (size_t)(gs0 + s * (F + 1)) * N + j;
                h.pos[v] = TP[x];
            }
        }

        // ------------------------------------------------------------ phase 2: LocalShapeConstraints
        const int lsIters = mode == kFusedFull ? c->reserved0 : 0;
        if (lsIters > 0) {
            const float stiff = 0.5f * fminf(c->localStiffness, 0.95f);
            if constexpr (KI) {
                for (int done = 0; done < lsIters;) {   // waves of up to one sweep per warp
                    const int KW = min(lsIters - done, nwarps);
                    if (warp < KW) sweep_wavefront<N>(TP, TI, lane, lane < count, warp, KW, stiff);
                    __syncthreads();
                    done += KW;
                }
            } else {
                if (warp == 0 && lane < count) {
                    const float4 b4 = SL[lane * 3 + 0];
                    const float4* init = h.init + (size_t)(gs0 + lane * (F + 1)) * N;
                    for (int k = 0; k < lsIters; ++k) sweep_single_global<N>(TP + lane * RS, init, Q4{b4.x, b4.y, b4.z, b4.w}, stiff);
                }
                __syncthreads();
            }
        }

        // ------------------------------------------------------------ phase 3a: wind, length, tangents, clamp
        const float dt = c->timeStep;
        for (int pass = warp; post && pass * SPW < count; pass += nwarps) {
            const int s = pass * SPW + slot;
            const bool active = s < count;
            const int gs = gs0 + s * (F + 1);
            const int base = s * RS + q * VPL;
            const size_t vrow = (size_t)gs * N;   // the strand's first vertex
            float4 p[VPL], pv[VPL], tn[VPL];
            float len[VPL];
#pragma unroll
            for (int k = 0; k < VPL; ++k) {
                if (active) {
                    p[k] = TP[base + k];
                    pv[k] = h.prev[vrow + q * VPL + k];
                    tn[k] = h.tan[vrow + q * VPL + k];
                    len[k] = __ldg(h.rest + vrow + q * VPL + k);
                } else {
                    p[k] = pv[k] = tn[k] = make_float4(0.f, 0.f, 0.f, 0.f);
                    len[k] = 0.0f;
                }
            }
            // wind: every displacement from the pre-wind positions
            if (c->anyWind) {
                const float a = (float)(gs % 20) / 20.0f;
                const float3 w = add(add(add(mul(a, xyz(c->wind[0])), mul(1.0f - a, xyz(c->wind[1]))),
                                         mul(a, xyz(c->wind[2]))),
                                     mul(1.0f - a, xyz(c->wind[3])));
                float4 nxt[VPL];
#pragma unroll
                for (int k = 0; k + 1 < VPL; ++k) nxt[k] = p[k + 1];
                nxt[VPL - 1] = shfl4_down(p[0], 1);
                float3 disp[VPL];
#pragma unroll
                for (int k = 0; k < VPL; ++k) {
                    const int j = q * VPL + k;
                    disp[k] = mk3(0.f, 0.f, 0.f);
                    if (j >= 2 && j < N - 1) {
                        const float3 vv = sub(xyz(p[k]), xyz(nxt[k]));
                        const float3 force = neg(cross(cross(vv, w), vv));
                        disp[k] = mul(mul(force, dt), dt);
                    }
                }
#pragma unroll
                for (int k = 0; k < VPL; ++k) {
                    const int j = q * VPL + k;
                    if (j >= 2 && j < N - 1) {
                        p[k].x = p[k].x + disp[k].x; p[k].y = p[k].y + disp[k].y; p[k].z = p[k].z + disp[k].z;
                    }
                }
            }
            // length constraints
            const int lenIters = c->lengthIterations;
            for (int iter = 0; iter < lenIters; ++iter) {
                if constexpr (VPL == 1) {
                    {
                        const float4 o = shfl4(p[0], lane ^ 1);
                        const float ol = __shfl_sync(FULL, len[0], lane ^ 1);
                        const bool even = (q & 1) == 0;
                        const DC r = even ? distance_constraint(p[0], o, len[0]) : distance_constraint(o, p[0], ol);
                        p[0] = even ? r.p0 : r.p1;
                    }
                    {
                        const bool odd = (q & 1) != 0;
                        const int src = odd ? ((lane + 1) & 31) : ((lane + 31) & 31);
                        const float4 o = shfl4(p[0], src);
                        const float ol = __shfl_sync(FULL, len[0], src);
                        if (odd && q <= N - 3) p[0] = distance_constraint(p[0], o, len[0]).p0;
                        else if (!odd && q >= 2) p[0] = distance_constraint(o, p[0], ol).p1;
                    }
                } else {
#pragma unroll
                    for (int k = 0; k < VPL; k += 2) {
                        const DC r = distance_constraint(p[k], p[k + 1], len[k]);
                        p[k] = r.p0; p[k + 1] = r.p1;
                    }
#pragma unroll
                    for (int k = 1; k + 1 < VPL; k += 2) {
                        const DC r = distance_constraint(p[k], p[k + 1], len[k]);
                        p[k] = r.p0; p[k + 1] = r.p1;
                    }
                    const float4 nextFirst = shfl4_down(p[0], 1);
                    const float4 prevLast = shfl4_up(p[VPL - 1], 1);
                    const float prevLen = __shfl_up_sync(FULL, len[VPL - 1], 1);
                    const float4 myLast = p[VPL - 1];
                    const float4 myFirst = p[0];
                    if (q < L - 1) p[VPL - 1] = distance_constraint(myLast, nextFirst, len[VPL - 1]).p0;
                    if (q >= 1) p[0] = distance_constraint(prevLast, myFirst, prevLen).p1;
                }
            }
            // tangents
            {
                const float4 nx = shfl4_down(p[0], 1);
                const float4 pvl = shfl4_up(p[VPL - 1], 1);
#pragma unroll
                for (int k = 0; k < VPL; ++k) {
                    const int j = q * VPL + k;
                    float3 t;
                    if (j == N - 1) {
                        const float4 before = (k > 0) ? p[k > 0 ? k - 1 : 0] : pvl;
                        t = sub(xyz(p[k]), xyz(before));
                    } else {
                        const float4 after = (k + 1 < VPL) ? p[k + 1 < VPL ? k + 1 : k] : nx;
                        t = sub(xyz(after), xyz(p[k]));
                    }
                    tn[k] = with_xyz(tn[k], normalize(t));
                }
            }
            // velocity clamp
            const float clamp2 = c->clamp * c->clamp;
#pragma unroll
            for (int k = 0; k < VPL; ++k) {
                float3 d = sub(xyz(p[k]), xyz(pv[k]));
                const float speedSqr = dot(d, d);
                if (speedSqr > clamp2) {
                    d = mul(d, clamp2 / speedSqr);
                    pv[k] = with_xyz(pv[k], sub(xyz(p[k]), d));
                }
            }
            if (active) {   // the guide state goes out: Pos, Prev, Tangent
#pragma unroll
                for (int k = 0; k < VPL; ++k) {
                    h.pos[vrow + q * VPL + k] = p[k];
                    h.prev[vrow + q * VPL + k] = pv[k];
                    h.tan[vrow + q * VPL + k] = tn[k];
                }
            }
        }
        __syncthreads();

        fence_proxy_async_smem();   // this group's shared-memory accesses come before the next group's copies
        __syncthreads();
    }
}

// ============================================================================================
// LocalShapeConstraints (TressFXSimulation.hlsl:773-829) as the whole CPU re-dispatch loop
// (TressFXSimulation.cpp:64-72), between the kFusedPre and kFusedPost passes: one thread per guide
// strand, on the positions in global memory (each strand's rows stay in L1 across the sweep).  Up
// to four consecutive sweeps run together as a wavefront inside the thread: sweep k works on vertex
// j = t - 2k + 1 at step t, so it reads vertex j+1 as sweep k-1 left it one step earlier and vertex 1
// as it left it two steps earlier -- registers handed from sweep to sweep, exactly the values the
// sequential sweeps give -- and the four steps of one t are independent, so their latencies overlap.
// More sweeps run in waves of four.  Many strands per SM (no shared-memory tiles) hide the rest.
// The bind pose of vertex j is qrot(skinning quaternion, InitialPos_j), as phase 1b computes it.
template <int N>
__device__ __forceinline__ float3 bind_pose(const HairView& h, size_t vg, Q4 bq, int j) {
    return qrot(bq, xyz(__ldg(h.init + vg + j)));
}

template <int N>
__global__ void __launch_bounds__(128) k_local_sweep(const BatchObject* __restrict__ objs,
                                                     const WorkItem* __restrict__ items, int numItems) {
    constexpr int GS = fused_group_strands(N);
    constexpr int IPW = 32 / GS;     // work items per warp
    constexpr int KMAX = 4;
    const int lane = threadIdx.x & 31;
    const int it = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5) * IPW + lane / GS;
    if (it >= numItems) return;
    const WorkItem wi = items[it];
    const int s = lane % GS;
    if (s >= wi.count) return;
    const BatchObject& ob = objs[wi.obj];
    const HairView h = ob.hair;
    const DevSimConsts* __restrict__ c = ob.consts;
    const int iters = c->reserved0;
    if (iters <= 0) return;
    const int gs = (wi.firstGuide + s) * (h.F + 1);
    const size_t vg = (size_t)gs * N;
    float4* __restrict__ P = h.pos + vg;
    const float4 bq4 = h.sld[3 * gs];
    const Q4 bq{bq4.x, bq4.y, bq4.z, bq4.w};
    const float stiff = 0.5f * fminf(c->localStiffness, 0.95f);
    const float4 p0 = P[0];          // vertex 0 is never moved by a sweep
    const float3 b0v = bind_pose<N>(h, vg, bq, 0), b1v = bind_pose<N>(h, vg, bq, 1);
    for (int done = 0; done < iters; done += KMAX) {
        const int K = min(iters - done, KMAX);
        float4 pm1[KMAX], cur[KMAX], o1[KMAX], o2[KMAX];
        float3 bm1[KMAX], b0[KMAX];
#pragma unroll
        for (int k = 0; k < KMAX; ++k) {
            pm1[k] = cur[k] = o1[k] = o2[k] = make_float4(0.f, 0.f, 0.f, 0.f);
            bm1[k] = b0[k] = mk3(0.f, 0.f, 0.f);
        }
        const int T = (N - 2) + 2 * (K - 1);
        // sweep 0 reads vertex t+2 (position and InitialPos) at step t: those loads are issued two steps
        // ahead (a miss costs an L2 round trip, which two steps cover); the later sweeps read
        // InitialPos rows that sweep 0 brought into L1.  Indices past the strand's end are clamped.
        float4 qP0 = P[min(2, N - 1)], qP1 = P[min(3, N - 1)];
        float4 qI0 = __ldg(h.init + vg + min(2, N - 1)), qI1 = __ldg(h.init + vg + min(3, N - 1));
        for (int t = 0; t < T; ++t) {
            const float4 pAhead = qP0, iAhead = qI0;   // vertex t+2
            qP0 = qP1;
            qI0 = qI1;
            qP1 = P[min(t + 4, N - 1)];
            qI1 = __ldg(h.init + vg + min(t + 4, N - 1));
            float4 out[KMAX];
#pragma unroll
            for (int k = 0; k < KMAX; ++k) {
                out[k] = o1[k];
                if (k >= K) continue;
                const int j = t - 2 * k + 1;
                if (j >= 1 && j <= N - 2) {
                    if (j == 1) {
                        pm1[k] = p0;
                        cur[k] = k == 0 ? P[1] : o2[k - 1];   // vertex 1 as sweep k-1 left it
                        bm1[k] = b0v;
                        b0[k] = b1v;
                    }
                    float4 pp1 = k == 0 ? pAhead : o1[k - 1];   // vertex j+1 as sweep k-1 left it
                    const float3 bp1 = k == 0 ? qrot(bq, xyz(iAhead)) : bind_pose<N>(h, vg, bq, j + 1);
                    local_shape_step(pm1[k], cur[k], pp1, bm1[k], b0[k], bp1, stiff);
                    out[k] = cur[k];
                    if (k == K - 1) {
                        P[j] = cur[k];
                        if (j == N - 2) P[N - 1] = pp1;
                    }
                    pm1[k] = cur[k];
                    cur[k] = pp1;
                    bm1[k] = b0[k];
                    b0[k] = bp1;
                } else if (j == N - 1) {
                    out[k] = cur[k];   // vertex N-1 after the sweep's last step
                }
            }
#pragma unroll
            for (int k = 0; k < KMAX; ++k) {
                o2[k] = o1[k];
                o1[k] = out[k];
            }
        }
    }
}

// GetSignedDistance + TrilinearInterpolate (TressFXSDFCollision.hlsl:414-527) on the corner-expanded
// grid: the same cell, bounds test, corner values and interpolation as sdf_lookup.
__device__ __forceinline__ float sdf_lookup8(const float4* __restrict__ sdf8, const SdfGrid& g, float3 p) {
    if (sdf_surely_outside(g, p)) return 1e10f;
    const int3 gc = sdf_coords(g, p);
    if (!(0 <= gc.x && gc.x < g.nx - 2) || !(0 <= gc.y && gc.y < g.ny - 2) || !(0 <= gc.z && gc.z < g.nz - 2))
        return 1e10f;
    const long long base = ((long long)g.ny * g.nx) * gc.z + (long long)g.nx * gc.y + gc.x;
    const float4 lo = __ldg(sdf8 + 2 * base), hi = __ldg(sdf8 + 2 * base + 1);
    const float d[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if (d[j] == 1e10f) return 1e10f;
    const float3 cp = sdf_cell_pos(g, gc.x, gc.y, gc.z);
    const float3 ip = divs(sub(p, cp), g.cell);
    const float b0 = lerp_ref(lerp_ref(d[0], d[1], ip.x), lerp_ref(d[2], d[3], ip.x), ip.y);
    const float b1 = lerp_ref(lerp_ref(d[4], d[5], ip.x), lerp_ref(d[6], d[7], ip.x), ip.y);
    return lerp_ref(b0, b1, ip.z);
}

// sdf_collide_from with every lookup on the expanded grid.
__device__ __forceinline__ bool sdf_collide_from8(const float4* __restrict__ sdf8, const SdfGrid& g, float margin,
                                                  float3 p, float distance, float3& proj) {
    if (distance > margin) return false;
    const float h = 0.1f * g.cell;
    const float fx = sdf_lookup8(sdf8, g, add(p, mul(mk3(1.0f, 0.0f, 0.0f), h)));
    const float fy = sdf_lookup8(sdf8, g, add(p, mul(mk3(0.0f, 1.0f, 0.0f), h)));
    const float fz = sdf_lookup8(sdf8, g, add(p, mul(mk3(0.0f, 0.0f, 1.0f), h)));
    const float3 grad = mk3((fx - distance) / h, (fy - distance) / h, (fz - distance) / h);
    const float3 nrm = normalize(grad);
    if (distance < margin) {
        proj = add(p, mul(nrm, margin - distance));
        return true;
    }
    return false;
}

// The part of the collision after the first lookup (the vertices within the margin).
__device__ __forceinline__ bool collide_near(const float* __restrict__ sdf, const float4* __restrict__ sdf8,
                                             const SdfGrid& g, float margin, float3 p, float distance, float3* proj) {
    float3 q = p;
    const bool hit = sdf8 ? sdf_collide_from8(sdf8, g, margin, p, distance, q) : sdf_collide_from(sdf, g, margin, p, distance, q);
    *proj = q;
    return hit;
}

// What the vertices of one group share: the object's buffers, SDF, grid, margin, tip separation.
struct FollowGroup {
    HairView h;
    const float* sdf;
    const float4* sdf8;
    SdfGrid sg;
    float margin, tip;
    int firstStrand;     // first strand of the group (guide strands and their follows)
};

__device__ __forceinline__ bool follow_group(const BatchObject& ob, const WorkItem& wi, FollowGroup& fg) {
    fg.h = ob.hair;
    fg.sdf = ob.sdf;
    fg.sdf8 = ob.sdf8;
    if (fg.h.F == 0 && !fg.sdf) return false;
    fg.sg = SdfGrid{0.f, 0.f, 0.f, 1.f, 0, 0, 0, 0};
    fg.margin = 0.0f;
    if (fg.sdf) { fg.sg = ob.sdfFrame->grid; fg.margin = ob.sdfFrame->margin; }
    fg.tip = ob.consts->tipSeparation;
    fg.firstStrand = wi.firstGuide * (fg.h.F + 1);
    return true;
}

// Guide vertex e of a group: its follow vertices and the collision of all of them.  NF: every object
// of the class has no follow hairs (F = 0 known at compile time, which frees registers).
template <int N, bool NF>
__device__ __forceinline__ void follow_collide_vertex(const FollowGroup& fg, int e) {
    constexpr float kInvN = 1.0f / (float)N;   // exact: N is a power of two, so j * kInvN == j / N
    const HairView& h = fg.h;
    const int F = NF ? 0 : h.F;
    const float* __restrict__ sdf = fg.sdf;
    const float4* __restrict__ sdf8 = fg.sdf8;
    const SdfGrid& sg = fg.sg;
    const float margin = fg.margin, tip = fg.tip;
    const int s = e / N, j = e % N;
    const int gs = fg.firstStrand + s * (F + 1);
    const size_t vg = (size_t)gs * N + j;
    const float4 gp = h.pos[vg];
    const float4 tn = F > 0 ? h.tan[vg] : make_float4(0.f, 0.f, 0.f, 0.f);   // copied to the follow vertices only
    const bool collide = sdf && j >= 2;
    const float factor = tip * ((float)j * kInvN) + 1.0f;
    for (int i = 0; i <= F; ++i) {
        const size_t v = vg + (size_t)i * N;
        float3 pt = xyz(gp);
        float w = gp.w;
        if (i > 0) {
            const float4 off = __ldg(h.followOffset + gs + i);
            pt = add(xyz(gp), mul(factor, xyz(off)));
            // inverse mass of the follow vertex: only this thread writes the word, after this read
            w = __ldg(&h.pos[v].w);
        }
        float3 proj = pt;
        bool hit = false;
        if (collide) {
            const float dist = sdf8 ? sdf_lookup8(sdf8, sg, pt) : sdf_lookup(sdf, sg, pt);
            if (dist <= margin) hit = collide_near(sdf, sdf8, sg, margin, pt, dist, &proj);
        }
        if (i > 0) {
            h.pos[v] = make_float4(proj.x, proj.y, proj.z, w);
            h.tan[v] = tn;
        } else if (hit) {
            h.pos[v] = with_xyz(gp, proj);
        }
        if (hit) h.prev[v] = with_xyz(h.prev[v], proj);
    }
}

// ============================================================================================
// follow hairs + collision
//
// UpdateFollowHairVertices (TressFXSimulation.hlsl:978-1001) and CollideHairVerticesWithSdf_forward
// (TressFXSDFCollision.hlsl:531-595) for the groups of one vertices-per-strand class, after
// k_fused_strands has written the guides' constrained state and the frame's SDFs are built.  One
// thread per guide vertex; it makes the vertex's F follow vertices (hair i = 1..F) from the guide's
// pre-collision position, then collides the guide vertex and every follow vertex (one vertex at a
// time: at 64 registers four blocks fit per SM, and that occupancy hides the gathers better than
// loads of several hairs in flight per thread did).  Each group
// is cut into chunksPerItem chunks of guide vertices (a multiple of 256), which persistent blocks take
// in turn: with few groups per block, smaller chunks spread groups of unequal cost (collisions) evenly
// over the SMs; with many, whole groups keep the per-chunk overhead low.
template <int N, bool NF>
__global__ void __launch_bounds__(256, NF ? 5 : 4) k_follow_collide(const BatchObject* __restrict__ objs,
                                                           const WorkItem* __restrict__ items, int numItems,
                                                           int chunksPerItem) {
    constexpr int kGroupVerts = fused_group_strands(N) * N;
    const int chunkLen = ((kGroupVerts + chunksPerItem - 1) / chunksPerItem + 255) & ~255;
    const int numChunks = numItems * chunksPerItem;
    for (int c = blockIdx.x; c < numChunks; c += gridDim.x) {
        const int it = c / chunksPerItem;
        const WorkItem wi = items[it];
        const int begin = (c - it * chunksPerItem) * chunkLen;
        const int end = min(begin + chunkLen, wi.count * N);
        FollowGroup fg;
        if (!follow_group(objs[wi.obj], wi, fg)) continue;
        for (int e = begin + (int)threadIdx.x; e < end; e += blockDim.x) follow_collide_vertex<N, NF>(fg, e);
    }
}

// ============================================================================================
// follow hairs + collision with per-warp lookup queues (classes whose objects have follow hairs)
//
// The same work as k_follow_collide, with the warp's lanes decoupled from its lookups: lane l owns one
// guide vertex, makes and writes its follow vertices, and queues every vertex (guide or follow) the
// collision may move (j >= 2, not certainly outside the grid).  The warp runs the first lookup on 32
// queued vertices at a time, then the gradient stage on 32 of those within the margin at a time, so
// both run on full warps: a strand reaches from the scalp, where vertices touch the surface, out to
// tips far from it, and with follow hairs a lane has F + 1 vertices of that mix.  A moved vertex gets
// Pos and Prev from the lane that collided it, after the owner's write of the follow's Pos
// (__syncwarp orders the two).  The queues are emptied at the end of each chunk.
constexpr int kFollowWarps = 8;
struct FollowQueues {
    int idx1[kFollowWarps][64];      // stage 1: offset of the vertex in the group
    float4 pos1[kFollowWarps][64];   //          its position and inverse mass
    int idx2[kFollowWarps][64];      // stage 2: the same, for vertices within the margin
    float4 pos2[kFollowWarps][64];
    float dist2[kFollowWarps][64];   //          and their first lookup's distance
};

// Lane k < n takes entry k of a queue; the entries from 32 on move to the front.
__device__ __forceinline__ bool queue_take(int* idx, float4* pos, float* dist, int& n, int lane, int& ri, float4& rp,
                                           float& rd) {
    __syncwarp();
    const bool have = lane < n;
    if (have) { ri = idx[lane]; rp = pos[lane]; if (dist) rd = dist[lane]; }
    __syncwarp();
    if (lane < n - 32) { idx[lane] = idx[lane + 32]; pos[lane] = pos[lane + 32]; if (dist) dist[lane] = dist[lane + 32]; }
    __syncwarp();
    n = max(n - 32, 0);
    return have;
}

// Stage 2 on up to 32 queued vertices: the gradient lookups and, inside the margin, the projection.
__device__ __forceinline__ void follow_stage2(const FollowGroup& fg, size_t vbase, FollowQueues& Q, int warp, int lane,
                                              int& n2) {
    int ri = 0; float4 rp = make_float4(0.f, 0.f, 0.f, 0.f); float rd = 0.0f;
    if (!queue_take(Q.idx2[warp], Q.pos2[warp], Q.dist2[warp], n2, lane, ri, rp, rd)) return;
    float3 proj;
    if (collide_near(fg.sdf, fg.sdf8, fg.sg, fg.margin, xyz(rp), rd, &proj)) {
        const size_t v = vbase + (size_t)ri;
        fg.h.pos[v] = make_float4(proj.x, proj.y, proj.z, rp.w);
        fg.h.prev[v] = with_xyz(fg.h.prev[v], proj);
    }
}

// Stage 1 on up to 32 queued vertices: the first lookup; those within the margin join stage 2.
__device__ __forceinline__ void follow_stage1(const FollowGroup& fg, size_t vbase, FollowQueues& Q, int warp, int lane,
                                              int& n1, int& n2) {
    int ri = 0; float4 rp = make_float4(0.f, 0.f, 0.f, 0.f); float rd = 0.0f;
    const bool have = queue_take(Q.idx1[warp], Q.pos1[warp], nullptr, n1, lane, ri, rp, rd);
    bool near = false;
    if (have) {
        rd = fg.sdf8 ? sdf_lookup8(fg.sdf8, fg.sg, xyz(rp)) : sdf_lookup(fg.sdf, fg.sg, xyz(rp));
        near = rd <= fg.margin;
    }
    const unsigned m = __ballot_sync(0xffffffffu, near);
    if (near) {
        const int k = n2 + __popc(m & ((1u << lane) - 1u));
        Q.idx2[warp][k] = ri; Q.pos2[warp][k] = rp; Q.dist2[warp][k] = rd;
    }
    n2 += __popc(m);
    if (n2 >= 32) follow_stage2(fg, vbase, Q, warp, lane, n2);
}

// QueueFirst = false: each lane runs its vertices' first lookup itself and only the vertices within
// the margin are queued (for classes without follow hairs, where a lane has one vertex per step).
template <int N, bool QueueFirst, bool NF>
__global__ void __launch_bounds__(256, NF ? 5 : 4) k_follow_collide_queued(const BatchObject* __restrict__ objs,
                                                                  const WorkItem* __restrict__ items, int numItems,
                                                                  int chunksPerItem) {
    constexpr int kGroupVerts = fused_group_strands(N) * N;
    constexpr float kInvN = 1.0f / (float)N;   // exact: N is a power of two, so j * kInvN == j / N
    __shared__ FollowQueues Q;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const int chunkLen = ((kGroupVerts + chunksPerItem - 1) / chunksPerItem + 255) & ~255;
    const int numChunks = numItems * chunksPerItem;
    for (int c = blockIdx.x; c < numChunks; c += gridDim.x) {
        const int it = c / chunksPerItem;
        const WorkItem wi = items[it];
        const int begin = (c - it * chunksPerItem) * chunkLen;
        const int end = min(begin + chunkLen, wi.count * N);
        FollowGroup fg;
        if (!follow_group(objs[wi.obj], wi, fg)) continue;
        const HairView& h = fg.h;
        const int F = NF ? 0 : h.F;
        const size_t vbase = (size_t)fg.firstStrand * N;
        int n1 = 0, n2 = 0;
        for (int base = begin + warp * 32; base < end; base += blockDim.x) {
            const int e = base + lane;
            const bool active = e < end;
            const int s = e / N, j = e % N;
            const int gs = fg.firstStrand + s * (F + 1);
            const size_t vg = (size_t)gs * N + j;
            float4 gp = make_float4(0.f, 0.f, 0.f, 0.f), tn = gp;
            if (active) {
                gp = h.pos[vg];
                if (F > 0) tn = h.tan[vg];   // copied to the follow vertices only
            }
            const bool collide = active && fg.sdf && j >= 2;
            const float factor = fg.tip * ((float)j * kInvN) + 1.0f;
            for (int i = 0; i <= F; ++i) {
                const size_t v = vg + (size_t)i * N;
                float3 pt = xyz(gp);
                float w = gp.w;
                if (active && i > 0) {
                    const float4 off = __ldg(h.followOffset + gs + i);
                    pt = add(xyz(gp), mul(factor, xyz(off)));
                    // inverse mass of the follow vertex: only this lane writes the word, after this read
                    w = __ldg(&h.pos[v].w);
                    h.pos[v] = make_float4(pt.x, pt.y, pt.z, w);
                    h.tan[v] = tn;
                }
                const bool need = collide && !sdf_surely_outside(fg.sg, pt);
                if (QueueFirst) {
                    const unsigned m = __ballot_sync(0xffffffffu, need);
                    if (need) {
                        const int k = n1 + __popc(m & below);
                        Q.idx1[warp][k] = (int)(v - vbase);
                        Q.pos1[warp][k] = make_float4(pt.x, pt.y, pt.z, w);
                    }
                    n1 += __popc(m);
                    if (n1 >= 32) follow_stage1(fg, vbase, Q, warp, lane, n1, n2);
                } else {
                    float d = 0.0f;
                    if (need) d = fg.sdf8 ? sdf_lookup8(fg.sdf8, fg.sg, pt) : sdf_lookup(fg.sdf, fg.sg, pt);
                    const bool near = need && d <= fg.margin;
                    const unsigned m = __ballot_sync(0xffffffffu, near);
                    if (near) {
                        const int k = n2 + __popc(m & below);
                        Q.idx2[warp][k] = (int)(v - vbase);
                        Q.pos2[warp][k] = make_float4(pt.x, pt.y, pt.z, w);
                        Q.dist2[warp][k] = d;
                    }
                    n2 += __popc(m);
                    if (n2 >= 32) follow_stage2(fg, vbase, Q, warp, lane, n2);
                }
            }
        }
        while (n1 > 0) follow_stage1(fg, vbase, Q, warp, lane, n1, n2);
        while (n2 > 0) follow_stage2(fg, vbase, Q, warp, lane, n2);
        __syncwarp();
    }
}

// ============================================================================================
// readback snapshot: every object's positions, one after the other, as float4 (xyzw) or packed xyz
__global__ void __launch_bounds__(256) k_snapshot_positions(const BatchObject* __restrict__ objs,
                                                            const long long* __restrict__ first, int nobj,
                                                            long long total, float* __restrict__ out, int xyzOnly) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += stride) {
        int lo = 0, hi = nobj - 1;
        while (lo < hi) {   // last object whose first vertex <= t
            const int mid = (lo + hi + 1) >> 1;
            if (first[mid] <= t) lo = mid; else hi = mid - 1;
        }
        const float4 p = objs[lo].hair.pos[t - first[lo]];
        if (xyzOnly) {
            out[3 * t] = p.x; out[3 * t + 1] = p.y; out[3 * t + 2] = p.z;
        } else {
            reinterpret_cast<float4*>(out)[t] = p;
        }
    }
}

cudaError_t launch_snapshot_positions(const BatchObject* objs, const long long* first, int nobj, long long total,
                                      float* out, int xyzOnly, cudaStream_t s) {
    if (total <= 0) return cudaSuccess;
    const unsigned blocks = (unsigned)std::min<long long>((total + 255) / 256, (long long)sm_count() * 16);
    k_snapshot_positions<<<blocks, 256, 0, s>>>(objs, first, nobj, total, out, xyzOnly);
    return cudaGetLastError();
}

// ============================================================================================
// host launch helpers
template <int N, int VPL>
static cudaError_t launch_fused_nv(const FusedLaunch& fl, cudaStream_t s) {
    // the dynamic shared-memory attribute is set by fused_blocks_per_sm before the first launch
    k_fused_strands<N, VPL><<<fl.blocks, fl.warpsPerBlock * 32, fused_smem_for(N), s>>>(fl.objs, fl.items, fl.numItems,
                                                                                        fl.err, fl.mode, fl.waitPolls);
    return cudaGetLastError();
}

bool fused_config_valid(int n, int vpl) {
    if (vpl < 1 || n % vpl != 0) return false;
    const int L = n / vpl;
    if (L > 32 || 32 % L != 0 || L < 2) return false;
    if (vpl > 1 && (vpl % 2) != 0) return false;
    return vpl <= 4;
}

int fused_smem_bytes(int n, int, int) { return fused_smem_for(n); }

template <int N>
static cudaError_t launch_sweep_n(const FusedLaunch& fl, cudaStream_t s) {
    constexpr int IPW = 32 / fused_group_strands(N);
    const long long threads = (long long)((fl.numItems + IPW - 1) / IPW) * 32;
    k_local_sweep<N><<<(unsigned)((threads + 127) / 128), 128, 0, s>>>(fl.objs, fl.items, fl.numItems);
    return cudaGetLastError();
}

cudaError_t launch_local_sweep(const FusedLaunch& fl, cudaStream_t s) {
    if (fl.numItems <= 0) return cudaSuccess;
    switch (fl.n) {
        case 4: return launch_sweep_n<4>(fl, s);
        case 8: return launch_sweep_n<8>(fl, s);
        case 16: return launch_sweep_n<16>(fl, s);
        case 32: return launch_sweep_n<32>(fl, s);
        case 64: return launch_sweep_n<64>(fl, s);
        default: return cudaErrorInvalidValue;
    }
}
int fused_group_size(int n) { return fused_group_strands(n); }

#define TFX_FUSED_CASE(NN, VV) \
    if (fl.n == NN && fl.vpl == VV) return launch_fused_nv<NN, VV>(fl, s);

cudaError_t launch_fused_strands(const FusedLaunch& fl, cudaStream_t s) {
    TFX_FUSED_CASE(4, 1)
    TFX_FUSED_CASE(4, 2)
    TFX_FUSED_CASE(8, 1)
    TFX_FUSED_CASE(8, 2)
    TFX_FUSED_CASE(8, 4)
    TFX_FUSED_CASE(16, 1)
    TFX_FUSED_CASE(16, 2)
    TFX_FUSED_CASE(16, 4)
    TFX_FUSED_CASE(32, 1)
    TFX_FUSED_CASE(32, 2)
    TFX_FUSED_CASE(32, 4)
    TFX_FUSED_CASE(64, 2)
    TFX_FUSED_CASE(64, 4)
    return cudaErrorInvalidValue;
}

#define TFX_FUSED_OCC(NN, VV)                                                                                     \
    if (n == NN && vpl == VV) {                                                                                   \
        int nb = 0;                                                                                               \
        cudaError_t e = cudaFuncSetAttribute(k_fused_strands<NN, VV>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                             fused_smem_for(NN));                                                 \
        if (e != cudaSuccess) return 0;                                                                           \
        e = cudaFuncSetAttribute(k_fused_strands<NN, VV>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);    \
        if (e != cudaSuccess) return 0;                                                                           \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fused_strands<NN, VV>, warps * 32, fused_smem_for(NN)); \
        return nb;                                                                                                \
    }

int fused_blocks_per_sm(int n, int vpl, int warps) {
    TFX_FUSED_OCC(4, 1)
    TFX_FUSED_OCC(4, 2)
    TFX_FUSED_OCC(8, 1)
    TFX_FUSED_OCC(8, 2)
    TFX_FUSED_OCC(8, 4)
    TFX_FUSED_OCC(16, 1)
    TFX_FUSED_OCC(16, 2)
    TFX_FUSED_OCC(16, 4)
    TFX_FUSED_OCC(32, 1)
    TFX_FUSED_OCC(32, 2)
    TFX_FUSED_OCC(32, 4)
    TFX_FUSED_OCC(64, 2)
    TFX_FUSED_OCC(64, 4)
    return 0;
}

int follow_max_chunks_per_item(int n) { return (fused_group_strands(n) * n + 255) / 256; }

template <int N, bool NF>
static cudaError_t launch_follow_nf(const FollowLaunch& fl, cudaStream_t s) {
    if (fl.queued == 1)
        k_follow_collide_queued<N, true, NF><<<fl.blocks, 256, 0, s>>>(fl.objs, fl.items, fl.numItems, fl.chunks);
    else if (fl.queued == 2)
        k_follow_collide_queued<N, false, NF><<<fl.blocks, 256, 0, s>>>(fl.objs, fl.items, fl.numItems, fl.chunks);
    else
        k_follow_collide<N, NF><<<fl.blocks, 256, 0, s>>>(fl.objs, fl.items, fl.numItems, fl.chunks);
    return cudaGetLastError();
}

template <int N>
static cudaError_t launch_follow_n(const FollowLaunch& fl, cudaStream_t s) {
    return fl.noFollow ? launch_follow_nf<N, true>(fl, s) : launch_follow_nf<N, false>(fl, s);
}

template <bool NF>
static cudaError_t follow_occupancy(int n, int mode, int* nb) {
#define TFX_FOLLOW_OCC(NN)                                                                                                \
    case NN:                                                                                                              \
        return mode == 1   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(nb, k_follow_collide_queued<NN, true, NF>, 256, 0)  \
               : mode == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(nb, k_follow_collide_queued<NN, false, NF>, 256, 0) \
                           : cudaOccupancyMaxActiveBlocksPerMultiprocessor(nb, k_follow_collide<NN, NF>, 256, 0);
    switch (n) {
        TFX_FOLLOW_OCC(4)
        TFX_FOLLOW_OCC(8)
        TFX_FOLLOW_OCC(16)
        TFX_FOLLOW_OCC(32)
        TFX_FOLLOW_OCC(64)
        default: return cudaErrorInvalidValue;
    }
#undef TFX_FOLLOW_OCC
}

int follow_blocks_per_sm(int n, int mode, bool noFollow) {
    int nb = 0;
    const cudaError_t e = noFollow ? follow_occupancy<true>(n, mode, &nb) : follow_occupancy<false>(n, mode, &nb);
    return e == cudaSuccess ? nb : 0;
}

cudaError_t launch_follow_collide(const FollowLaunch& fl, cudaStream_t s) {
    if (fl.numItems <= 0) return cudaSuccess;
    switch (fl.n) {
        case 4: return launch_follow_n<4>(fl, s);
        case 8: return launch_follow_n<8>(fl, s);
        case 16: return launch_follow_n<16>(fl, s);
        case 32: return launch_follow_n<32>(fl, s);
        case 64: return launch_follow_n<64>(fl, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_batch_mesh_skin(const BatchMesh* meshes, int nmeshes, int totalVerts, cudaStream_t s) {
    if (totalVerts <= 0) return cudaSuccess;
    k_batch_mesh_skin<<<(totalVerts + 255) / 256, 256, 0, s>>>(meshes, nmeshes, totalVerts);
    return cudaGetLastError();
}

// CollideHairVerticesWithSdf_forward (TressFXSDFCollision.hlsl:531-595) of every vertex of a level's
// objects against that pair's SDF (the decoded float grid), one thread per vertex; vertices 0 and 1 of a
// strand are left alone, as the shader does.  Same arithmetic as k_sdf_collide.
__global__ void __launch_bounds__(256) k_collide_level(const BatchObject* __restrict__ objs, const BatchSdf* __restrict__ sdfs,
                                                       const BatchCollide* __restrict__ pairs, int npairs, long long total) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += stride) {
        int lo = 0, hi = npairs - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (pairs[mid].firstVertex <= i) lo = mid; else hi = mid - 1;
        }
        const BatchCollide pc = pairs[lo];
        const HairView& h = objs[pc.obj].hair;
        const long long v = i - pc.firstVertex;
        const int local = (int)(v % h.n);
        if (local == 0 || local == 1) continue;
        const BatchSdf& sd = sdfs[pc.sdf];
        const SdfGrid g = sd.frame->grid;
        const float margin = sd.frame->margin;
        const float* sdf = reinterpret_cast<const float*>(sd.words);
        const float4 hv = h.pos[v];
        float3 proj;
        if (sdf_collide_point(sdf, g, margin, xyz(hv), proj)) {
            h.pos[v] = with_xyz(hv, proj);
            h.prev[v] = with_xyz(h.prev[v], proj);
        }
    }
}

cudaError_t launch_collide_level(const BatchObject* objs, const BatchSdf* sdfs, const BatchCollide* pairs, int npairs,
                                 long long totalVertices, cudaStream_t s) {
    if (npairs <= 0 || totalVertices <= 0) return cudaSuccess;
    const unsigned blocks = (unsigned)std::min<long long>((totalVertices + 255) / 256, (long long)sm_count() * 16);
    k_collide_level<<<blocks, 256, 0, s>>>(objs, sdfs, pairs, npairs, totalVertices);
    return cudaGetLastError();
}

cudaError_t launch_batch_sdf(const SdfBatchLaunch& L, cudaStream_t s) {
    if (L.nsdf <= 0) return cudaSuccess;
    const long long q = L.totalQuads;
    const unsigned gq = (unsigned)std::min<long long>((q + 255) / 256, (long long)sm_count() * 32);
    k_batch_sdf_init<<<gq, 256, 0, s>>>(L.sdfs, L.nsdf, q);
    if (L.totalTris > 0) {
        const int warpsPerBlock = L.constructThreads / 32;
        const int per = sdf_construct_chunk(L.totalTris, sm_count());
        const long long chunks = ((long long)L.totalTris + per - 1) / per;
        const unsigned blocks =
            (unsigned)std::min<long long>((chunks + warpsPerBlock - 1) / warpsPerBlock, (long long)sm_count() * 64);
        const bool staged = per >= kTriJobsStagedFrom;
        if (warpsPerBlock == 2 && staged)
            k_batch_sdf_construct<2, true><<<blocks, 64, 0, s>>>(L.sdfs, L.nsdf, L.totalTris, per);
        else if (warpsPerBlock == 2)
            k_batch_sdf_construct<2, false><<<blocks, 64, 0, s>>>(L.sdfs, L.nsdf, L.totalTris, per);
        else if (warpsPerBlock == 8 && staged)
            k_batch_sdf_construct<8, true><<<blocks, 256, 0, s>>>(L.sdfs, L.nsdf, L.totalTris, per);
        else if (warpsPerBlock == 8)
            k_batch_sdf_construct<8, false><<<blocks, 256, 0, s>>>(L.sdfs, L.nsdf, L.totalTris, per);
        else if (staged)
            k_batch_sdf_construct<4, true><<<blocks, 128, 0, s>>>(L.sdfs, L.nsdf, L.totalTris, per);
        else
            k_batch_sdf_construct<4, false><<<blocks, 128, 0, s>>>(L.sdfs, L.nsdf, L.totalTris, per);
    }
    k_batch_sdf_finalize<<<gq, 256, 0, s>>>(L.sdfs, L.nsdf, q);
    if (L.expand) return launch_batch_sdf_expand(L, s);
    return cudaGetLastError();
}

cudaError_t launch_batch_sdf_expand(const SdfBatchLaunch& L, cudaStream_t s) {
    if (L.nsdf <= 0 || !L.expand || L.expCells <= 0) return cudaSuccess;
    const unsigned ge = (unsigned)std::min<long long>((L.expCells + 255) / 256, (long long)sm_count() * 32);
    k_batch_sdf_expand<<<ge, 256, 0, s>>>(L.sdfs, L.expSdf, L.expFirst, L.nexp, L.expCells);
    return cudaGetLastError();
}

}  // namespace tfx
