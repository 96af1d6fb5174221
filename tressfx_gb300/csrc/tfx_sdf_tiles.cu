// The batched SDF build as a tile-binned construct with exact pair culling.
//
// InitializeSignedDistanceField + ConstructSignedDistanceField + FinalizeSignedDistanceField
// (TressFXSDFCollision.hlsl:301-412) give every cell the minimum, over the triangles whose cell box
// (:351-363) contains the cell, of FloatFlip3(SignedDistancePointToTriangle(cell corner, triangle)),
// and FloatFlip3(1e10) where no box reaches.  The reference evaluates every (triangle, cell) pair of
// every box and resolves the minimum with an atomicMin per pair in device memory.  Here:
//
//  1. k_sdf_bin_count writes each triangle's record (vertices, cell box and the terms of a lower bound
//     on its distance) and counts the 8x8x4-cell tiles its box overlaps; k_sdf_bin_scan_* and
//     k_sdf_bin_fill list each tile's candidate triangles.  A triangle whose box spans more than
//     SDF_BIG_TILES tiles goes to its SDF's big list, which every tile of the SDF scans.
//  2. k_sdf_tiles gives each tile to one block of eight warps, warp w owning a 4x4x2-cell brick, lane l
//     one cell of it, with the cell's running minimum word in shared memory and its magnitude in a
//     register.  The tile's candidate records are staged in shared memory; each warp keeps those whose
//     box overlaps its brick, ordered nearest first (counting sort on the distance from the brick's
//     centre to the triangle, in quarter cells), and walks them: a lane tests whether its cell lies in
//     the record's box and whether the lower bound proves the pair farther than its cell's current word;
//     the pairs left are queued and evaluated 32 at a time, one per lane, into the cell's word with an
//     atomicMin in shared memory.  The block then writes the decoded floats of its cells (the finalized
//     grid): no separate initialise or finalise pass, no atomic in device memory per pair.
//
// Exactness.  Every evaluated pair uses the reference's arithmetic (signed_dist_pre, bit-identical to
// SignedDistancePointToTriangle), and the minimum over FloatFlip3 words does not depend on the order.
// A pair is skipped only when its computed distance is provably larger in magnitude than the cell's
// current word; FloatFlip3 orders words by |d| first, so its word is then larger and cannot be the
// minimum.  The proof: both branches of SignedDistancePointToTriangle return the distance from p to a
// point q that lies in the triangle up to rounding (barycentrics >= -1e-8 summing to one, or a point on
// an edge), so the computed |d| >= (dist(p, T) - delta)(1 - 5 eps) with delta <= 15 eps max|x_i| +
// 6e-8 R, whatever the triangle's shape.  dist(p, T) is bounded below by splitting p - c (c the
// centroid) along a unit normal m: dist^2 >= (|h_p| - w)+^2 + (|u_p| - R)+^2, with h_p = <p - c, m>,
// u_p the rest, w = max_i |<x_i - c, m>| and R = max_i |x_i - c| (valid for any c and any unit m, since
// the triangle is the hull of its vertices; a degenerate triangle takes m = 0, the sphere bound).  The
// bound is evaluated in float and compared with 2^-18-relative and 2^-18 x (max|x_i| + R + w) absolute
// slack, several times the rounding of either side.  Any NaN makes the bound 0 or the test false, which
// evaluates the pair.
#include "tfx_batch.h"
#include "tfx_sdf_math.cuh"

namespace tfx {

namespace {

constexpr int TX = 8, TY = 8, TZ = 4;              // cells per tile edge
constexpr int TILE_CELLS = TX * TY * TZ;           // 256: eight 4x4x2 bricks
constexpr int TILE_THREADS = 256;                  // a warp per brick, a lane per cell
constexpr int TILE_WARPS = TILE_THREADS / 32;
constexpr int CH = 256;                            // candidate records in shared memory at a time
constexpr int REC = 20;                            // words of a triangle record
constexpr int RS = 21;                             // their stride in shared memory (odd: lanes on different records do not conflict)
constexpr int NBUCKET = 16;                        // quarter-cell distance buckets of a brick's list, the last open
constexpr int QCAP = 64;                           // queue entries per warp
constexpr int SCAN_BLOCK = 1024;
constexpr unsigned FULL = 0xffffffffu;

// record layout (words): x0 x1 x2 | centroid | unit normal or 0 | R | w | slack | packed box lo, hi
constexpr int R_X = 0;
constexpr int R_C = 9;
constexpr int R_M = 12;
constexpr int R_R = 15;
constexpr int R_W = 16;
constexpr int R_S = 17;
constexpr int R_LO = 18;
constexpr int R_HI = 19;

__device__ __forceinline__ int pack_cell(int3 c) { return c.x | (c.y << 10) | (c.z << 20); }
__device__ __forceinline__ int3 unpack_cell(int v) { return make_int3(v & 1023, (v >> 10) & 1023, (v >> 20) & 1023); }

__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ int sdf_of_triangle(const BatchSdf* __restrict__ sdfs, int nsdf, int t) {
    int lo = 0, hi = nsdf - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sdfs[mid].firstTriangle <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int sdf_of_tile(const BatchSdf* __restrict__ sdfs, int nsdf, int tile) {
    int lo = 0, hi = nsdf - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sdfs[mid].firstTile <= tile) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// The tiles of an SDF that the packed cell box [lo, hi] overlaps.
__device__ __forceinline__ void box_tiles(int lo, int hi, int3& a, int3& b) {
    const int3 l = unpack_cell(lo), h = unpack_cell(hi);
    a = make_int3(l.x / TX, l.y / TY, l.z / TZ);
    b = make_int3(h.x / TX, h.y / TY, h.z / TZ);
}

__device__ __forceinline__ int tile_start(const SdfTileLaunch& L, int tile) {
    return L.tileStart[tile] + L.blockSum[tile / SCAN_BLOCK];
}

// Global triangle index of candidate `cand` of a tile: its own list first, then its SDF's big list.
__device__ __forceinline__ int candidate_triangle(const SdfTileLaunch& L, const BatchSdf& s, int listStart, int nList,
                                                  int cand) {
    return cand < nList ? L.list[listStart + cand] : L.bigList[s.firstTriangle + (cand - nList)];
}

// ------------------------------------------------------------------------------------------ binning
// The record of triangle t (REC words): its vertices, the bound's terms and the reference's cell box.
__device__ void make_record(const BatchSdf& s, const SdfGrid& g, int tri, float* rec, int& boxLo, int& boxHi) {
    const float3 x0 = xyz(__ldg(s.mesh + 2 * (size_t)__ldg(s.indices + 3 * tri + 0)));
    const float3 x1 = xyz(__ldg(s.mesh + 2 * (size_t)__ldg(s.indices + 3 * tri + 1)));
    const float3 x2 = xyz(__ldg(s.mesh + 2 * (size_t)__ldg(s.indices + 3 * tri + 2)));
    int3 lo, hi;
    tri_cell_box(g, x0, x1, x2, lo, hi);   // the reference's clamped box: never empty
    const float third = 1.0f / 3.0f;
    const float3 c = mul(add(add(x0, x1), x2), third);
    const float3 a0 = sub(x0, c), a1 = sub(x1, c), a2 = sub(x2, c);
    const float R = sqrtf(fmaxf(fmaxf(dot(a0, a0), dot(a1, a1)), dot(a2, a2)));
    const float3 n = cross(sub(x1, x0), sub(x2, x0));
    const float nn = dot(n, n);
    float3 m = mk3(0.0f, 0.0f, 0.0f);
    if (nn > 1e-30f && nn < 1e30f) m = mul(n, rsqrtf(nn));
    const float w = fmaxf(fmaxf(fabsf(dot(a0, m)), fabsf(dot(a1, m))), fabsf(dot(a2, m)));
    const float Mt = fmaxf(fmaxf(fabsf(x0.x) + fabsf(x0.y) + fabsf(x0.z), fabsf(x1.x) + fabsf(x1.y) + fabsf(x1.z)),
                           fabsf(x2.x) + fabsf(x2.y) + fabsf(x2.z));
    boxLo = pack_cell(lo);
    boxHi = pack_cell(hi);
    const float v[REC] = {x0.x, x0.y, x0.z, x1.x, x1.y, x1.z, x2.x, x2.y, x2.z, c.x, c.y, c.z, m.x, m.y, m.z, R, w,
                          0x1p-18f * ((Mt + R) + w) + 2e-7f * R, __int_as_float(boxLo), __int_as_float(boxHi)};
#pragma unroll
    for (int k = 0; k < REC; ++k) rec[k] = v[k];
}

__global__ void __launch_bounds__(256) k_sdf_bin_count(SdfTileLaunch L) {
    const int stride = gridDim.x * blockDim.x;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < L.totalTris; t += stride) {
        const int si = sdf_of_triangle(L.sdfs, L.nsdf, t);
        const BatchSdf& s = L.sdfs[si];
        const SdfGrid g = s.frame->grid;
        float rec[REC];
        int plo, phi;
        make_record(s, g, t - s.firstTriangle, rec, plo, phi);
        float4* dst = reinterpret_cast<float4*>(L.records + (size_t)t * REC);
#pragma unroll
        for (int k = 0; k < REC / 4; ++k) dst[k] = make_float4(rec[4 * k], rec[4 * k + 1], rec[4 * k + 2], rec[4 * k + 3]);
        int3 a, b;
        box_tiles(plo, phi, a, b);
        const int ntiles = (b.x - a.x + 1) * (b.y - a.y + 1) * (b.z - a.z + 1);
        if (ntiles > SDF_BIG_TILES) {
            const int k = atomicAdd(L.bigCount + si, 1);
            L.bigList[s.firstTriangle + k] = t;
            continue;
        }
        for (int z = a.z; z <= b.z; ++z)
            for (int y = a.y; y <= b.y; ++y)
                for (int x = a.x; x <= b.x; ++x) atomicAdd(L.tileCount + s.firstTile + (z * s.tilesY + y) * s.tilesX + x, 1);
    }
}

// Block-wide inclusive scan of one int per thread (1024 threads); returns the inclusive value.
__device__ __forceinline__ int block_scan_1024(int v, int* warpSums) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warpSums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int s = warpSums[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, s, o);
            if (lane >= o) s += y;
        }
        warpSums[lane] = s;
    }
    __syncthreads();
    return x + (warp > 0 ? warpSums[warp - 1] : 0);
}

// Exclusive prefix of the tile counts within blocks of 1024 tiles; the counts become the fill cursors.
__global__ void __launch_bounds__(SCAN_BLOCK) k_sdf_bin_scan_local(SdfTileLaunch L) {
    __shared__ int warpSums[32];
    const int i = blockIdx.x * SCAN_BLOCK + threadIdx.x;
    const int v = i < L.totalTiles ? L.tileCount[i] : 0;
    const int incl = block_scan_1024(v, warpSums);
    if (i < L.totalTiles) {
        L.tileStart[i] = incl - v;
        L.tileCount[i] = 0;
    }
    if (threadIdx.x == SCAN_BLOCK - 1) L.blockSum[blockIdx.x] = incl;
}

// Exclusive prefix of the block totals, in place (one block, any number of scan blocks).
__global__ void __launch_bounds__(SCAN_BLOCK) k_sdf_bin_scan_top(int* __restrict__ blockSum, int nb) {
    __shared__ int warpSums[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += SCAN_BLOCK) {
        const int i = base + threadIdx.x;
        const int v = i < nb ? blockSum[i] : 0;
        const int incl = block_scan_1024(v, warpSums);
        const int c = carry;
        __syncthreads();
        if (i < nb) blockSum[i] = c + incl - v;
        if (threadIdx.x == SCAN_BLOCK - 1) carry = c + incl;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_sdf_bin_fill(SdfTileLaunch L) {
    const int stride = gridDim.x * blockDim.x;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < L.totalTris; t += stride) {
        const int si = sdf_of_triangle(L.sdfs, L.nsdf, t);
        const BatchSdf& s = L.sdfs[si];
        const float* rec = L.records + (size_t)t * REC;
        int3 a, b;
        box_tiles(__float_as_int(rec[R_LO]), __float_as_int(rec[R_HI]), a, b);
        if ((b.x - a.x + 1) * (b.y - a.y + 1) * (b.z - a.z + 1) > SDF_BIG_TILES) continue;
        for (int z = a.z; z <= b.z; ++z)
            for (int y = a.y; y <= b.y; ++y)
                for (int x = a.x; x <= b.x; ++x) {
                    const int tile = s.firstTile + (z * s.tilesY + y) * s.tilesX + x;
                    const long long at = (long long)tile_start(L, tile) + atomicAdd(L.tileCount + tile, 1);
                    if (at < L.listCapacity) L.list[at] = t;
                }
    }
}

// ------------------------------------------------------------------------------------------ tiles
struct TileSmem {
    float rec[CH * RS];                    // the records of the current chunk of candidates
    uint32_t words[TILE_CELLS];            // FloatFlip3 words of the tile's cells, warp-major (brick, lane)
    uint16_t list[TILE_WARPS][CH];         // per warp: chunk records overlapping its brick, nearest first
    uint32_t queue[TILE_WARPS][QCAP];      // per warp: pairs to evaluate, lane | record << 5
    int bucket[TILE_WARPS][NBUCKET];       // per warp: counting-sort counters, then cursors
    int tile;
};

// Squared lower bound on the distance from p to the record's triangle, and in `extra` the per-pair
// slack 2^-18 (|h| + |u|) (see the exactness note above).
__device__ __forceinline__ float lower_bound2(const float* r, float3 p, float& extra) {
    const float dx = p.x - r[R_C], dy = p.y - r[R_C + 1], dz = p.z - r[R_C + 2];
    const float mx = r[R_M], my = r[R_M + 1], mz = r[R_M + 2];
    const float h = __fmaf_rn(dz, mz, __fmaf_rn(dy, my, __fmul_rn(dx, mx)));
    const float ux = __fmaf_rn(-h, mx, dx), uy = __fmaf_rn(-h, my, dy), uz = __fmaf_rn(-h, mz, dz);
    const float u = sqrt_approx(__fmaf_rn(uz, uz, __fmaf_rn(uy, uy, __fmul_rn(ux, ux))));
    const float ah = fabsf(h);
    const float a = fmaxf(ah - r[R_W], 0.0f), b = fmaxf(u - r[R_R], 0.0f);
    extra = 0x1p-18f * (ah + u);
    return __fmaf_rn(b, b, __fmul_rn(a, a));
}

// True when the pair's computed |d| provably exceeds `cur` (the magnitude of the cell's word).
__device__ __forceinline__ bool provably_farther(const float* r, float3 p, float cur) {
    float extra;
    const float lb2 = lower_bound2(r, p, extra);
    const float thr = __fmaf_rn(cur, 1.0f + 0x1p-18f, r[R_S] + extra);
    return lb2 > __fmul_rn(__fmul_rn(thr, thr), 1.0f + 0x1p-16f);
}

// Ordering key of a record for a brick: distance from the brick's centre to the centroid, less R, in
// quarter cells (clamped to the buckets).  Only the order of evaluation depends on it.
__device__ __forceinline__ int record_bucket(const float* r, float3 bc, float invQuarter) {
    const float dx = bc.x - r[R_C], dy = bc.y - r[R_C + 1], dz = bc.z - r[R_C + 2];
    const float d = sqrt_approx(__fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)))) - r[R_R];
    const float q = d * invQuarter;
    return q <= 0.0f ? 0 : (q >= (float)(NBUCKET - 1) ? NBUCKET - 1 : (int)q);
}

__device__ __forceinline__ bool box_overlaps_brick(const float* r, int3 b0) {
    const int3 lo = unpack_cell(__float_as_int(r[R_LO])), hi = unpack_cell(__float_as_int(r[R_HI]));
    return lo.x <= b0.x + 3 && hi.x >= b0.x && lo.y <= b0.y + 3 && hi.y >= b0.y && lo.z <= b0.z + 1 && hi.z >= b0.z;
}

__device__ __forceinline__ int3 brick_cell(int3 b0, int l) { return make_int3(b0.x + (l & 3), b0.y + ((l >> 2) & 3), b0.z + (l >> 4)); }

// Queue entry: the reference's exact arithmetic for the pair, folded into the cell's word.
__device__ __forceinline__ void evaluate_entry(TileSmem& S, const SdfGrid& g, int3 b0, int warp, uint32_t e) {
    const int l = (int)(e & 31u), r = (int)(e >> 5);
    const float* x = &S.rec[r * RS + R_X];
    const TriPre T = tri_pre(mk3(x[0], x[1], x[2]), mk3(x[3], x[4], x[5]), mk3(x[6], x[7], x[8]));
    const int3 c = brick_cell(b0, l);
    atomicMin(&S.words[warp * 32 + l], float_flip3(signed_dist_pre(sdf_cell_pos(g, c.x, c.y, c.z), T)));
}

__global__ void __launch_bounds__(TILE_THREADS, 4) k_sdf_tiles(SdfTileLaunch L) {
    __shared__ TileSmem S;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t far = float_flip3(1e10f);
    const unsigned lanesBelow = (1u << lane) - 1u;
    for (;;) {
        if (tid == 0) S.tile = atomicAdd(L.workCounter, 1);
        __syncthreads();
        const int tile = S.tile;
        __syncthreads();
        if (tile >= L.totalTiles) break;
        const int si = sdf_of_tile(L.sdfs, L.nsdf, tile);
        const BatchSdf& s = L.sdfs[si];
        const SdfGrid g = s.frame->grid;
        const int lt = tile - s.firstTile;
        const int tx = lt % s.tilesX, ty = (lt / s.tilesX) % s.tilesY, tz = lt / (s.tilesX * s.tilesY);
        // this warp's brick and this lane's cell
        const int3 b0 = make_int3(tx * TX + (warp & 1) * 4, ty * TY + ((warp >> 1) & 1) * 4, tz * TZ + (warp >> 2) * 2);
        const int3 cc = brick_cell(b0, lane);
        const bool valid = cc.x < g.nx && cc.y < g.ny && cc.z < g.nz;
        float* out = reinterpret_cast<float*>(s.words);
        const long long cellIndex = ((long long)cc.z * g.ny + cc.y) * g.nx + cc.x;
        const int nList = L.tileCount[tile];        // the fill's cursor: the tile's list length
        const int listStart = tile_start(L, tile);
        const int nCand = nList + L.bigCount[si];

        if (nCand == 0) {   // no box reaches the tile: FloatFlip3(1e10) decodes to 1e10
            if (valid) out[cellIndex] = 1e10f;
            continue;
        }
        const float3 p = sdf_cell_pos(g, cc.x, cc.y, cc.z);
        const float3 bc = add(mk3(g.ox, g.oy, g.oz), mk3(((float)b0.x + 1.5f) * g.cell, ((float)b0.y + 1.5f) * g.cell,
                                                        ((float)b0.z + 0.5f) * g.cell));
        const float invQuarter = 4.0f / g.cell;
        float cur = 1e10f;                           // magnitude of this cell's word
        S.words[tid] = far;
        uint32_t* Q = S.queue[warp];
        uint16_t* list = S.list[warp];
        int* bucket = S.bucket[warp];

        for (int c0 = 0; c0 < nCand; c0 += CH) {
            const int cn = min(CH, nCand - c0);
            for (int k = tid; k < cn * REC; k += TILE_THREADS) {
                const int r = k / REC, w = k - r * REC;
                const int t = candidate_triangle(L, s, listStart, nList, c0 + r);
                S.rec[r * RS + w] = __ldg(L.records + (size_t)t * REC + w);
            }
            __syncthreads();

            // the chunk's records overlapping this brick, nearest first (counting sort by bucket)
            if (lane < NBUCKET) bucket[lane] = 0;
            __syncwarp();
            for (int r = lane; r < cn; r += 32) {
                const float* rec = &S.rec[r * RS];
                if (box_overlaps_brick(rec, b0)) atomicAdd(&bucket[record_bucket(rec, bc, invQuarter)], 1);
            }
            __syncwarp();
            int m = 0;
            {
                int v = lane < NBUCKET ? bucket[lane] : 0, x = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(FULL, x, o);
                    if (lane >= o) x += y;
                }
                m = __shfl_sync(FULL, x, 31);
                __syncwarp();
                if (lane < NBUCKET) bucket[lane] = x - v;
            }
            __syncwarp();
            for (int r = lane; r < cn; r += 32) {
                const float* rec = &S.rec[r * RS];
                if (box_overlaps_brick(rec, b0)) list[atomicAdd(&bucket[record_bucket(rec, bc, invQuarter)], 1)] = (uint16_t)r;
            }
            __syncwarp();

            // walk the list: queue the pairs the bound cannot exclude, evaluate them 32 at a time
            int qc = 0;
            for (int i = 0; i < m; ++i) {
                const int r = list[i];
                const float* rec = &S.rec[r * RS];
                const int3 lo = unpack_cell(__float_as_int(rec[R_LO])), hi = unpack_cell(__float_as_int(rec[R_HI]));
                const bool inside = valid && cc.x >= lo.x && cc.x <= hi.x && cc.y >= lo.y && cc.y <= hi.y && cc.z >= lo.z &&
                                    cc.z <= hi.z;
                const bool want = inside && !provably_farther(rec, p, cur);
                const unsigned bal = __ballot_sync(FULL, want);
                if (want) Q[qc + __popc(bal & lanesBelow)] = (uint32_t)lane | ((uint32_t)r << 5);
                qc += __popc(bal);
                if (qc >= 32) {
                    __syncwarp();
                    evaluate_entry(S, g, b0, warp, Q[qc - 32 + lane]);
                    qc -= 32;
                    __syncwarp();
                    cur = fabsf(__uint_as_float(ifloat_flip3(S.words[tid])));
                }
            }
            __syncwarp();
            if (lane < qc) evaluate_entry(S, g, b0, warp, Q[lane]);
            __syncwarp();
            cur = fabsf(__uint_as_float(ifloat_flip3(S.words[tid])));
            __syncthreads();   // the next chunk overwrites the records
        }

        // FinalizeSignedDistanceField: the decoded float of this lane's cell
        if (valid) out[cellIndex] = __uint_as_float(ifloat_flip3(S.words[tid]));
        __syncthreads();
    }
}

}  // namespace

int sdf_tile_blocks_per_sm() {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_sdf_tiles, TILE_THREADS, 0) != cudaSuccess) return 1;
    return nb > 0 ? nb : 1;
}

cudaError_t launch_sdf_tiles(const SdfTileLaunch& L, cudaStream_t s) {
    if (L.nsdf <= 0 || L.totalTiles <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(L.tileCount, 0, L.zeroBytes, s);   // tile counts, big counts, work counter
    if (e != cudaSuccess) return e;
    const int sms = sm_count();
    if (L.totalTris > 0) {
        const unsigned gt = (unsigned)std::min((L.totalTris + 255) / 256, sms * 8);
        k_sdf_bin_count<<<gt, 256, 0, s>>>(L);
        const int nb = (L.totalTiles + SCAN_BLOCK - 1) / SCAN_BLOCK;
        k_sdf_bin_scan_local<<<nb, SCAN_BLOCK, 0, s>>>(L);
        k_sdf_bin_scan_top<<<1, SCAN_BLOCK, 0, s>>>(L.blockSum, nb);
        k_sdf_bin_fill<<<gt, 256, 0, s>>>(L);
    }
    k_sdf_tiles<<<(unsigned)std::max(1, std::min(L.blocks, L.totalTiles)), TILE_THREADS, 0, s>>>(L);
    return cudaGetLastError();
}

}  // namespace tfx
