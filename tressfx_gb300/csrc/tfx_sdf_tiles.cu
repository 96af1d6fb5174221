// The batched SDF build as a tile-binned construct with exact pair culling.
//
// InitializeSignedDistanceField + ConstructSignedDistanceField + FinalizeSignedDistanceField
// (TressFXSDFCollision.hlsl:301-412) give every cell the minimum, over the triangles whose cell box
// (:351-363) contains the cell, of FloatFlip3(SignedDistancePointToTriangle(cell corner, triangle)),
// and FloatFlip3(1e10) where no box reaches.  The reference evaluates every (triangle, cell) pair of
// every box and resolves the minimum with an atomicMin per pair in device memory.  Here:
//
//  1. k_sdf_bin_count / k_sdf_bin_scan_* / k_sdf_bin_fill bin each triangle into the 8x8x8-cell tiles
//     its box overlaps (a triangle whose box spans more than BIG_TILES tiles goes to its SDF's big list,
//     which every tile of the SDF scans), so that each tile knows its candidate triangles.
//  2. k_sdf_tiles gives each tile to one block, which keeps the tile's 512 FloatFlip3 words in shared
//     memory.  Pass A seeds every cell with the candidate of smallest lower bound and evaluates that pair
//     exactly; pass B visits the remaining pairs of the tile and evaluates a pair only when a lower bound
//     on its distance does not prove it larger than the cell's current word; the survivors are queued
//     per warp and evaluated 32 at a time.  The block then writes the decoded floats of its cells (the
//     finalized grid): no separate initialise or finalise pass, no atomic in device memory per pair.
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

constexpr int TILE = 8;                            // cells per tile edge
constexpr int TILE_CELLS = TILE * TILE * TILE;     // 512
constexpr int TILE_THREADS = 256;
constexpr int TILE_WARPS = TILE_THREADS / 32;
constexpr int CHUNK = 64;                          // triangle records in shared memory at a time
constexpr int REC = 45;                            // words per record; odd, so 32 lanes reading 32 records do not conflict
constexpr int QCAP = 64;                           // queue entries per warp
constexpr int SCAN_BLOCK = 1024;
constexpr unsigned FULL = 0xffffffffu;

// record layout (words)
constexpr int R_TRI = 0;       // TriPre: 33 floats (x0 x1 x2 x02n x12n l0 l1 l2 nTri e01 e12 e02 d01 d12 d02)
constexpr int R_C = 33;        // centroid
constexpr int R_M = 36;        // unit normal, or 0
constexpr int R_R = 39;        // max |x_i - c|
constexpr int R_W = 40;        // max |<x_i - c, m>|
constexpr int R_S = 41;        // absolute slack
constexpr int R_LO = 42;       // packed cell box
constexpr int R_HI = 43;
constexpr int R_CAND = 44;     // candidate index within the tile

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

__device__ __forceinline__ void tri_vertices(const BatchSdf& s, int tri, float3& x0, float3& x1, float3& x2) {
    x0 = xyz(__ldg(s.mesh + 2 * (size_t)__ldg(s.indices + 3 * tri + 0)));
    x1 = xyz(__ldg(s.mesh + 2 * (size_t)__ldg(s.indices + 3 * tri + 1)));
    x2 = xyz(__ldg(s.mesh + 2 * (size_t)__ldg(s.indices + 3 * tri + 2)));
}

// The tiles of SDF s that the packed cell box [lo, hi] overlaps.
__device__ __forceinline__ void box_tiles(int lo, int hi, int3& a, int3& b) {
    const int3 l = unpack_cell(lo), h = unpack_cell(hi);
    a = make_int3(l.x / TILE, l.y / TILE, l.z / TILE);
    b = make_int3(h.x / TILE, h.y / TILE, h.z / TILE);
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
__global__ void __launch_bounds__(256) k_sdf_bin_count(SdfTileLaunch L) {
    const int stride = gridDim.x * blockDim.x;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < L.totalTris; t += stride) {
        const int si = sdf_of_triangle(L.sdfs, L.nsdf, t);
        const BatchSdf& s = L.sdfs[si];
        const SdfGrid g = s.frame->grid;
        float3 x0, x1, x2;
        tri_vertices(s, t - s.firstTriangle, x0, x1, x2);
        int3 lo, hi;
        tri_cell_box(g, x0, x1, x2, lo, hi);   // the reference's clamped box: never empty
        const int plo = pack_cell(lo), phi = pack_cell(hi);
        L.triBox[t] = make_int2(plo, phi);
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
        const int2 box = L.triBox[t];
        int3 a, b;
        box_tiles(box.x, box.y, a, b);
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
    uint32_t words[TILE_CELLS];            // FloatFlip3 words of the tile's cells
    unsigned long long seed[TILE_CELLS];   // (lower bound bits << 32) | candidate, min over the candidates
    float rec[CHUNK * REC];                // triangle records of the current chunk
    uint32_t queue[TILE_WARPS][QCAP];      // per warp: pairs to evaluate, cell | record << 9
    int tile;
};

// The record of candidate `cand` into rec: the reference's per-triangle terms and the bound's terms.
__device__ void make_record(const SdfTileLaunch& L, const BatchSdf& s, int listStart, int nList, int cand, float* rec) {
    const int t = candidate_triangle(L, s, listStart, nList, cand);
    float3 x0, x1, x2;
    tri_vertices(s, t - s.firstTriangle, x0, x1, x2);
    const TriPre T = tri_pre(x0, x1, x2);
    const float v[33] = {T.x0.x, T.x0.y, T.x0.z, T.x1.x, T.x1.y, T.x1.z, T.x2.x, T.x2.y, T.x2.z,
                         T.x02n.x, T.x02n.y, T.x02n.z, T.x12n.x, T.x12n.y, T.x12n.z, T.l0, T.l1, T.l2,
                         T.nTri.x, T.nTri.y, T.nTri.z, T.e01.x, T.e01.y, T.e01.z, T.e12.x, T.e12.y, T.e12.z,
                         T.e02.x, T.e02.y, T.e02.z, T.d01, T.d12, T.d02};
#pragma unroll
    for (int k = 0; k < 33; ++k) rec[R_TRI + k] = v[k];
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
    rec[R_C + 0] = c.x; rec[R_C + 1] = c.y; rec[R_C + 2] = c.z;
    rec[R_M + 0] = m.x; rec[R_M + 1] = m.y; rec[R_M + 2] = m.z;
    rec[R_R] = R;
    rec[R_W] = w;
    rec[R_S] = 0x1p-18f * ((Mt + R) + w) + 2e-7f * R;
    const int2 box = L.triBox[t];
    rec[R_LO] = __int_as_float(box.x);
    rec[R_HI] = __int_as_float(box.y);
    rec[R_CAND] = __int_as_float(cand);
}

__device__ __forceinline__ TriPre record_tri(const float* r) {
    TriPre T;
    T.x0 = mk3(r[0], r[1], r[2]); T.x1 = mk3(r[3], r[4], r[5]); T.x2 = mk3(r[6], r[7], r[8]);
    T.x02n = mk3(r[9], r[10], r[11]); T.x12n = mk3(r[12], r[13], r[14]);
    T.l0 = r[15]; T.l1 = r[16]; T.l2 = r[17];
    T.nTri = mk3(r[18], r[19], r[20]);
    T.e01 = mk3(r[21], r[22], r[23]); T.e12 = mk3(r[24], r[25], r[26]); T.e02 = mk3(r[27], r[28], r[29]);
    T.d01 = r[30]; T.d12 = r[31]; T.d02 = r[32];
    return T;
}

// Bound terms of one record, in registers for a warp's sweep over its cells.
struct Bound {
    float cx, cy, cz, mx, my, mz, R, w, S;
};
__device__ __forceinline__ Bound record_bound(const float* r) {
    return Bound{r[R_C], r[R_C + 1], r[R_C + 2], r[R_M], r[R_M + 1], r[R_M + 2], r[R_R], r[R_W], r[R_S]};
}

// Squared lower bound on the distance from p to the triangle, and in `extra` the per-pair slack
// 2^-18 (|h| + |u|).
__device__ __forceinline__ float lower_bound2(const Bound& B, float3 p, float& extra) {
    const float dx = p.x - B.cx, dy = p.y - B.cy, dz = p.z - B.cz;
    const float h = __fmaf_rn(dz, B.mz, __fmaf_rn(dy, B.my, __fmul_rn(dx, B.mx)));
    const float ux = __fmaf_rn(-h, B.mx, dx), uy = __fmaf_rn(-h, B.my, dy), uz = __fmaf_rn(-h, B.mz, dz);
    const float u = sqrt_approx(__fmaf_rn(uz, uz, __fmaf_rn(uy, uy, __fmul_rn(ux, ux))));
    const float ah = fabsf(h);
    const float a = fmaxf(ah - B.w, 0.0f), b = fmaxf(u - B.R, 0.0f);
    extra = 0x1p-18f * (ah + u);
    return __fmaf_rn(b, b, __fmul_rn(a, a));
}

// True when the pair's computed |d| provably exceeds `cur` (the magnitude of the cell's word).
__device__ __forceinline__ bool provably_farther(const Bound& B, float3 p, float cur) {
    float extra;
    const float lb2 = lower_bound2(B, p, extra);
    const float thr = __fmaf_rn(cur, 1.0f + 0x1p-18f, B.S + extra);
    return lb2 > __fmul_rn(__fmul_rn(thr, thr), 1.0f + 0x1p-16f);
}

// The cells of a record's box inside the tile [t0, t0 + 8)^3: first cell and extents (0 when empty).
struct BoxInTile {
    int3 lo;
    int ex, ey, vol;
    float inxy, inx;
};
__device__ __forceinline__ BoxInTile box_in_tile(const float* r, int3 t0) {
    const int3 l = unpack_cell(__float_as_int(r[R_LO])), h = unpack_cell(__float_as_int(r[R_HI]));
    BoxInTile b;
    b.lo = make_int3(max(l.x, t0.x), max(l.y, t0.y), max(l.z, t0.z));
    const int3 hi = make_int3(min(h.x, t0.x + TILE - 1), min(h.y, t0.y + TILE - 1), min(h.z, t0.z + TILE - 1));
    b.ex = hi.x - b.lo.x + 1;
    b.ey = hi.y - b.lo.y + 1;
    const int ez = hi.z - b.lo.z + 1;
    b.vol = (b.ex > 0 && b.ey > 0 && ez > 0) ? b.ex * b.ey * ez : 0;
    b.inxy = b.vol ? 1.0f / (float)(b.ex * b.ey) : 0.0f;
    b.inx = b.vol ? 1.0f / (float)b.ex : 0.0f;
    return b;
}
// Cell c (< vol <= 512) of the box: global coordinates.  (c + 0.5) / m truncates to the integer quotient
// for c < 2^22 (see sdf_construct_triangle_warp).
__device__ __forceinline__ int3 box_cell(const BoxInTile& b, int c) {
    const int cz = (int)(((float)c + 0.5f) * b.inxy);
    const int r = c - cz * b.ex * b.ey;
    const int cy = (int)(((float)r + 0.5f) * b.inx);
    return make_int3(b.lo.x + (r - cy * b.ex), b.lo.y + cy, b.lo.z + cz);
}
__device__ __forceinline__ int local_cell(int3 x, int3 t0) {
    return ((x.z - t0.z) * TILE + (x.y - t0.y)) * TILE + (x.x - t0.x);
}

// Queue entry: evaluate the pair exactly (the reference's arithmetic) and fold it into the word.
__device__ __forceinline__ void evaluate_entry(TileSmem& S, const SdfGrid& g, int3 t0, uint32_t e) {
    const int cl = (int)(e & 511u), r = (int)(e >> 9);
    const TriPre T = record_tri(&S.rec[r * REC]);
    const int x = t0.x + (cl & 7), y = t0.y + ((cl >> 3) & 7), z = t0.z + (cl >> 6);
    atomicMin(&S.words[cl], float_flip3(signed_dist_pre(sdf_cell_pos(g, x, y, z), T)));
}

__global__ void __launch_bounds__(TILE_THREADS) k_sdf_tiles(SdfTileLaunch L) {
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
        const int3 t0 = make_int3(tx * TILE, ty * TILE, tz * TILE);
        const int nList = L.tileCount[tile];        // the fill's cursor: the tile's list length
        const int listStart = tile_start(L, tile);
        const int nCand = nList + L.bigCount[si];
        float* out = reinterpret_cast<float*>(s.words);
        const long long nxy = (long long)g.nx * g.ny;

        if (nCand == 0) {   // no box reaches the tile: FloatFlip3(1e10) decodes to 1e10
            for (int cl = tid; cl < TILE_CELLS; cl += TILE_THREADS) {
                const int x = t0.x + (cl & 7), y = t0.y + ((cl >> 3) & 7), z = t0.z + (cl >> 6);
                if (x < g.nx && y < g.ny && z < g.nz) out[z * nxy + (long long)y * g.nx + x] = 1e10f;
            }
            continue;
        }
        for (int cl = tid; cl < TILE_CELLS; cl += TILE_THREADS) {
            S.words[cl] = far;
            S.seed[cl] = ~0ull;
        }
        __syncthreads();

        // ---- pass A: per cell, the candidate of smallest lower bound
        for (int c0 = 0; c0 < nCand; c0 += CHUNK) {
            const int cn = min(CHUNK, nCand - c0);
            if (tid < cn) make_record(L, s, listStart, nList, c0 + tid, &S.rec[tid * REC]);
            __syncthreads();
            for (int r = warp; r < cn; r += TILE_WARPS) {
                const float* rec = &S.rec[r * REC];
                const BoxInTile b = box_in_tile(rec, t0);
                const Bound B = record_bound(rec);
                for (int base = 0; base < b.vol; base += 32) {
                    const int c = base + lane;
                    if (c < b.vol) {
                        const int3 x = box_cell(b, c);
                        float extra;
                        const float lb2 = lower_bound2(B, sdf_cell_pos(g, x.x, x.y, x.z), extra);
                        const unsigned long long key =
                            ((unsigned long long)__float_as_uint(lb2) << 32) | (unsigned)(c0 + r);
                        atomicMin(&S.seed[local_cell(x, t0)], key);
                    }
                }
            }
            __syncthreads();
        }
        // ---- the seeds, exactly
        for (int cl = tid; cl < TILE_CELLS; cl += TILE_THREADS) {
            const unsigned long long key = S.seed[cl];
            if (key == ~0ull) continue;
            const int t = candidate_triangle(L, s, listStart, nList, (int)(unsigned)key);
            float3 x0, x1, x2;
            tri_vertices(s, t - s.firstTriangle, x0, x1, x2);
            const int x = t0.x + (cl & 7), y = t0.y + ((cl >> 3) & 7), z = t0.z + (cl >> 6);
            S.words[cl] = float_flip3(signed_dist_pre(sdf_cell_pos(g, x, y, z), tri_pre(x0, x1, x2)));
        }
        __syncthreads();

        // ---- pass B: every other pair that the bound cannot exclude
        uint32_t* Q = S.queue[warp];
        for (int c0 = 0; c0 < nCand; c0 += CHUNK) {
            const int cn = min(CHUNK, nCand - c0);
            if (tid < cn) make_record(L, s, listStart, nList, c0 + tid, &S.rec[tid * REC]);
            __syncthreads();
            int qc = 0;
            for (int r = warp; r < cn; r += TILE_WARPS) {
                const float* rec = &S.rec[r * REC];
                const BoxInTile b = box_in_tile(rec, t0);
                const Bound B = record_bound(rec);
                const unsigned cand = (unsigned)(c0 + r);
                for (int base = 0; base < b.vol; base += 32) {
                    const int c = base + lane;
                    bool want = false;
                    int cl = 0;
                    if (c < b.vol) {
                        const int3 x = box_cell(b, c);
                        cl = local_cell(x, t0);
                        if ((unsigned)S.seed[cl] != cand) {
                            const float cur = __uint_as_float(S.words[cl] >> 1);
                            want = !provably_farther(B, sdf_cell_pos(g, x.x, x.y, x.z), cur);
                        }
                    }
                    const unsigned m = __ballot_sync(FULL, want);
                    if (want) Q[qc + __popc(m & lanesBelow)] = (uint32_t)cl | ((uint32_t)r << 9);
                    qc += __popc(m);
                    if (qc >= 32) {
                        __syncwarp();
                        evaluate_entry(S, g, t0, Q[qc - 32 + lane]);
                        qc -= 32;
                        __syncwarp();
                    }
                }
            }
            __syncwarp();
            if (lane < qc) evaluate_entry(S, g, t0, Q[lane]);
            __syncthreads();
        }

        // ---- FinalizeSignedDistanceField: the decoded floats of the tile's cells
        for (int cl = tid; cl < TILE_CELLS; cl += TILE_THREADS) {
            const int x = t0.x + (cl & 7), y = t0.y + ((cl >> 3) & 7), z = t0.z + (cl >> 6);
            if (x < g.nx && y < g.ny && z < g.nz)
                out[z * nxy + (long long)y * g.nx + x] = __uint_as_float(ifloat_flip3(S.words[cl]));
        }
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
