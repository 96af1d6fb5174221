// Iso-surface extraction of a signed distance grid (TressFXSDFMarchingCubes, src/TressFX/
// TressFXSDFMarchingCubes.cpp:27-233, and RunMarchingCubesOnSdf, src/Shaders/TressFXMarchingCubes.hlsl:
// 147-280), headless: the triangle soup lands in a device vertex buffer.
//
// The reference appends each cube's triangles at an atomically reserved offset, so its vertex order
// changes from run to run.  Here the offsets are an exclusive prefix sum of the cubes' vertex counts
// in cell-index order -- the order a one-thread-at-a-time dispatch of the shader produces -- so the
// buffer is deterministic and bit-comparable.  Three launches:
//   k_mc_count: one cell per thread, the vertex count every block of 256 cells reserves;
//   k_mc_scan:  one block, the exclusive prefix of those counts (64-bit) and the total (the shader's
//               counter, which also counts cubes that did not fit);
//   k_mc_write: each block rescans its cells in shared memory and spreads its triangles over its
//               threads, one triangle per thread; a cube is written only if its range ends below
//               max_vertices (the shader's `offset + num < max`), and whatever InitializeMCVertices
//               would leave zero is zeroed.
// The grid (a few MB) stays in L2 between the passes.
#include <cstring>
#include <new>

#include "tfx_handles.h"

namespace tfx {

// The shader's two lookup tables (MARCHING_CUBES_EDGE_TABLE / _TRIANGLE_TABLE layout) and, per cube
// configuration, the vertex count the shader reserves: 0 where the edge table entry is 0, else the
// triangle-table entries before the first -1.
struct McTables {
    int32_t edge[256];
    int32_t tri[256 * 16];
    int32_t count[256];
};

namespace {

constexpr int kMcThreads = 256;       // cells of a block, one per thread
constexpr int kMcScanThreads = 1024;

// Corner k of a cube sits at cell + kCorner[k] (TressFXMarchingCubes.hlsl:165-173); edge e joins the
// corners kEdgeA[e] -> kEdgeB[e], in the argument order of its VertexLerp call (:211-222).
__constant__ int8_t kCornerX[8] = {0, 1, 1, 0, 0, 1, 1, 0};
__constant__ int8_t kCornerY[8] = {0, 0, 0, 0, 1, 1, 1, 1};
__constant__ int8_t kCornerZ[8] = {0, 0, 1, 1, 0, 0, 1, 1};
__constant__ int8_t kEdgeA[12] = {0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 2, 3};
__constant__ int8_t kEdgeB[12] = {1, 2, 3, 0, 5, 6, 7, 4, 4, 5, 6, 7};

// Division of 32-bit unsigned n by an invariant d >= 1 with a multiply-high (Granlund and
// Montgomery, "Division by invariant integers using multiplication", 1994, figure 4.1):
// l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1, q = (umulhi(n, m) + n) >> l, the sum taken in
// 64 bits.  Exact for every n < 2^32.
struct FastDiv {
    uint32_t d, m, l;
};

__host__ FastDiv fast_div(uint32_t d) {
    uint32_t l = 0;
    while (l < 32 && (1ull << l) < d) ++l;
    const uint64_t m = (((1ull << l) - d) << 32) / d + 1;
    return FastDiv{d, (uint32_t)m, l};
}

__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
    return (uint32_t)(((uint64_t)__umulhi(n, f.m) + n) >> f.l);
}

// The grid's two divisors: cells per line (X) and per plane (X * Y).
struct McDims {
    FastDiv line, plane;
};

// The cell of linear index `index` (x fastest), as GetSdfCellPositionFromIndex computes it.
__device__ __forceinline__ int3 mc_cell_xyz(const McDims& dm, int index) {
    const uint32_t u = (uint32_t)index;
    const uint32_t z = fdiv(u, dm.plane);
    const uint32_t rem = u - z * dm.plane.d;
    const uint32_t y = fdiv(rem, dm.line);
    return make_int3((int)(rem - y * dm.line.d), (int)y, (int)z);
}

// The eight corner values of cube `c` and its cubeIndex; -1 for cells on the upper faces of the grid.
__device__ __forceinline__ int mc_config(const float* __restrict__ sdf, const SdfGrid& g, int3 c, float iso, float s[8]) {
    if (c.x >= g.nx - 1 || c.y >= g.ny - 1 || c.z >= g.nz - 1) return -1;
    const int plane = g.nx * g.ny;
    const float* p = sdf + (plane * c.z + g.nx * c.y + c.x);
    // corners 0..7: (0,0,0) (1,0,0) (1,0,1) (0,0,1) (0,1,0) (1,1,0) (1,1,1) (0,1,1)
    s[0] = __ldg(p);
    s[1] = __ldg(p + 1);
    s[2] = __ldg(p + plane + 1);
    s[3] = __ldg(p + plane);
    s[4] = __ldg(p + g.nx);
    s[5] = __ldg(p + g.nx + 1);
    s[6] = __ldg(p + plane + g.nx + 1);
    s[7] = __ldg(p + plane + g.nx);
    int cfg = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (s[k] < iso) cfg |= 1 << k;
    return cfg;
}

// GetSdfCellPosition of corner k: float3(cell + offset) * cellSize, then + origin.
__device__ __forceinline__ float3 mc_corner(int3 c, const SdfGrid& g, int k) {
    const float3 p = make_float3((float)(c.x + kCornerX[k]) * g.cell, (float)(c.y + kCornerY[k]) * g.cell,
                                 (float)(c.z + kCornerZ[k]) * g.cell);
    return make_float3(p.x + g.ox, p.y + g.oy, p.z + g.oz);
}

// VertexLerp on edge e: p1 + (p2 - p1) * ((iso - s1) / (s2 - s1)); s = the cube's corner values.
__device__ __forceinline__ float3 mc_edge_vertex(int3 c, const SdfGrid& g, const float* s, int e, float iso) {
    const int a = kEdgeA[e], b = kEdgeB[e];
    const float sa = s[a * kMcThreads], sb = s[b * kMcThreads];
    const float interp = (iso - sa) / (sb - sa);
    const float3 p1 = mc_corner(c, g, a), p2 = mc_corner(c, g, b);
    return make_float3(p1.x + (p2.x - p1.x) * interp, p1.y + (p2.y - p1.y) * interp, p1.z + (p2.z - p1.z) * interp);
}

// Exclusive scan of one value per thread over a block of NT threads; *total receives the sum.
template <int NT, class T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* red, T* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T n = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += n;
    }
    __syncthreads();
    if (lane == 31) red[warp] = incl;
    __syncthreads();
    T before = 0, all = 0;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) {
        const T t = red[w];
        before += (w < warp) ? t : (T)0;
        all += t;
    }
    *total = all;
    return before + incl - v;
}

// Pass 1: the vertices every block of 256 cells reserves.
__global__ void __launch_bounds__(kMcThreads) k_mc_count(const float* __restrict__ sdf, SdfGrid g, McDims dm,
                                                         float iso, const McTables* __restrict__ T, int totalCells,
                                                         int* __restrict__ blockSums) {
    __shared__ int cnt[256];
    __shared__ int red[kMcThreads / 32];
    cnt[threadIdx.x] = T->count[threadIdx.x];
    __syncthreads();
    const int idx = blockIdx.x * kMcThreads + (int)threadIdx.x;
    int nv = 0;
    if (idx < totalCells) {
        float s[8];
        const int cfg = mc_config(sdf, g, mc_cell_xyz(dm, idx), iso, s);
        nv = cfg >= 0 ? cnt[cfg] : 0;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) nv += __shfl_xor_sync(0xffffffffu, nv, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = nv;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
#pragma unroll
        for (int w = 0; w < kMcThreads / 32; ++w) t += red[w];
        blockSums[blockIdx.x] = t;
    }
}

// Pass 2 (one block): exclusive prefix of the block sums in 64 bits; blockOff[nb] = the total, and
// the counter (an int, as in the shader) its low 32 bits.  Each thread takes 8 consecutive sums of a
// 8192-sum tile (all loads in flight at once), scans them serially, and the block scans the thread
// totals.
constexpr int kMcScanPer = 8;
__global__ void __launch_bounds__(kMcScanThreads) k_mc_scan(const int* __restrict__ blockSums, int nb,
                                                            long long* __restrict__ blockOff, int* __restrict__ counter) {
    __shared__ long long red[kMcScanThreads / 32];
    long long carry = 0;
    for (int base = 0; base < nb; base += kMcScanThreads * kMcScanPer) {
        const int b0 = base + (int)threadIdx.x * kMcScanPer;
        int v[kMcScanPer];
#pragma unroll
        for (int k = 0; k < kMcScanPer; ++k) v[k] = b0 + k < nb ? __ldg(blockSums + b0 + k) : 0;
        long long mine = 0;
#pragma unroll
        for (int k = 0; k < kMcScanPer; ++k) mine += v[k];
        long long total;
        long long run = carry + block_exclusive_scan<kMcScanThreads>(mine, red, &total);
#pragma unroll
        for (int k = 0; k < kMcScanPer; ++k) {
            if (b0 + k < nb) blockOff[b0 + k] = run;
            run += v[k];
        }
        carry += total;
    }
    if (threadIdx.x == 0) {
        blockOff[nb] = carry;
        *counter = (int)carry;
    }
}

__device__ __forceinline__ void mc_zero(float4* out, long long v) {
    out[2 * v] = make_float4(0.f, 0.f, 0.f, 0.f);
    out[2 * v + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Pass 3: the block's cells are scanned in shared memory (vertex and triangle counts packed in one
// int), each cell's thread zeroes what of its range will not be written (a cube that does not end
// below maxVerts, or the vertices past a count that is not a multiple of 3), then the block's
// triangles are spread over its threads, one triangle (three 32-byte vertices) per thread.  Vertices
// [total, maxVerts) are zeroed by all blocks together.
__global__ void __launch_bounds__(kMcThreads) k_mc_write(const float* __restrict__ sdf, SdfGrid g, McDims dm,
                                                         float iso, const McTables* __restrict__ T, int totalCells,
                                                         const int* __restrict__ blockSums,
                                                         const long long* __restrict__ blockOff, int nb, int maxVerts,
                                                         float4* __restrict__ out) {
    __shared__ float cs[8 * kMcThreads];      // corner values, [corner][cell]
    __shared__ int ccfg[kMcThreads];          // cubeIndex of a cube whose triangles are written, else -1
    __shared__ int cex[kMcThreads + 1];       // exclusive prefix: vertices in the low 16 bits, triangles above
    __shared__ int red[kMcThreads / 32];
    const long long total = __ldg(blockOff + nb);
    for (long long v = total + (long long)blockIdx.x * kMcThreads + threadIdx.x; v < maxVerts;
         v += (long long)gridDim.x * kMcThreads)
        mc_zero(out, v);
    const int mine = __ldg(blockSums + blockIdx.x);
    const long long off = __ldg(blockOff + blockIdx.x);
    if (mine == 0 || off >= maxVerts) return;
    const int cell0 = blockIdx.x * kMcThreads;
    const int idx = cell0 + (int)threadIdx.x;
    int nv = 0, cfg = -1;
    if (idx < totalCells) {
        float s[8];
        cfg = mc_config(sdf, g, mc_cell_xyz(dm, idx), iso, s);
        if (cfg >= 0) {
            nv = __ldg(T->count + cfg);
#pragma unroll
            for (int k = 0; k < 8; ++k) cs[k * kMcThreads + threadIdx.x] = s[k];
        }
    }
    const int ntri = nv / 3;
    int sum;
    const int ex = block_exclusive_scan<kMcThreads>(nv | (ntri << 16), red, &sum);
    cex[threadIdx.x] = ex;
    if (threadIdx.x == 0) cex[kMcThreads] = sum;
    const long long cellOff = off + (ex & 0xffff);
    const bool fits = nv > 0 && cellOff + nv < maxVerts;
    ccfg[threadIdx.x] = fits ? cfg : -1;
    if (nv > 0) {
        for (int k = fits ? 3 * ntri : 0; k < nv && cellOff + k < maxVerts; ++k) mc_zero(out, cellOff + k);
    }
    __syncthreads();
    const int mineT = sum >> 16;
    for (int k = threadIdx.x; k < mineT; k += kMcThreads) {
        // the cube holding triangle k: the last c with a triangle prefix <= k
        int lo = 0, hi = kMcThreads - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if ((cex[mid] >> 16) <= k) lo = mid; else hi = mid - 1;
        }
        const int c = lo;
        const int cf = ccfg[c];
        if (cf < 0) continue;
        const int t = k - (cex[c] >> 16);
        const int3 xyz = mc_cell_xyz(dm, cell0 + c);
        const int* tri = T->tri + 16 * cf + 3 * t;
        const float* cv = cs + c;
        const float3 v0 = mc_edge_vertex(xyz, g, cv, __ldg(tri), iso);
        const float3 v1 = mc_edge_vertex(xyz, g, cv, __ldg(tri + 1), iso);
        const float3 v2 = mc_edge_vertex(xyz, g, cv, __ldg(tri + 2), iso);
        // normalize(cross(v1 - v0, v2 - v0)) = n * (1 / sqrt(dot(n, n)))
        const float3 a = make_float3(v1.x - v0.x, v1.y - v0.y, v1.z - v0.z);
        const float3 b = make_float3(v2.x - v0.x, v2.y - v0.y, v2.z - v0.z);
        const float3 nn = make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
        const float inv = 1.0f / sqrtf(nn.x * nn.x + nn.y * nn.y + nn.z * nn.z);
        const float4 n4 = make_float4(nn.x * inv, nn.y * inv, nn.z * inv, 0.f);
        float4* o = out + 2 * (off + (cex[c] & 0xffff) + 3 * t);
        o[0] = make_float4(v0.x, v0.y, v0.z, 0.f);
        o[1] = n4;
        o[2] = make_float4(v1.x, v1.y, v1.z, 0.f);
        o[3] = n4;
        o[4] = make_float4(v2.x, v2.y, v2.z, 0.f);
        o[5] = n4;
    }
}

}  // namespace

int mc_num_blocks(long long cells) { return (int)((cells + kMcThreads - 1) / kMcThreads); }
size_t mc_scratch_bytes(long long cells) {
    const size_t nb = (size_t)mc_num_blocks(cells);
    return ((nb * sizeof(int) + 15) & ~(size_t)15) + (nb + 1) * sizeof(long long);
}

cudaError_t launch_marching_cubes(const float* sdf, const SdfGrid& g, float iso, const McTables* tables, int maxVerts,
                                  void* scratch, float4* out, int* counter, cudaStream_t s) {
    const long long cells = (long long)g.nx * g.ny * g.nz;
    const int nb = mc_num_blocks(cells);
    int* blockSums = (int*)scratch;
    long long* blockOff = (long long*)((char*)scratch + (((size_t)nb * sizeof(int) + 15) & ~(size_t)15));
    const McDims dm{fast_div((uint32_t)g.nx), fast_div((uint32_t)g.nx * (uint32_t)g.ny)};
    k_mc_count<<<nb, kMcThreads, 0, s>>>(sdf, g, dm, iso, tables, (int)cells, blockSums);
    k_mc_scan<<<1, kMcScanThreads, 0, s>>>(blockSums, nb, blockOff, counter);
    k_mc_write<<<nb, kMcThreads, 0, s>>>(sdf, g, dm, iso, tables, (int)cells, blockSums, blockOff, nb, maxVerts, out);
    return cudaGetLastError();
}

// The product's triangle table, derived from the cube's faces.  Walking each face's corners in the
// order that runs counter-clockwise seen from outside the cube, a crossing edge where the walk
// enters the inside (value < iso) is joined to the next crossing where it leaves; on a face with
// four crossings this keeps the two inside corners apart, and since the rule reads only the face's
// own corners, the two cubes sharing a face draw the same segments there (the surface is closed
// across cubes).  The joined segments chain into loops through the shared edges; each loop is fanned
// from its first crossing.  Triangles come out wound so that cross(v1 - v0, v2 - v0) points away
// from the inside.
void mc_default_tables(int32_t edge[256], int32_t tri[256 * 16]) {
    static const int ea[12] = {0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 2, 3}, eb[12] = {1, 2, 3, 0, 5, 6, 7, 4, 4, 5, 6, 7};
    // faces as corner cycles, counter-clockwise seen from outside: y=0, y=1, z=0, z=1, x=0, x=1
    static const int face[6][4] = {{0, 1, 2, 3}, {4, 7, 6, 5}, {0, 4, 5, 1}, {3, 2, 6, 7}, {0, 3, 7, 4}, {1, 5, 6, 2}};
    auto edge_of = [&](int a, int b) {
        for (int e = 0; e < 12; ++e)
            if ((ea[e] == a && eb[e] == b) || (ea[e] == b && eb[e] == a)) return e;
        return -1;
    };
    for (int cfg = 0; cfg < 256; ++cfg) {
        bool in[8];
        for (int k = 0; k < 8; ++k) in[k] = (cfg >> k) & 1;
        int mask = 0;
        for (int e = 0; e < 12; ++e)
            if (in[ea[e]] != in[eb[e]]) mask |= 1 << e;
        edge[cfg] = mask;
        int next[12];
        for (int e = 0; e < 12; ++e) next[e] = -1;
        for (int f = 0; f < 6; ++f) {
            int ce[4], kind[4], m = 0;
            for (int k = 0; k < 4; ++k) {
                const int a = face[f][k], b = face[f][(k + 1) & 3];
                if (in[a] != in[b]) {
                    ce[m] = edge_of(a, b);
                    kind[m] = in[b] ? 1 : -1;
                    ++m;
                }
            }
            for (int i = 0; i < m; ++i) {
                if (kind[i] != 1) continue;
                int j = (i + 1) % m;
                while (kind[j] != -1) j = (j + 1) % m;
                next[ce[i]] = ce[j];
            }
        }
        int* t = tri + 16 * cfg;
        for (int i = 0; i < 16; ++i) t[i] = -1;
        bool seen[12] = {};
        int w = 0;
        for (int e0 = 0; e0 < 12; ++e0) {
            if (next[e0] < 0 || seen[e0]) continue;
            int loop[12], len = 0;
            for (int e = e0; !seen[e]; e = next[e]) {
                seen[e] = true;
                loop[len++] = e;
            }
            for (int i = 1; i + 1 < len; ++i) {
                t[w++] = loop[0];
                t[w++] = loop[i];
                t[w++] = loop[i + 1];
            }
        }
    }
}

}  // namespace tfx

// ============================================================================ C ABI
using namespace tfx;

struct tfx_mc_t {
    tfx_context ctx = nullptr;
    int maxVerts = 0;
    int64_t maxCells = 0;
    float isoLevel = 0.f;        // SetSDFIsoLevel, in cells
    void* arena = nullptr;
    float4* verts = nullptr;     // {position, normal}[maxVerts]
    int* counter = nullptr;
    McTables* tables = nullptr;
    void* scratch = nullptr;      // block sums + block offsets
};

static void mc_count_table(const int32_t* edge, const int32_t* tri, McTables* T) {
    std::memcpy(T->edge, edge, sizeof(T->edge));
    std::memcpy(T->tri, tri, sizeof(T->tri));
    for (int c = 0; c < 256; ++c) {
        int nv = 0;
        while (nv < 16 && tri[16 * c + nv] != -1) ++nv;
        T->count[c] = edge[c] ? nv : 0;
    }
}

extern "C" int tfx_mc_default_tables(int32_t* edge_table, int32_t* tri_table) {
    if (!edge_table || !tri_table) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mc_default_tables: null argument");
    mc_default_tables(edge_table, tri_table);
    return TFX_OK;
}

extern "C" int tfx_mc_set_tables(tfx_mc mc, const int32_t* edge_table, const int32_t* tri_table) {
    if (!mc) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mc_set_tables: null handle");
    if (!edge_table != !tri_table) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mc_set_tables: give both tables or neither");
    McTables T;
    if (edge_table) {
        for (int i = 0; i < 256 * 16; ++i)
            if (tri_table[i] < -1 || tri_table[i] > 11)
                return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mc_set_tables: triangle table entry %d = %d is not an edge", i,
                            tri_table[i]);
        mc_count_table(edge_table, tri_table, &T);
    } else {
        int32_t e[256], t[256 * 16];
        mc_default_tables(e, t);
        mc_count_table(e, t, &T);
    }
    TFX_CUDA(cudaSetDevice(mc->ctx->device), "cudaSetDevice");
    TFX_CUDA(cudaMemcpyAsync(mc->tables, &T, sizeof(T), cudaMemcpyHostToDevice, mc->ctx->stream), "tfx_mc_set_tables");
    TFX_CUDA(cudaStreamSynchronize(mc->ctx->stream), "cudaStreamSynchronize");
    return TFX_OK;
}

extern "C" int tfx_mc_create(tfx_context ctx, int max_vertices, int64_t max_cells, tfx_mc* out) {
    if (!out) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mc_create: out is null");
    *out = nullptr;
    if (!ctx || max_vertices < 0 || max_cells <= 0 || max_cells > 0x7fffffffLL - kMcThreads)
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mc_create: max_vertices %d max_cells %lld", max_vertices,
                    (long long)max_cells);
    TFX_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    auto* h = new (std::nothrow) tfx_mc_t();
    if (!h) return fail(TFX_ERR_OUT_OF_MEMORY, "tfx_mc_create: host allocation");
    h->ctx = ctx;
    h->maxVerts = max_vertices;
    h->maxCells = max_cells;
    const size_t vb = ((size_t)max_vertices * 32 + 255) & ~(size_t)255;
    const size_t tb = (sizeof(McTables) + 255) & ~(size_t)255;
    const size_t bb = mc_scratch_bytes(max_cells);
    const size_t total = vb + 256 + tb + bb;
    cudaError_t e = cudaMalloc(&h->arena, total);
    if (e != cudaSuccess) {
        delete h;
        return cuda_fail(e, "tfx_mc_create: device allocation");
    }
    char* p = (char*)h->arena;
    h->verts = (float4*)p;
    h->counter = (int*)(p + vb);
    h->tables = (McTables*)(p + vb + 256);
    h->scratch = p + vb + 256 + tb;
    context_retain(ctx);
    // InitializeMCVertices before the first Update: zero vertices, zero counter
    e = cudaMemsetAsync(h->arena, 0, vb + 256, ctx->stream);
    if (e != cudaSuccess) {
        tfx_mc_destroy(h);
        return cuda_fail(e, "tfx_mc_create: memset");
    }
    if (int r = tfx_mc_set_tables(h, nullptr, nullptr)) {
        tfx_mc_destroy(h);
        return r;
    }
    *out = h;
    return TFX_OK;
}

extern "C" int tfx_mc_destroy(tfx_mc mc) {
    if (!mc) return TFX_OK;
    cudaSetDevice(mc->ctx->device);
    if (mc->arena) {
        cudaStreamSynchronize(mc->ctx->stream);
        cudaFree(mc->arena);
    }
    context_release(mc->ctx);
    delete mc;
    return TFX_OK;
}

extern "C" int tfx_mc_set_iso_level(tfx_mc mc, float iso_level) {
    if (!mc) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mc_set_iso_level: null handle");
    mc->isoLevel = iso_level;
    return TFX_OK;
}

extern "C" int tfx_mc_run(tfx_mc mc, const float* sdf_device, const tfx_sdf_grid* grid) {
    if (!mc || !sdf_device || !grid) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mc_run: null argument");
    if (grid->num_cells_x <= 0 || grid->num_cells_y <= 0 || grid->num_cells_z <= 0 || !(grid->cell_size > 0.0f))
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mc_run: grid %dx%dx%d cell %g", grid->num_cells_x, grid->num_cells_y,
                    grid->num_cells_z, (double)grid->cell_size);
    const int64_t cells = (int64_t)grid->num_cells_x * grid->num_cells_y * grid->num_cells_z;
    if (cells > mc->maxCells)
        return fail(TFX_ERR_SIZE, "tfx_mc_run: grid of %lld cells exceeds max_cells %lld", (long long)cells,
                    (long long)mc->maxCells);
    const SdfGrid g{grid->origin[0], grid->origin[1], grid->origin[2], grid->cell_size,
                    grid->num_cells_x, grid->num_cells_y, grid->num_cells_z, 0};
    // g_MarchingCubesIsolevel = m_CellSize * m_SDFIsoLevel (TressFXSDFMarchingCubes.cpp:191)
    const float iso = grid->cell_size * mc->isoLevel;
    TFX_CUDA(cudaSetDevice(mc->ctx->device), "cudaSetDevice");
    cudaError_t e = launch_marching_cubes(sdf_device, g, iso, mc->tables, mc->maxVerts, mc->scratch, mc->verts,
                                          mc->counter, mc->ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "marching cubes launch");
    return TFX_OK;
}

extern "C" int tfx_mc_update(tfx_mc mc, tfx_sdf sdf, const tfx_sdf_grid* grid) {
    if (!mc || !sdf || !grid) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mc_update: null argument");
    void* buf = nullptr;
    size_t bytes = 0;
    if (int r = tfx_sdf_get_buffer(sdf, &buf, &bytes)) return r;
    const int64_t cells = (int64_t)grid->num_cells_x * grid->num_cells_y * grid->num_cells_z;
    if (cells < 0 || (size_t)cells * 4 > bytes)
        return fail(TFX_ERR_SIZE, "tfx_mc_update: grid of %lld cells exceeds the SDF allocation", (long long)cells);
    return tfx_mc_run(mc, (const float*)buf, grid);
}

extern "C" int tfx_mc_get_buffers(tfx_mc mc, void** vertices, int32_t** num_vertices) {
    if (!mc) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mc_get_buffers: null handle");
    if (vertices) *vertices = mc->verts;
    if (num_vertices) *num_vertices = mc->counter;
    return TFX_OK;
}

extern "C" int tfx_mc_read(tfx_mc mc, void* host_vertices, size_t bytes, int32_t* num_vertices) {
    if (!mc || (!host_vertices && bytes)) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mc_read: bad argument");
    if (bytes > (size_t)mc->maxVerts * 32)
        return fail(TFX_ERR_SIZE, "tfx_mc_read: %zu bytes > %d vertices", bytes, mc->maxVerts);
    TFX_CUDA(cudaSetDevice(mc->ctx->device), "cudaSetDevice");
    if (bytes)
        TFX_CUDA(cudaMemcpyAsync(host_vertices, mc->verts, bytes, cudaMemcpyDeviceToHost, mc->ctx->stream), "tfx_mc_read");
    if (num_vertices)
        TFX_CUDA(cudaMemcpyAsync(num_vertices, mc->counter, sizeof(int32_t), cudaMemcpyDeviceToHost, mc->ctx->stream),
                 "tfx_mc_read");
    TFX_CUDA(cudaStreamSynchronize(mc->ctx->stream), "cudaStreamSynchronize");
    return TFX_OK;
}
