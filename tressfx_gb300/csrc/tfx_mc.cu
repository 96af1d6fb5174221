// Iso-surface extraction of a signed distance grid (TressFXSDFMarchingCubes, src/TressFX/
// TressFXSDFMarchingCubes.cpp:27-233, and RunMarchingCubesOnSdf, src/Shaders/TressFXMarchingCubes.hlsl:
// 147-280), headless: the triangle soup lands in a device vertex buffer.
//
// The reference appends each cube's triangles at an atomically reserved offset, so its vertex order
// changes from run to run.  Here the offsets are an exclusive prefix sum of the cubes' vertex counts
// in cell-index order -- the order a one-thread-at-a-time dispatch of the shader produces -- so the
// buffer is deterministic and bit-comparable.  Two passes over the grid:
//   k_mc_count: 4096 cells per block (16 per thread, coalesced along x), one vertex-count sum per block;
//   k_mc_write: each block sums the counts of the blocks before it, scans its own cells and writes
//               the triangles of every cube whose range ends before max_vertices (the shader's
//               `offset + num < max`), zeros what InitializeMCVertices would leave zero, and block 0
//               stores the total (the shader's counter, which also counts cubes that did not fit).
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

constexpr int kMcThreads = 256;
constexpr int kMcPerThread = 16;
constexpr int kMcBlockCells = kMcThreads * kMcPerThread;

// Corner k of a cube sits at cell + kCorner[k] (TressFXMarchingCubes.hlsl:165-173); edge e joins the
// corners kEdgeA[e] -> kEdgeB[e], in the argument order of its VertexLerp call (:211-222).
__constant__ int8_t kCornerX[8] = {0, 1, 1, 0, 0, 1, 1, 0};
__constant__ int8_t kCornerY[8] = {0, 0, 0, 0, 1, 1, 1, 1};
__constant__ int8_t kCornerZ[8] = {0, 0, 1, 1, 0, 0, 1, 1};
__constant__ int8_t kEdgeA[12] = {0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 2, 3};
__constant__ int8_t kEdgeB[12] = {1, 2, 3, 0, 5, 6, 7, 4, 4, 5, 6, 7};

struct McCell {
    int x, y, z;
    float s[8];
    int config;          // cubeIndex; -1 for cells on the upper faces of the grid
};

__device__ __forceinline__ McCell mc_cell(const float* __restrict__ sdf, const SdfGrid& g, int index, float iso) {
    McCell c;
    const uint32_t perLine = (uint32_t)g.nx, perPlane = (uint32_t)(g.nx * g.ny);
    const uint32_t u = (uint32_t)index;
    c.z = (int)(u / perPlane);
    const uint32_t rem = u % perPlane;
    c.y = (int)(rem / perLine);
    c.x = (int)(rem % perLine);
    c.config = -1;
    if (c.x >= g.nx - 1 || c.y >= g.ny - 1 || c.z >= g.nz - 1) return c;
    const int plane = g.nx * g.ny;
    const float* p = sdf + (plane * c.z + g.nx * c.y + c.x);
    // corners 0..7: (0,0,0) (1,0,0) (1,0,1) (0,0,1) (0,1,0) (1,1,0) (1,1,1) (0,1,1)
    c.s[0] = __ldg(p);
    c.s[1] = __ldg(p + 1);
    c.s[2] = __ldg(p + plane + 1);
    c.s[3] = __ldg(p + plane);
    c.s[4] = __ldg(p + g.nx);
    c.s[5] = __ldg(p + g.nx + 1);
    c.s[6] = __ldg(p + plane + g.nx + 1);
    c.s[7] = __ldg(p + plane + g.nx);
    int cfg = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (c.s[k] < iso) cfg |= 1 << k;
    c.config = cfg;
    return c;
}

// GetSdfCellPosition: float3(cell) * cellSize, then + origin.
__device__ __forceinline__ float3 mc_corner(const McCell& c, const SdfGrid& g, int k) {
    float3 p = make_float3((float)(c.x + kCornerX[k]) * g.cell, (float)(c.y + kCornerY[k]) * g.cell,
                           (float)(c.z + kCornerZ[k]) * g.cell);
    return make_float3(p.x + g.ox, p.y + g.oy, p.z + g.oz);
}

// VertexLerp: p1 + (p2 - p1) * ((iso - s1) / (s2 - s1)).
__device__ __forceinline__ float3 mc_edge_vertex(const McCell& c, const SdfGrid& g, int e, float iso) {
    const int a = kEdgeA[e], b = kEdgeB[e];
    float sa = 0.f, sb = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        sa = (k == a) ? c.s[k] : sa;
        sb = (k == b) ? c.s[k] : sb;
    }
    const float interp = (iso - sa) / (sb - sa);
    const float3 p1 = mc_corner(c, g, a), p2 = mc_corner(c, g, b);
    return make_float3(p1.x + (p2.x - p1.x) * interp, p1.y + (p2.y - p1.y) * interp, p1.z + (p2.z - p1.z) * interp);
}

__device__ __forceinline__ int block_sum(int v, int* red) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    int t = 0;
#pragma unroll
    for (int w = 0; w < kMcThreads / 32; ++w) t += red[w];
    return t;
}

// Exclusive scan over the block; *total receives the block's sum.
__device__ __forceinline__ int block_exclusive_scan(int v, int* red, int* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int n = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += n;
    }
    __syncthreads();
    if (lane == 31) red[warp] = incl;
    __syncthreads();
    int before = 0, all = 0;
#pragma unroll
    for (int w = 0; w < kMcThreads / 32; ++w) {
        const int t = red[w];
        before += (w < warp) ? t : 0;
        all += t;
    }
    *total = all;
    return before + incl - v;
}

__global__ void __launch_bounds__(kMcThreads) k_mc_count(const float* __restrict__ sdf, SdfGrid g, float iso,
                                                         const McTables* __restrict__ T, int totalCells,
                                                         int* __restrict__ blockSums) {
    __shared__ int cnt[256];
    __shared__ int red[kMcThreads / 32];
    cnt[threadIdx.x] = T->count[threadIdx.x];
    __syncthreads();
    const int base = blockIdx.x * kMcBlockCells;
    int sum = 0;
#pragma unroll 4
    for (int j = 0; j < kMcPerThread; ++j) {
        const int idx = base + j * kMcThreads + (int)threadIdx.x;
        if (idx >= totalCells) break;
        const McCell c = mc_cell(sdf, g, idx, iso);
        if (c.config >= 0) sum += cnt[c.config];
    }
    const int t = block_sum(sum, red);
    if (threadIdx.x == 0) blockSums[blockIdx.x] = t;
}

__device__ __forceinline__ void mc_zero(float4* out, long long v) {
    out[2 * v] = make_float4(0.f, 0.f, 0.f, 0.f);
    out[2 * v + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void __launch_bounds__(kMcThreads) k_mc_write(const float* __restrict__ sdf, SdfGrid g, float iso,
                                                         const McTables* __restrict__ T, int totalCells,
                                                         const int* __restrict__ blockSums, int numBlocks, int maxVerts,
                                                         float4* __restrict__ out, int* __restrict__ counter) {
    __shared__ int cnt[256];
    __shared__ int red[kMcThreads / 32];
    cnt[threadIdx.x] = T->count[threadIdx.x];
    // prefix of the earlier blocks and the grand total, summed in 64 bits (the counter, an int as in
    // the shader, receives the low 32 bits)
    long long before = 0, all = 0;
    for (int b = threadIdx.x; b < numBlocks; b += kMcThreads) {
        const int s = __ldg(blockSums + b);
        all += s;
        before += (b < (int)blockIdx.x) ? s : 0;
    }
    {
        __shared__ long long red2[2][kMcThreads / 32];
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            before += __shfl_xor_sync(0xffffffffu, before, o);
            all += __shfl_xor_sync(0xffffffffu, all, o);
        }
        if ((threadIdx.x & 31) == 0) {
            red2[0][threadIdx.x >> 5] = before;
            red2[1][threadIdx.x >> 5] = all;
        }
        __syncthreads();
        before = 0;
        all = 0;
#pragma unroll
        for (int w = 0; w < kMcThreads / 32; ++w) {
            before += red2[0][w];
            all += red2[1][w];
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *counter = (int)all;
    // vertices past the last reservation keep InitializeMCVertices' zeros
    for (long long v = all + (long long)blockIdx.x * kMcThreads + threadIdx.x; v < maxVerts;
         v += (long long)gridDim.x * kMcThreads)
        mc_zero(out, v);
    const int mine = __ldg(blockSums + blockIdx.x);
    if (mine == 0 || before >= maxVerts) {
        // nothing of this block fits: zero the part of its reservations below maxVerts
        if (mine != 0)
            for (long long v = before + threadIdx.x; v < before + mine && v < maxVerts; v += kMcThreads) mc_zero(out, v);
        return;
    }
    const int base = blockIdx.x * kMcBlockCells;
    long long running = before;
    for (int j = 0; j < kMcPerThread; ++j) {
        const int idx = base + j * kMcThreads + (int)threadIdx.x;
        McCell c;
        c.config = -1;
        if (idx < totalCells) c = mc_cell(sdf, g, idx, iso);
        const int nv = c.config >= 0 ? cnt[c.config] : 0;
        int rowTotal;
        const long long offset = running + block_exclusive_scan(nv, red, &rowTotal);
        running += rowTotal;
        if (nv == 0) continue;
        if (offset + nv < maxVerts) {
            const int* tri = T->tri + 16 * c.config;
            const int ntri = nv / 3;
            for (int t = 0; t < ntri; ++t) {
                const float3 v0 = mc_edge_vertex(c, g, __ldg(tri + 3 * t), iso);
                const float3 v1 = mc_edge_vertex(c, g, __ldg(tri + 3 * t + 1), iso);
                const float3 v2 = mc_edge_vertex(c, g, __ldg(tri + 3 * t + 2), iso);
                // normalize(cross(v1 - v0, v2 - v0)) = n * (1 / sqrt(dot(n, n)))
                const float3 a = make_float3(v1.x - v0.x, v1.y - v0.y, v1.z - v0.z);
                const float3 b = make_float3(v2.x - v0.x, v2.y - v0.y, v2.z - v0.z);
                const float3 n = make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
                const float inv = 1.0f / sqrtf(n.x * n.x + n.y * n.y + n.z * n.z);
                const float4 nn = make_float4(n.x * inv, n.y * inv, n.z * inv, 0.f);
                float4* o = out + 2 * (offset + 3 * t);
                o[0] = make_float4(v0.x, v0.y, v0.z, 0.f);
                o[1] = nn;
                o[2] = make_float4(v1.x, v1.y, v1.z, 0.f);
                o[3] = nn;
                o[4] = make_float4(v2.x, v2.y, v2.z, 0.f);
                o[5] = nn;
            }
            for (int k = 3 * ntri; k < nv; ++k) mc_zero(out, offset + k);   // a count not divisible by 3
        } else {
            for (long long v = offset; v < offset + nv && v < maxVerts; ++v) mc_zero(out, v);
        }
    }
}

}  // namespace

int mc_num_blocks(long long cells) { return (int)((cells + kMcBlockCells - 1) / kMcBlockCells); }

cudaError_t launch_marching_cubes(const float* sdf, const SdfGrid& g, float iso, const McTables* tables, int maxVerts,
                                  int* blockSums, float4* out, int* counter, cudaStream_t s) {
    const long long cells = (long long)g.nx * g.ny * g.nz;
    const int nb = mc_num_blocks(cells);
    if (nb == 0) {
        cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(int), s);
        if (e == cudaSuccess && maxVerts > 0) e = cudaMemsetAsync(out, 0, (size_t)maxVerts * 32, s);
        return e;
    }
    k_mc_count<<<nb, kMcThreads, 0, s>>>(sdf, g, iso, tables, (int)cells, blockSums);
    k_mc_write<<<nb, kMcThreads, 0, s>>>(sdf, g, iso, tables, (int)cells, blockSums, nb, maxVerts, out, counter);
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
    int* blockSums = nullptr;
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
    if (!ctx || max_vertices < 0 || max_cells <= 0 || max_cells > 0x7fffffffLL - kMcBlockCells)
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
    const size_t bb = (size_t)mc_num_blocks(max_cells) * sizeof(int);
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
    h->blockSums = (int*)(p + vb + 256 + tb);
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
    cudaError_t e = launch_marching_cubes(sdf_device, g, iso, mc->tables, mc->maxVerts, mc->blockSums, mc->verts,
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
