// tfx_sdf_build_static: the SDF build (Initialize, Construct, Finalize) into a caller-provided float
// grid, allocating nothing.  It is for callers that cannot allocate device memory while they run:
// an engine that sets its GPU memory budget once at start-up and forbids allocation per frame, or a
// frame recorded in a CUDA graph, where an allocation would stall or invalidate the recording.  The
// FloatFlip3 word grid that the build accumulates its atomicMin into (the scratch that
// tfx_sdf_create allocates for the other entry points) is a file-scope device array of
// TFX_SDF_STATIC_MAX_CELLS words, which every device that loads the library holds until exit.
//
// Rules of use:
//   - the array's device address is looked up (cudaGetSymbolAddress, with the context's device
//     current) by the first call on each context and kept in the context; make that first call
//     before any stream capture.  A device reset ends the context, and a new context looks the
//     address up again;
//   - nothing has to start at zero: every call first writes FloatFlip3(1e10) into all cells it uses;
//   - there is one array per device, so calls whose work can overlap on one device (two contexts,
//     two streams, two host threads) race on it; calls on one context are stream-ordered and safe;
//   - the triangle indices must be below num_vertices; they are not checked.
#include <mutex>

#include "tfx_handles.h"
#include "tfx_sdf_math.cuh"

namespace {

using namespace tfx;

__device__ __align__(256) uint32_t g_sdf_static_words[TFX_SDF_STATIC_MAX_CELLS];

std::mutex g_symbol_mutex;

// FinalizeSignedDistanceField (TressFXSDFCollision.hlsl:400-412), decoding into a separate output:
// out[c] = asfloat(IFloatFlip3(words[c])).  Four cells per thread.
__global__ void __launch_bounds__(256) k_sdf_finalize_into(const uint32_t* __restrict__ words, float* __restrict__ out,
                                                           long long cells) {
    const long long quads = (cells + 3) / 4;
    for (long long qd = blockIdx.x * (long long)blockDim.x + threadIdx.x; qd < quads;
         qd += (long long)gridDim.x * blockDim.x) {
        const long long c = 4 * qd;
        if (c + 4 <= cells) {
            const uint4 u = *reinterpret_cast<const uint4*>(words + c);
            out[c + 0] = __uint_as_float(ifloat_flip3(u.x));
            out[c + 1] = __uint_as_float(ifloat_flip3(u.y));
            out[c + 2] = __uint_as_float(ifloat_flip3(u.z));
            out[c + 3] = __uint_as_float(ifloat_flip3(u.w));
        } else {
            for (long long i = c; i < cells; ++i) out[i] = __uint_as_float(ifloat_flip3(words[i]));
        }
    }
}

// The array's device address for this context (looked up on the context's first call; the caller has
// made the context's device current).
int static_words(tfx_context ctx, uint32_t** out) {
    std::lock_guard<std::mutex> lock(g_symbol_mutex);
    if (!ctx->sdfStaticWords) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_sdf_static_words);
        if (e != cudaSuccess) return cuda_fail(e, "tfx_sdf_build_static: cudaGetSymbolAddress");
        ctx->sdfStaticWords = static_cast<uint32_t*>(p);
    }
    *out = ctx->sdfStaticWords;
    return TFX_OK;
}

// Puts the calling thread's current device back on every return path.
struct CurrentDeviceGuard {
    int saved = -1;
    CurrentDeviceGuard() {
        if (cudaGetDevice(&saved) != cudaSuccess) saved = -1;
    }
    ~CurrentDeviceGuard() {
        if (saved >= 0) cudaSetDevice(saved);
    }
};

}  // namespace

extern "C" int tfx_sdf_build_static(tfx_context ctx, const tfx_sdf_grid* grid, const void* mesh_vertices,
                                    int num_vertices, const uint32_t* indices, int num_triangles, float* sdf_out) {
    if (!ctx || !grid || !sdf_out) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_sdf_build_static: null argument");
    if (num_vertices < 0 || num_triangles < 0 || (num_triangles > 0 && (!mesh_vertices || !indices)))
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_sdf_build_static: bad mesh (%d vertices, %d triangles)", num_vertices,
                    num_triangles);
    if (((uintptr_t)mesh_vertices & 15) != 0)
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_sdf_build_static: mesh buffer not 16-byte aligned");
    if (((uintptr_t)sdf_out & 3) != 0)
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_sdf_build_static: output buffer not 4-byte aligned");
    if (grid->num_cells_x <= 0 || grid->num_cells_y <= 0 || grid->num_cells_z <= 0 || !(grid->cell_size > 0.0f))
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_sdf_build_static: grid %dx%dx%d cell %g", grid->num_cells_x,
                    grid->num_cells_y, grid->num_cells_z, (double)grid->cell_size);
    const int64_t cells = (int64_t)grid->num_cells_x * grid->num_cells_y * grid->num_cells_z;
    if (cells > TFX_SDF_STATIC_MAX_CELLS)
        return fail(TFX_ERR_SIZE, "tfx_sdf_build_static: grid of %lld cells exceeds the static scratch of %d cells",
                    (long long)cells, TFX_SDF_STATIC_MAX_CELLS);
    CurrentDeviceGuard keep;
    TFX_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    uint32_t* words = nullptr;
    if (int r = static_words(ctx, &words)) return r;
    const SdfGrid g{grid->origin[0], grid->origin[1], grid->origin[2], grid->cell_size,
                    grid->num_cells_x, grid->num_cells_y, grid->num_cells_z, 0};
    cudaError_t e = launch_sdf_initialize(words, cells, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "tfx_sdf_build_static: initialize launch");
    e = launch_sdf_construct(words, g, static_cast<const float4*>(mesh_vertices), indices, num_triangles, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "tfx_sdf_build_static: construct launch");
    const long long quads = (cells + 3) / 4;
    const unsigned blocks = (unsigned)std::min<long long>((quads + 255) / 256, (long long)sm_count() * 16);
    k_sdf_finalize_into<<<blocks, 256, 0, ctx->stream>>>(words, sdf_out, cells);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "tfx_sdf_build_static: finalize launch");
    return TFX_OK;
}
