// tfx_hair_count_nonfinite: a report-only health check of a hair object's state.  The reference's only
// guard against a diverging simulation is the velocity clamp of LengthConstriantsWindAndCollision
// (TressFXSimulation.hlsl:959-964), which cannot repair a NaN or an infinity once one appears: every
// later stage propagates it along the strand.  This scan counts the vertices of Pos and of Prev with a
// non-finite component (x, y, z or the inverse mass w), changes nothing, and lets the host decide
// (reset the object, restore a snapshot) before a renderer draws the frame.
#include "tfx_handles.h"

namespace {

using namespace tfx;

__device__ __forceinline__ bool finite4(float4 v) {
    return isfinite(v.x) && isfinite(v.y) && isfinite(v.z) && isfinite(v.w);
}

// One float4 of each buffer per thread (coalesced 16-byte loads), a ballot per warp, one atomic per
// warp and buffer.
__global__ void __launch_bounds__(256) k_count_nonfinite(const float4* __restrict__ pos, const float4* __restrict__ prev,
                                                         long long vtot, unsigned long long* __restrict__ counts) {
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    unsigned long long badPos = 0, badPrev = 0;
    for (long long base = blockIdx.x * (long long)blockDim.x; base < vtot; base += stride) {
        const long long v = base + threadIdx.x;
        bool bp = false, bq = false;
        if (v < vtot) {
            bp = !finite4(__ldg(pos + v));
            bq = !finite4(__ldg(prev + v));
        }
        badPos += __popc(__ballot_sync(0xffffffffu, bp));
        badPrev += __popc(__ballot_sync(0xffffffffu, bq));
    }
    if (lane == 0) {
        if (badPos) atomicAdd(counts + 0, badPos);
        if (badPrev) atomicAdd(counts + 1, badPrev);
    }
}

}  // namespace

extern "C" int tfx_hair_count_nonfinite(tfx_hair h, int64_t counts[2]) {
    if (!h || !counts) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_hair_count_nonfinite: null argument");
    TFX_CUDA(cudaSetDevice(h->ctx->device), "cudaSetDevice");
    cudaStream_t s = h->ctx->stream;
    TFX_CUDA(cudaMemsetAsync(h->health, 0, 2 * sizeof(unsigned long long), s), "tfx_hair_count_nonfinite: clear");
    const long long work = (h->Vtot + 255) / 256;
    const unsigned blocks = (unsigned)std::max<long long>(1, std::min<long long>(work, (long long)sm_count() * 8));
    k_count_nonfinite<<<blocks, 256, 0, s>>>(h->view.pos, h->view.prev, h->Vtot, h->health);
    TFX_CUDA(cudaGetLastError(), "tfx_hair_count_nonfinite: launch");
    unsigned long long host[2] = {0, 0};
    TFX_CUDA(cudaMemcpyAsync(host, h->health, sizeof(host), cudaMemcpyDeviceToHost, s), "tfx_hair_count_nonfinite: copy");
    TFX_CUDA(cudaStreamSynchronize(s), "tfx_hair_count_nonfinite: synchronize");
    counts[0] = (int64_t)host[0];
    counts[1] = (int64_t)host[1];
    return TFX_OK;
}
