// Definitions of the opaque C-ABI handles and the error helpers shared by the C-ABI translation
// units (tfx_capi.cu, tfx_batch_capi.cu).
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <string>
#include <vector>

#include "../../include/tressfx_gb300.h"
#include "tfx_internal.h"

// A context is reference counted: every hair object, SDF, mesh and batch created on it holds a
// reference, so tfx_context_destroy may be called before the objects are destroyed; the stream is
// released with the last reference.
struct tfx_context_t {
    int device = 0;
    int numSMs = 0;
    cudaStream_t stream = nullptr;
    std::atomic<int> refs{1};
    std::vector<std::string> stampNames;
    std::vector<cudaEvent_t> stampEvents;
    uint32_t* sdfStaticWords = nullptr;   // device address of tfx_sdf_build_static's array, once looked up
};

struct tfx_hair_t {
    tfx_context ctx = nullptr;
    int G = 0, n = 0, F = 0;
    int64_t Vtot = 0, Stot = 0;
    int maxBone = 0;                               // highest bone index the guide skinning reads
    void* arena = nullptr;
    size_t arenaBytes = 0;
    tfx::HairView view{};
    tfx::DevSimConsts* consts = nullptr;           // device
    tfx::DevSimConsts* staging[2] = {nullptr, nullptr};  // pinned host (double buffered like m_SimCB[2])
    cudaEvent_t stagingDone[2] = {nullptr, nullptr};
    bool stagingUsed[2] = {false, false};
    int stagingNext = 0;
    struct Buf { void* ptr; size_t bytes; } bufs[10]{};
    unsigned long long* health = nullptr;          // device: non-finite counts of Pos and Prev
};

struct tfx_sdf_t {
    tfx_context ctx = nullptr;
    uint32_t* grid = nullptr;
    int64_t alloc = 0;
    const float4* mesh = nullptr;
    int nverts = 0;
    const uint32_t* idx = nullptr;
    int ntri = 0;
};

struct tfx_mesh_t {
    tfx_context ctx = nullptr;
    int nverts = 0, ntri = 0;
    int maxBone = 0;
    void* arena = nullptr;
    float4* bind = nullptr;     // {position, normal}[nverts]
    float4* skinned = nullptr;  // {position, normal}[nverts]
    float4* skin = nullptr;     // {boneIndex, boneWeight}[nverts]
    uint32_t* idx = nullptr;
    float4* bones = nullptr;    // 512 matrices
    float* staging[2] = {nullptr, nullptr};
    cudaEvent_t stagingDone[2] = {nullptr, nullptr};
    bool stagingUsed[2] = {false, false};
    int stagingNext = 0;
};

namespace tfx {
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);
void context_retain(tfx_context c);
void context_release(tfx_context c);
size_t align256(size_t x);
// Fills the 128-byte scalar header of a DevSimConsts from a TressFXSimulationParams block.
void fill_consts_header(DevSimConsts* c, const tfx_sim_params* p, int cpuLocalIterations);
}  // namespace tfx

#define TFX_CUDA(call, what)                                     \
    do {                                                         \
        cudaError_t _e = (call);                                 \
        if (_e != cudaSuccess) return tfx::cuda_fail(_e, what);  \
    } while (0)
