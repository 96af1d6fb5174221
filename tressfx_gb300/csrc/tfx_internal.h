// Internal structures shared by the C ABI (tfx_capi.cu) and the kernel translation units.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace tfx {

// Per-object simulation constants as the kernels read them from device memory.  Filled by
// tfx_hair_update_constants from a tfx_sim_params block (TressFXSimulationParams layout); the
// damping decay exp(-damping*dt*60) of Integrate() (TressFXSimulation.hlsl:444) is a per-dispatch
// uniform and is evaluated once on the host with expf.
struct DevSimConsts {
    float4 wind[4];
    float damping, localStiffness, globalStiffness, globalRange;
    float gravity, timeStep, tipSeparation, decay;
    int lengthIterations, localIterations, anyWind, reserved0;
    float vspCoeff, vspAccelThreshold, reset, clamp;
    float4 bones[512 * 4];  // 512 row-major 4x4 matrices
};
static_assert(offsetof(DevSimConsts, bones) == 128, "DevSimConsts header must stay 128 bytes");

// Device view of one hair object: the TressFXDynamicState UAVs and TressFXHairObject SRVs.
struct HairView {
    float4* pos;
    float4* prev;
    float4* prevprev;
    float4* tan;
    float4* sld;                 // StrandLevelData: 3 float4 per strand
    const float4* init;
    const float* rest;
    const float4* followOffset;
    const float4* skin;          // 2 float4 per strand: bone indices, bone weights
    const DevSimConsts* consts;
    int G;                       // guide strands
    int n;                       // vertices per strand
    int F;                       // follow hairs per guide
    int reserved;
};

struct SdfGrid {
    float ox, oy, oz, cell;
    int nx, ny, nz, reserved;
};

// Streaming multiprocessors of the current device, looked up once per device ordinal.  Grid-stride
// launches size their grids as a multiple of it.
int sm_count();

// Launchers (tfx_sim_kernels.cu / tfx_sdf_kernels.cu). Return cudaGetLastError() of the launch.
cudaError_t launch_integrate(const HairView& h, cudaStream_t s);
cudaError_t launch_strand_level(const HairView& h, cudaStream_t s);
cudaError_t launch_vsp(const HairView& h, cudaStream_t s);
cudaError_t launch_local_shape(const HairView& h, cudaStream_t s);
cudaError_t launch_length_wind(const HairView& h, cudaStream_t s);
cudaError_t launch_follow(const HairView& h, cudaStream_t s);

cudaError_t launch_sdf_initialize(uint32_t* sdf, int64_t cells, cudaStream_t s);
cudaError_t launch_sdf_construct(uint32_t* sdf, const SdfGrid& g, const float4* mesh, const uint32_t* idx,
                                 int ntri, cudaStream_t s);
cudaError_t launch_sdf_finalize(uint32_t* sdf, int64_t cells, cudaStream_t s);
cudaError_t launch_sdf_collide(const uint32_t* sdf, const SdfGrid& g, float margin, float4* pos, float4* prev,
                               int n, int64_t vtot, cudaStream_t s);
// Strand quad expansion (TressFXStrands.hlsl GetExpandedTressFXVert), by value into the kernel.
struct ExpandParams {
    float baseColor[4], tipColor[4];
    float tipPercentage, fiberRatio, fiberRadius;
    int n, enableThinTip, shadow;
    float eye[3];
    float winH;
    float viewProj[16];   // row-major, applied as mul(M, v)
};
cudaError_t launch_expand_strands(const float4* pos, const float4* tan, int64_t vtot, const ExpandParams& P, float4* out,
                                  cudaStream_t s);
cudaError_t launch_sdf_collide_mixed(const uint32_t* sdf, const SdfGrid& g, float margin, float4* pos, float4* prev,
                                     int64_t vtot, cudaStream_t s);
cudaError_t launch_mesh_skin(float4* out, const float4* in, const float4* skin, const float4* bones, int nverts,
                             cudaStream_t s);

}  // namespace tfx
