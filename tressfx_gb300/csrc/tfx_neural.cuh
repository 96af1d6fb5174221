// Learned collision proxy: a pose-conditioned neural SDF.
//
// d(x, pose) ~ MLP(features(x, pose)) with 102 inputs (normalised xyz, 3 pose angles, sin and cos of
// pi * f_k * x_d for 16 frequencies f_k = 2^(k/3), k = 0..15, per axis), four hidden layers of 64 with
// SiLU and one output: the signed distance in grid cells, truncated to +-band.  BF16 weights and
// activations, FP32 accumulation, on the tensor cores (mma.sync m16n8k16): a warp carries a tile of 16
// points through all five layers in registers, the weights staged once per block in shared memory.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "tfx_internal.h"

namespace tfx {
namespace nsdf {

constexpr int NFEAT = 102;   // used inputs
constexpr int KIN = 112;     // inputs padded to 7 k-tiles of 16
constexpr int HID = 64;
constexpr int NFREQ = 16;
constexpr int OUTN = 8;      // output padded to one n-tile (column 0 used)

// shared / global bf16 weight block (rows padded for conflict-free fragment loads)
constexpr int RS1 = 120;     // row stride of the [64][112] first layer
constexpr int RSH = 72;      // row stride of 64-wide rows
constexpr int OFF_WT1 = 0;                        // [64 out][RS1]   W1 transposed
constexpr int OFF_WT2 = OFF_WT1 + HID * RS1;      // [64 out][RSH]   W2..W4 transposed
constexpr int OFF_WT3 = OFF_WT2 + HID * RSH;
constexpr int OFF_WT4 = OFF_WT3 + HID * RSH;
constexpr int OFF_WT5 = OFF_WT4 + HID * RSH;      // [8 out][RSH]    W5 transposed
constexpr int OFF_WN2 = OFF_WT5 + OUTN * RSH;     // [64 in][RSH]    W2..W4 as stored (for backward)
constexpr int OFF_WN3 = OFF_WN2 + HID * RSH;
constexpr int OFF_WN4 = OFF_WN3 + HID * RSH;
constexpr int WBF_FWD = OFF_WN2;                  // elements the forward pass needs
constexpr int WBF_ALL = OFF_WN4 + HID * RSH;      // elements forward + backward need
constexpr int NBIAS = 4 * HID + OUTN;             // b1..b4, b5 (fp32)

// master fp32 parameters, [in][out] matrices followed by their bias
constexpr int P_W1 = 0, P_B1 = P_W1 + KIN * HID;
constexpr int P_W2 = P_B1 + HID, P_B2 = P_W2 + HID * HID;
constexpr int P_W3 = P_B2 + HID, P_B3 = P_W3 + HID * HID;
constexpr int P_W4 = P_B3 + HID, P_B4 = P_W4 + HID * HID;
constexpr int P_W5 = P_B4 + HID, P_B5 = P_W5 + HID * OUTN;
constexpr int NPARAM = P_B5 + OUTN;

// Normalisation of the inputs.
struct Frame {
    float cx, cy, cz;        // box centre (world)
    float ihx, ihy, ihz;     // 1 / box half extent
    float poseScale;         // pose angle (radians) * poseScale
    float cell;              // grid cell (world): outputs are in cells
};

// One training / evaluation sample: normalised nothing -- world position, target distance in cells
// (truncated to +-band), pose angles (radians), weight.
struct Sample {
    float x, y, z, target;
    float p0, p1, p2, weight;
};

struct Pose {
    float a0, a1, a2;        // joint angles (radians)
};

// Distances (world units) at `count` points (xyz of float4 records) under one pose.
cudaError_t launch_query(const __nv_bfloat16* wbf, const float* bias, const Frame& fr, const float4* points, int count,
                         Pose pose, float* out, cudaStream_t s);
cudaError_t launch_query_samples(const __nv_bfloat16* wbf, const float* bias, const Frame& fr, const Sample* samples,
                                 int count, float* out, cudaStream_t s);
cudaError_t launch_train_step(const __nv_bfloat16* wbf, const float* bias, const Frame& fr, const Sample* pool,
                              long long poolSize, int batch, uint32_t seed, __nv_bfloat16* acts, float* grads,
                              float* lossSum, cudaStream_t s);
cudaError_t launch_adam(float* params, const float* grads, float* m, float* v, int step, float lr, float gradScale,
                        __nv_bfloat16* wbf, float* bias, cudaStream_t s);
cudaError_t launch_init_params(float* params, uint32_t seed, __nv_bfloat16* wbf, float* bias, cudaStream_t s);
// `count` training samples for one pose: near the skinned mesh ({pos, normal}[nverts]) and uniform in
// the grid box, each labelled with the trilinear value of the pose's grid (cells, truncated to
// +-band); points the grid leaves unset (1e10) are labelled +band where they lie outside the mesh's
// bounding sphere (centre, radius) and get weight 0 otherwise.
cudaError_t launch_sample(const float4* mesh, int nverts, const float* grid, const SdfGrid& g, float band, float sigma,
                          float3 sphereCentre, float sphereRadius, Pose pose, int count, uint32_t seed, Sample* out,
                          cudaStream_t s);
size_t acts_elements(int batch);

// ---- the forward pass on the fifth-generation tensor cores (tcgen05, tfx_neural_tc.cu)
// Packed weights: W1..W4 as K-major bf16 MMA operands [64 neurons][K] (K = 112 for layer 1, 80 for
// layers 2-4, the halved bias in two extra input columns), then w5 (fp32, 64) and b5.
constexpr int TC_K1 = KIN;
constexpr int TC_KH = HID + 16;
constexpr int TC_W1_BYTES = HID * TC_K1 * 2;
constexpr int TC_WH_BYTES = HID * TC_KH * 2;
constexpr int TC_OFF_W1 = 0;
constexpr int TC_OFF_W2 = TC_OFF_W1 + TC_W1_BYTES;
constexpr int TC_OFF_W3 = TC_OFF_W2 + TC_WH_BYTES;
constexpr int TC_OFF_W4 = TC_OFF_W3 + TC_WH_BYTES;
constexpr int TC_OFF_W5 = TC_OFF_W4 + TC_WH_BYTES;
constexpr int TC_N5 = 16;                                  // output layer as an N = 16 MMA (column 0 used)
constexpr int TC_OFF_B5 = TC_OFF_W5 + TC_N5 * TC_KH * 2;   // b5 (fp32), then padding to 16 bytes
constexpr int TC_WBYTES = TC_OFF_B5 + 16;
constexpr int TC_NWG = 4;                                  // warpgroups (tiles in flight) per block
// shared memory: the weights once per block, then an mbarrier per warpgroup and the tensor-memory
// address slot (the A operands and accumulators live in tensor memory)
constexpr size_t TC_SMEM = (size_t)TC_WBYTES + 8 * TC_NWG + 16;
static_assert(TC_WBYTES % 16 == 0, "packed weights are staged as 16-byte words");
enum { TC_POINTS = 0, TC_SAMPLES = 1, TC_CLASSIFY = 2 };

struct TcArgs {
    const uint8_t* wtc;
    Frame fr;
    Pose pose;
    const float4* pts;           // TC_POINTS / TC_CLASSIFY: xyz of float4 records
    const Sample* samples;       // TC_SAMPLES
    int count;                   // TC_POINTS / TC_SAMPLES
    float* out;
    int* err;                    // set when a bounded wait for the tensor cores gave up
    // TC_CLASSIFY: band selection and cell marks (as k_nsdf_classify)
    long long vtot;
    int n;
    float margin, slackCells;
    SdfGrid grid;
    int* bandList;
    int* bandCount;
    uint32_t* marks;
};
cudaError_t launch_pack_tc(const float* params, uint8_t* wtc, cudaStream_t s);
cudaError_t launch_query_tc(const TcArgs& a, cudaStream_t s);
cudaError_t launch_query_samples_tc(const TcArgs& a, cudaStream_t s);
cudaError_t launch_classify_tc(const TcArgs& a, cudaStream_t s);

}  // namespace nsdf
}  // namespace tfx

namespace tfx {
namespace nsdf {

// Collision with the proxy (one object): classify every vertex with j >= 2 by the network; those within
// margin + one cell of the surface join the band list and mark the grid cells their exact lookups
// read (a 3x3x3 block from their cell); the grid is then built only on marked cells (skipped when the
// band is empty) and the band vertices are collided exactly as CollideHairVerticesWithSdf_forward does.
struct CollideArgs {
    const __nv_bfloat16* wbf;
    const float* bias;
    Frame fr;
    Pose pose;
    float4* pos;
    float4* prev;
    int n;                   // vertices per strand
    long long vtot;
    SdfGrid grid;
    float margin;            // world units
    float slackCells;        // band: network distance below margin + slackCells cells
    uint32_t* words;         // the SDF words (FloatFlip3 while built, floats after)
    uint32_t* marks;         // one bit per grid cell, then one bit per 4x4x4-cell block (any cell marked)
    int* bandList;           // vertex indices
    int* bandCount;
    const float4* mesh;      // skinned {pos, normal}
    const uint32_t* indices;
    int ntri;
    const uint8_t* wtc;      // packed weights of the tensor-core forward pass, or null for mma.sync
    int* err;
};
cudaError_t launch_collide(const CollideArgs& a, cudaStream_t s);

}  // namespace nsdf
}  // namespace tfx
