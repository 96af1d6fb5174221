// Kernels of the learned collision proxy (tfx_neural.cuh): inference, training (fused forward +
// backward, weight gradients, Adam) and training-sample generation from grid SDFs.
//
// mma.sync m16n8k16 (bf16 x bf16 -> f32) fragment layouts used throughout, with g = lane / 4 and
// i = lane % 4:  A (16 x 16, row-major) regs {row g, cols 2i..2i+1}, {row g+8, same}, {row g,
// cols 2i+8..}, {row g+8, cols 2i+8..};  B (16 x 8) regs {rows 2i..2i+1, col g}, {rows 2i+8.., col g};
// C (16 x 8, f32) {row g, cols 2i, 2i+1}, {row g+8, cols 2i, 2i+1}.  The C fragments of n-tiles 2k and
// 2k+1 are exactly the A fragment of k-tile k of the next layer, so activations never leave registers.
#include "tfx_neural.cuh"
#include "tfx_sdf_math.cuh"

namespace tfx {
namespace nsdf {

namespace {

__constant__ float c_freq[NFREQ] = {
    1.0f, 1.2599210498948732f, 1.5874010519681994f, 2.0f, 2.5198420997897464f, 3.174802103936399f,
    4.0f, 5.039684199579493f, 6.349604207872798f, 8.0f, 10.079368399158986f, 12.699208415745595f,
    16.0f, 20.158736798317972f, 25.39841683149119f, 32.0f};   // 2^(k/3)

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void mma16816(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// The network is an approximation.  Its activation, SiLU(z) = z * sigmoid(z) = 0.5 z (1 + tanh(z / 2)),
// is evaluated on bf16 pairs with the hardware tanh: one MUFU operation per two activations, and
// the result is directly the next layer's bf16 A-fragment register.
__device__ __forceinline__ uint32_t silu2(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(0.5f * a, 0.5f * b);
    uint32_t t;
    asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t) : "r"(*reinterpret_cast<uint32_t*>(&h)));
    const __nv_bfloat162 r = __hfma2(h, *reinterpret_cast<__nv_bfloat162*>(&t), h);
    return *reinterpret_cast<const uint32_t*>(&r);
}
__device__ __forceinline__ float2 unpack_bf16(uint32_t u) {
    return __bfloat1622float2(*reinterpret_cast<__nv_bfloat162*>(&u));
}
__device__ __forceinline__ float silu_grad(float z) {
    const float s = __fdividef(1.0f, 1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

// sin(pi x), cos(pi x): x reduced exactly to [-1, 1] (x - 2 * rint(x / 2) is exact in binary floating
// point), then the hardware sine / cosine of pi * x'.
__device__ __forceinline__ void sincospi_fast(float x, float* s, float* c) {
    const float r = x - 2.0f * rintf(0.5f * x);
    const float a = 3.14159265358979f * r;
    *s = __sinf(a);
    *c = __cosf(a);
}

__device__ __forceinline__ uint32_t hash32(uint32_t x) {   // lowbias32 (C. Wellons)
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}
__device__ __forceinline__ float u01(uint32_t h) { return (float)(h >> 8) * (1.0f / 16777216.0f); }

// A fragment of k-tile kt from a 16-row bf16 tile in shared memory (row stride rs elements).
__device__ __forceinline__ void load_a(const __nv_bfloat16* T, int rs, int kt, int lane, uint32_t (&a)[4]) {
    const int g = lane >> 2, i = lane & 3;
    const __nv_bfloat16* r0 = T + g * rs + kt * 16 + 2 * i;
    const __nv_bfloat16* r1 = r0 + 8 * rs;
    a[0] = *reinterpret_cast<const uint32_t*>(r0);
    a[1] = *reinterpret_cast<const uint32_t*>(r1);
    a[2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
    a[3] = *reinterpret_cast<const uint32_t*>(r1 + 8);
}
// B fragment (n-tile nt, k-tile kt) of a weight block stored with n as the row (row stride rs).
__device__ __forceinline__ void load_b(const __nv_bfloat16* W, int rs, int nt, int kt, int lane, uint32_t& b0,
                                       uint32_t& b1) {
    const int g = lane >> 2, i = lane & 3;
    const __nv_bfloat16* r = W + (nt * 8 + g) * rs + kt * 16 + 2 * i;
    b0 = *reinterpret_cast<const uint32_t*>(r);
    b1 = *reinterpret_cast<const uint32_t*>(r + 8);
}
// B fragments of n-tiles nt and nt+1 (k-tile kt) with one ldmatrix.x4: lanes 8m..8m+7 address the rows
// of 8x8 matrix m = (n-tile nt + m/2, k half m%2); rows are 16-byte aligned (row strides 144 / 240 B)
// and the eight rows of a matrix fall in distinct bank quads.
__device__ __forceinline__ void load_b2(const __nv_bfloat16* W, int rs, int nt, int kt, int lane, uint32_t (&b)[4]) {
    const int m = lane >> 3, r = lane & 7;
    const __nv_bfloat16* row = W + ((nt + (m >> 1)) * 8 + r) * rs + kt * 16 + (m & 1) * 8;
    const uint32_t addr = (uint32_t)__cvta_generic_to_shared(row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(b[0]), "=r"(b[1]), "=r"(b[2]), "=r"(b[3])
                 : "r"(addr));
}
// C fragments (8 n-tiles) initialised with a bias vector.
__device__ __forceinline__ void init_bias(float (&C)[8][4], const float* b, int lane) {
    const int i = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float b0 = b[nt * 8 + 2 * i], b1 = b[nt * 8 + 2 * i + 1];
        C[nt][0] = b0; C[nt][1] = b1; C[nt][2] = b0; C[nt][3] = b1;
    }
}
// A fragments of the next layer from C, through SiLU or as they are.
template <bool SILU>
__device__ __forceinline__ void c_to_a(const float (&C)[8][4], uint32_t (&A)[4][4]) {
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
        if constexpr (SILU) {
            A[kt][0] = silu2(C[2 * kt][0], C[2 * kt][1]);
            A[kt][1] = silu2(C[2 * kt][2], C[2 * kt][3]);
            A[kt][2] = silu2(C[2 * kt + 1][0], C[2 * kt + 1][1]);
            A[kt][3] = silu2(C[2 * kt + 1][2], C[2 * kt + 1][3]);
        } else {
            A[kt][0] = pack_bf16(C[2 * kt][0], C[2 * kt][1]);
            A[kt][1] = pack_bf16(C[2 * kt][2], C[2 * kt][3]);
            A[kt][2] = pack_bf16(C[2 * kt + 1][0], C[2 * kt + 1][1]);
            A[kt][3] = pack_bf16(C[2 * kt + 1][2], C[2 * kt + 1][3]);
        }
    }
}
// The activations held in A fragments, back in C-fragment order (for storing them).
__device__ __forceinline__ void a_to_c(const uint32_t (&A)[4][4], float (&H)[8][4]) {
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
        float2 v;
        v = unpack_bf16(A[kt][0]); H[2 * kt][0] = v.x; H[2 * kt][1] = v.y;
        v = unpack_bf16(A[kt][1]); H[2 * kt][2] = v.x; H[2 * kt][3] = v.y;
        v = unpack_bf16(A[kt][2]); H[2 * kt + 1][0] = v.x; H[2 * kt + 1][1] = v.y;
        v = unpack_bf16(A[kt][3]); H[2 * kt + 1][2] = v.x; H[2 * kt + 1][3] = v.y;
    }
}
// C += A (16 x 64) * W^T for a 64-wide layer whose weights are stored [n][k] with row stride RSH.
__device__ __forceinline__ void layer64(float (&C)[8][4], const uint32_t (&A)[4][4], const __nv_bfloat16* W, int lane) {
#pragma unroll
    for (int kt = 0; kt < 4; ++kt)
#pragma unroll
        for (int nt = 0; nt < 8; nt += 2) {
            uint32_t b[4];
            load_b2(W, RSH, nt, kt, lane, b);
            mma16816(C[nt], A[kt][0], A[kt][1], A[kt][2], A[kt][3], b[0], b[1]);
            mma16816(C[nt + 1], A[kt][0], A[kt][1], A[kt][2], A[kt][3], b[2], b[3]);
        }
}

// Features of one point into row s of the tile: the lane pair (2s, 2s+1) splits the work.
__device__ __forceinline__ void write_features(__nv_bfloat16* F, int s, int half, float ux, float uy, float uz, float p0,
                                               float p1, float p2, bool valid) {
    __nv_bfloat16* row = F + s * RS1;
    const float u[3] = {ux, uy, uz};
    if (half == 0) {
        row[0] = __float2bfloat16(valid ? ux : 0.f);
        row[1] = __float2bfloat16(valid ? uy : 0.f);
        row[2] = __float2bfloat16(valid ? uz : 0.f);
        row[3] = __float2bfloat16(valid ? p0 : 0.f);
        row[4] = __float2bfloat16(valid ? p1 : 0.f);
        row[5] = __float2bfloat16(valid ? p2 : 0.f);
    }
    // f_{k+3} = 2 f_k: the three base frequencies of this half (k0, k0+1, k0+2) by the hardware sine /
    // cosine, every later one by the double-angle formulas sin 2a = 2 sin a cos a, cos 2a = 1 - 2 sin^2 a
    const int k0 = half * (NFREQ / 2);
#pragma unroll
    for (int b = 0; b < 3; ++b) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            float sn = 0.f, cs = 0.f;
            if (valid) sincospi_fast(c_freq[k0 + b] * u[d], &sn, &cs);
#pragma unroll
            for (int k = k0 + b; k < k0 + NFREQ / 2; k += 3) {
                *reinterpret_cast<__nv_bfloat162*>(row + 6 + 6 * k + 2 * d) = __floats2bfloat162_rn(sn, cs);
                const float s2 = 2.0f * sn * cs, c2 = 1.0f - 2.0f * sn * sn;
                sn = s2; cs = c2;
            }
        }
    }
    if (half == 1)
#pragma unroll
        for (int f = NFEAT; f < KIN; ++f) row[f] = __float2bfloat16(0.f);
}

// Stores a C-fragment tile (rows = 16 samples, ntiles x 8 columns) as sample-pair-interleaved bf16:
// 32-bit word (pair p, column c) holds (row 2p, row 2p+1) of column c at base[p * F + c].
__device__ __forceinline__ void store_pairs(const float (&C)[8][4], int ntiles, uint32_t* base, int F, int lane) {
    const int g = lane >> 2, i = lane & 3;
    const bool even = (g & 1) == 0;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        if (nt >= ntiles) break;
        const float v00 = C[nt][0], v01 = C[nt][1], v10 = C[nt][2], v11 = C[nt][3];
        const float x0 = __shfl_xor_sync(0xffffffffu, even ? v01 : v00, 4);
        const float x1 = __shfl_xor_sync(0xffffffffu, even ? v11 : v10, 4);
        const int c0 = nt * 8 + 2 * i;
        if (even) {
            base[(g >> 1) * F + c0] = pack_bf16(v00, x0);
            base[((g + 8) >> 1) * F + c0] = pack_bf16(v10, x1);
        } else {
            base[(g >> 1) * F + c0 + 1] = pack_bf16(x0, v01);
            base[((g + 8) >> 1) * F + c0 + 1] = pack_bf16(x1, v11);
        }
    }
}

// Forward pass of the tile in F (16 points).  y0 / y1 = outputs (cells) of rows g / g+8 (valid in lanes
// with lane % 4 == 0).  With TRAIN, pre-activations go to zsave (per lane, [4][32]) and activations
// (pair layout) to hout[1..4].
template <bool TRAIN>
__device__ __forceinline__ void mlp_forward(const __nv_bfloat16* sW, const float* sB, const __nv_bfloat16* F, int lane,
                                            float* zsave, uint32_t* const* hout, float& y0, float& y1) {
    float C[8][4];
    init_bias(C, sB, lane);
#pragma unroll 1
    for (int kt = 0; kt < KIN / 16; ++kt) {
        uint32_t a[4];
        load_a(F, RS1, kt, lane, a);
#pragma unroll
        for (int nt = 0; nt < 8; nt += 2) {
            uint32_t b[4];
            load_b2(sW + OFF_WT1, RS1, nt, kt, lane, b);
            mma16816(C[nt], a[0], a[1], a[2], a[3], b[0], b[1]);
            mma16816(C[nt + 1], a[0], a[1], a[2], a[3], b[2], b[3]);
        }
    }
    const int woff[3] = {OFF_WT2, OFF_WT3, OFF_WT4};
#pragma unroll 1
    for (int l = 0; l < 3; ++l) {
        uint32_t A[4][4];
        c_to_a<true>(C, A);
        if constexpr (TRAIN) {
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
#pragma unroll
                for (int q = 0; q < 4; ++q) zsave[l * 32 + nt * 4 + q] = C[nt][q];
            float H[8][4];
            a_to_c(A, H);
            store_pairs(H, 8, hout[l], HID, lane);
        }
        init_bias(C, sB + (l + 1) * HID, lane);
        layer64(C, A, sW + woff[l], lane);
    }
    uint32_t A[4][4];
    c_to_a<true>(C, A);
    if constexpr (TRAIN) {
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) zsave[3 * 32 + nt * 4 + q] = C[nt][q];
        float H[8][4];
        a_to_c(A, H);
        store_pairs(H, 8, hout[3], HID, lane);
    }
    float C5[4];
    {
        const int i = lane & 3;
        const float b0 = sB[4 * HID + 2 * i], b1 = sB[4 * HID + 2 * i + 1];
        C5[0] = b0; C5[1] = b1; C5[2] = b0; C5[3] = b1;
    }
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
        uint32_t b0, b1;
        load_b(sW + OFF_WT5, RSH, 0, kt, lane, b0, b1);
        mma16816(C5, A[kt][0], A[kt][1], A[kt][2], A[kt][3], b0, b1);
    }
    y0 = C5[0];
    y1 = C5[2];
}

// Inference forward pass of a 32-point tile (two m-tiles sharing every weight fragment): rows
// g, g+8 of tile 0 and g, g+8 of tile 1 come back in y[0..3] (valid in lanes with lane % 4 == 0).
__device__ __forceinline__ void mlp_forward32(const __nv_bfloat16* sW, const float* sB, const __nv_bfloat16* F, int lane,
                                              float (&y)[4]) {
    float C[2][8][4];
    init_bias(C[0], sB, lane);
    init_bias(C[1], sB, lane);
#pragma unroll 1
    for (int kt = 0; kt < KIN / 16; ++kt) {
        uint32_t a0[4], a1[4];
        load_a(F, RS1, kt, lane, a0);
        load_a(F + 16 * RS1, RS1, kt, lane, a1);
#pragma unroll
        for (int nt = 0; nt < 8; nt += 2) {
            uint32_t b[4];
            load_b2(sW + OFF_WT1, RS1, nt, kt, lane, b);
            mma16816(C[0][nt], a0[0], a0[1], a0[2], a0[3], b[0], b[1]);
            mma16816(C[1][nt], a1[0], a1[1], a1[2], a1[3], b[0], b[1]);
            mma16816(C[0][nt + 1], a0[0], a0[1], a0[2], a0[3], b[2], b[3]);
            mma16816(C[1][nt + 1], a1[0], a1[1], a1[2], a1[3], b[2], b[3]);
        }
    }
    const int woff[3] = {OFF_WT2, OFF_WT3, OFF_WT4};
#pragma unroll 1
    for (int l = 0; l < 3; ++l) {
        uint32_t A0[4][4], A1[4][4];
        c_to_a<true>(C[0], A0);
        c_to_a<true>(C[1], A1);
        init_bias(C[0], sB + (l + 1) * HID, lane);
        init_bias(C[1], sB + (l + 1) * HID, lane);
        const __nv_bfloat16* W = sW + woff[l];
#pragma unroll
        for (int kt = 0; kt < 4; ++kt)
#pragma unroll
            for (int nt = 0; nt < 8; nt += 2) {
                uint32_t b[4];
                load_b2(W, RSH, nt, kt, lane, b);
                mma16816(C[0][nt], A0[kt][0], A0[kt][1], A0[kt][2], A0[kt][3], b[0], b[1]);
                mma16816(C[1][nt], A1[kt][0], A1[kt][1], A1[kt][2], A1[kt][3], b[0], b[1]);
                mma16816(C[0][nt + 1], A0[kt][0], A0[kt][1], A0[kt][2], A0[kt][3], b[2], b[3]);
                mma16816(C[1][nt + 1], A1[kt][0], A1[kt][1], A1[kt][2], A1[kt][3], b[2], b[3]);
            }
    }
    uint32_t A0[4][4], A1[4][4];
    c_to_a<true>(C[0], A0);
    c_to_a<true>(C[1], A1);
    float C5[2][4];
    {
        const int i = lane & 3;
        const float b0 = sB[4 * HID + 2 * i], b1 = sB[4 * HID + 2 * i + 1];
#pragma unroll
        for (int t = 0; t < 2; ++t) { C5[t][0] = b0; C5[t][1] = b1; C5[t][2] = b0; C5[t][3] = b1; }
    }
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
        uint32_t b0, b1;
        load_b(sW + OFF_WT5, RSH, 0, kt, lane, b0, b1);
        mma16816(C5[0], A0[kt][0], A0[kt][1], A0[kt][2], A0[kt][3], b0, b1);
        mma16816(C5[1], A1[kt][0], A1[kt][1], A1[kt][2], A1[kt][3], b0, b1);
    }
    y[0] = C5[0][0]; y[1] = C5[0][2]; y[2] = C5[1][0]; y[3] = C5[1][2];
}

template <int WORDS>
__device__ __forceinline__ void stage_weights(uint4* dst, const __nv_bfloat16* wbf, float* sB, const float* bias) {
    const uint4* src = reinterpret_cast<const uint4*>(wbf);
    for (int k = threadIdx.x; k < WORDS; k += blockDim.x) dst[k] = src[k];
    for (int k = threadIdx.x; k < NBIAS; k += blockDim.x) sB[k] = bias[k];
}

constexpr int FWD_U4 = WBF_FWD * 2 / 16;
constexpr int ALL_U4 = WBF_ALL * 2 / 16;
static_assert(WBF_FWD * 2 % 16 == 0 && WBF_ALL * 2 % 16 == 0, "weight blocks are copied as uint4");
constexpr int TILE_BYTES = 16 * RS1 * 2;
constexpr int QUERY_WARPS = 4;
constexpr size_t QUERY_SMEM = (size_t)WBF_FWD * 2 + NBIAS * 4 + QUERY_WARPS * 2 * TILE_BYTES;
constexpr int TRAIN_WARPS = 4;
constexpr size_t TRAIN_SMEM = (size_t)WBF_ALL * 2 + NBIAS * 4 + TRAIN_WARPS * (TILE_BYTES + 4 * 32 * 32 * 4);

// ------------------------------------------------------------------------------------------ query
template <bool SAMPLES>
__global__ void __launch_bounds__(QUERY_WARPS * 32) k_nsdf_query(const __nv_bfloat16* __restrict__ wbf,
                                                                 const float* __restrict__ bias, Frame fr,
                                                                 const float4* __restrict__ pts,
                                                                 const Sample* __restrict__ samples, int count, Pose pose,
                                                                 float* __restrict__ out) {
    extern __shared__ uint4 smem_q[];
    __nv_bfloat16* sW = reinterpret_cast<__nv_bfloat16*>(smem_q);
    float* sB = reinterpret_cast<float*>(sW + WBF_FWD);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __nv_bfloat16* sF = reinterpret_cast<__nv_bfloat16*>(sB + NBIAS) + warp * 32 * RS1;
    stage_weights<FWD_U4>(smem_q, wbf, sB, bias);
    __syncthreads();
    const int g = lane >> 2, i = lane & 3;
    const int nw = gridDim.x * QUERY_WARPS;
    for (int tile = blockIdx.x * QUERY_WARPS + warp; tile * 32 < count; tile += nw) {
        const int idx = tile * 32 + lane;
        const bool valid = idx < count;
        float px = 0.f, py = 0.f, pz = 0.f, a0 = pose.a0, a1 = pose.a1, a2 = pose.a2;
        if (valid) {
            if constexpr (SAMPLES) {
                const Sample S = samples[idx];
                px = S.x; py = S.y; pz = S.z; a0 = S.p0; a1 = S.p1; a2 = S.p2;
            } else {
                const float4 P = pts[idx];
                px = P.x; py = P.y; pz = P.z;
            }
        }
        const float ux = (px - fr.cx) * fr.ihx, uy = (py - fr.cy) * fr.ihy, uz = (pz - fr.cz) * fr.ihz;
        write_features(sF, lane, 0, ux, uy, uz, a0 * fr.poseScale, a1 * fr.poseScale, a2 * fr.poseScale, valid);
        write_features(sF, lane, 1, ux, uy, uz, a0 * fr.poseScale, a1 * fr.poseScale, a2 * fr.poseScale, valid);
        __syncwarp();
        float y[4];
        mlp_forward32(sW, sB, sF, lane, y);
        __syncwarp();
        if (i == 0) {
            const float sc = SAMPLES ? 1.0f : fr.cell;
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int row = tile * 32 + (r >> 1) * 16 + g + 8 * (r & 1);
                if (row < count) out[row] = y[r] * sc;
            }
        }
    }
}

// ------------------------------------------------------------------------------------------ training
// One minibatch: forward with saved activations, loss, backward to every layer's pre-activation
// gradient.  Activations and gradients go to `acts` in the pair layout for k_nsdf_wgrad:
//   H0 [B/2][KIN], H1..H4 [B/2][64], dZ1..dZ4 [B/2][64], dZ5 [B/2][8]   (32-bit words).
__global__ void __launch_bounds__(TRAIN_WARPS * 32) k_nsdf_train(const __nv_bfloat16* __restrict__ wbf,
                                                                 const float* __restrict__ bias, Frame fr,
                                                                 const Sample* __restrict__ pool, long long poolSize,
                                                                 int batch, uint32_t seed, uint32_t* __restrict__ acts,
                                                                 float* __restrict__ lossSum) {
    extern __shared__ uint4 smem_t[];
    __nv_bfloat16* sW = reinterpret_cast<__nv_bfloat16*>(smem_t);
    float* sB = reinterpret_cast<float*>(sW + WBF_ALL);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __nv_bfloat16* sF = reinterpret_cast<__nv_bfloat16*>(sB + NBIAS) + warp * 16 * RS1;
    float* sZ = reinterpret_cast<float*>(reinterpret_cast<__nv_bfloat16*>(sB + NBIAS) + TRAIN_WARPS * 16 * RS1) +
                warp * (4 * 32 * 32) + lane * 128;
    stage_weights<ALL_U4>(smem_t, wbf, sB, bias);
    __syncthreads();

    const long long B2 = batch / 2;
    uint32_t* H0 = acts;
    uint32_t* Hl[4] = {H0 + B2 * KIN, H0 + B2 * KIN + B2 * HID, H0 + B2 * KIN + 2 * B2 * HID, H0 + B2 * KIN + 3 * B2 * HID};
    uint32_t* dZ[4] = {Hl[3] + B2 * HID, Hl[3] + 2 * B2 * HID, Hl[3] + 3 * B2 * HID, Hl[3] + 4 * B2 * HID};
    uint32_t* dZ5 = dZ[3] + B2 * HID;

    const int s = lane >> 1, half = lane & 1, g = lane >> 2, i = lane & 3;
    const int nw = gridDim.x * TRAIN_WARPS;
    float lossAcc = 0.f;
    for (int tile = blockIdx.x * TRAIN_WARPS + warp; tile * 16 < batch; tile += nw) {
        const int b = tile * 16 + s;
        const uint32_t h = hash32(seed ^ hash32((uint32_t)b * 2654435761u));
        const long long idx = (long long)(((unsigned long long)h * (unsigned long long)poolSize) >> 32);
        const Sample S = pool[idx];
        write_features(sF, s, half, (S.x - fr.cx) * fr.ihx, (S.y - fr.cy) * fr.ihy, (S.z - fr.cz) * fr.ihz,
                       S.p0 * fr.poseScale, S.p1 * fr.poseScale, S.p2 * fr.poseScale, true);
        __syncwarp();
        // H0 in the pair layout
        uint32_t* h0 = H0 + (long long)tile * 8 * KIN;
        for (int w = lane; w < 8 * KIN; w += 32) {
            const int p = w / KIN, f = w - p * KIN;
            const __nv_bfloat16 lo = sF[(2 * p) * RS1 + f], hi = sF[(2 * p + 1) * RS1 + f];
            __nv_bfloat162 v; v.x = lo; v.y = hi;
            h0[w] = *reinterpret_cast<uint32_t*>(&v);
        }
        uint32_t* hout[4] = {Hl[0] + (long long)tile * 8 * HID, Hl[1] + (long long)tile * 8 * HID,
                             Hl[2] + (long long)tile * 8 * HID, Hl[3] + (long long)tile * 8 * HID};
        float y0, y1;
        mlp_forward<true>(sW, sB, sF, lane, sZ, hout, y0, y1);
        __syncwarp();
        // targets and weights of rows g, g+8 live in lanes 2g(+1), 2(g+8)
        const float t0 = __shfl_sync(0xffffffffu, S.target, 2 * g), t1 = __shfl_sync(0xffffffffu, S.target, 2 * (g + 8));
        const float w0 = __shfl_sync(0xffffffffu, S.weight, 2 * g), w1 = __shfl_sync(0xffffffffu, S.weight, 2 * (g + 8));
        y0 = __shfl_sync(0xffffffffu, y0, lane & ~3);
        y1 = __shfl_sync(0xffffffffu, y1, lane & ~3);
        const float e0 = y0 - t0, e1 = y1 - t1;
        if (i == 0) lossAcc += w0 * e0 * e0 + w1 * e1 * e1;
        const float inv = 1.0f / (float)batch;
        const float dy0 = 2.0f * w0 * e0 * inv, dy1 = 2.0f * w1 * e1 * inv;
        float D[8][4];
        // dZ5 (column 0 only)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) D[nt][q] = 0.f;
        if (i == 0) { D[0][0] = dy0; D[0][2] = dy1; }
        store_pairs(D, 1, dZ5 + (long long)tile * 8 * OUTN, OUTN, lane);
        // dH4 = dy * W5[:, 0], then through SiLU
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int n0 = nt * 8 + 2 * i;
            const float w50 = __bfloat162float(sW[OFF_WT5 + n0]), w51 = __bfloat162float(sW[OFF_WT5 + n0 + 1]);
            D[nt][0] = dy0 * w50 * silu_grad(sZ[3 * 32 + nt * 4 + 0]);
            D[nt][1] = dy0 * w51 * silu_grad(sZ[3 * 32 + nt * 4 + 1]);
            D[nt][2] = dy1 * w50 * silu_grad(sZ[3 * 32 + nt * 4 + 2]);
            D[nt][3] = dy1 * w51 * silu_grad(sZ[3 * 32 + nt * 4 + 3]);
        }
        const int wn[3] = {OFF_WN4, OFF_WN3, OFF_WN2};
#pragma unroll 1
        for (int l = 3; l >= 1; --l) {   // D = dZ of layer l+1 (1-based); produce dZ of layer l
            store_pairs(D, 8, dZ[l] + (long long)tile * 8 * HID, HID, lane);
            uint32_t A[4][4];
            c_to_a<false>(D, A);
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
#pragma unroll
                for (int q = 0; q < 4; ++q) D[nt][q] = 0.f;
            layer64(D, A, sW + wn[3 - l], lane);
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
#pragma unroll
                for (int q = 0; q < 4; ++q) D[nt][q] *= silu_grad(sZ[(l - 1) * 32 + nt * 4 + q]);
        }
        store_pairs(D, 8, dZ[0] + (long long)tile * 8 * HID, HID, lane);
        __syncwarp();
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lossAcc += __shfl_xor_sync(0xffffffffu, lossAcc, o);
    if (lane == 0) atomicAdd(lossSum, lossAcc);
}

// Weight and bias gradients, all five layers in one launch: dW_l = H_{l-1}^T dZ_l, db_l = 1^T dZ_l,
// summed over the batch.  A warp owns one 16-row tile of one layer (the last tile of a layer is the
// bias row) for one chunk of samples, and adds its sums into `grads` (parameter layout).
constexpr int WG_CHUNK = 512;
__global__ void __launch_bounds__(128) k_nsdf_wgrad(const uint32_t* __restrict__ acts, int batch, float* __restrict__ grads) {
    const int warpGlobal = blockIdx.x * 4 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    const int chunks = batch / WG_CHUNK;
    // jobs: layer 1 has 7 + 1 row tiles, layers 2..5 have 4 + 1
    const int tilesPerChunk = 8 + 4 * 5;
    if (warpGlobal >= tilesPerChunk * chunks) return;
    const int chunk = warpGlobal / tilesPerChunk;
    int job = warpGlobal - chunk * tilesPerChunk;
    int layer, mt;
    if (job < 8) { layer = 1; mt = job; } else { job -= 8; layer = 2 + job / 5; mt = job % 5; }
    const long long B2 = batch / 2;
    const uint32_t* H0 = acts;
    const uint32_t* Hprev;
    const uint32_t* dZ;
    int Fin, Fout, pW, pB;
    const uint32_t* Hl1 = H0 + B2 * KIN;
    const uint32_t* dZ1 = Hl1 + 4 * B2 * HID;
    switch (layer) {
        case 1: Hprev = H0; Fin = KIN; dZ = dZ1; Fout = HID; pW = P_W1; pB = P_B1; break;
        case 2: Hprev = Hl1; Fin = HID; dZ = dZ1 + B2 * HID; Fout = HID; pW = P_W2; pB = P_B2; break;
        case 3: Hprev = Hl1 + B2 * HID; Fin = HID; dZ = dZ1 + 2 * B2 * HID; Fout = HID; pW = P_W3; pB = P_B3; break;
        case 4: Hprev = Hl1 + 2 * B2 * HID; Fin = HID; dZ = dZ1 + 3 * B2 * HID; Fout = HID; pW = P_W4; pB = P_B4; break;
        default: Hprev = Hl1 + 3 * B2 * HID; Fin = HID; dZ = dZ1 + 4 * B2 * HID; Fout = OUTN; pW = P_W5; pB = P_B5; break;
    }
    const bool biasTile = mt == Fin / 16;
    const int ntiles = Fout / 8;
    const int g = lane >> 2, i = lane & 3;
    float C[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) C[nt][q] = 0.f;
    const uint32_t one2 = pack_bf16(1.0f, 1.0f);
    for (int k0 = chunk * WG_CHUNK; k0 < (chunk + 1) * WG_CHUNK; k0 += 16) {
        const long long p0 = k0 / 2 + i, p1 = p0 + 4;   // sample pairs of k rows 2i.. and 2i+8..
        uint32_t a0, a1, a2, a3;
        if (biasTile) {
            a0 = g == 0 ? one2 : 0u; a1 = 0u; a2 = g == 0 ? one2 : 0u; a3 = 0u;
        } else {
            const int f = mt * 16 + g;
            a0 = Hprev[p0 * Fin + f];
            a1 = Hprev[p0 * Fin + f + 8];
            a2 = Hprev[p1 * Fin + f];
            a3 = Hprev[p1 * Fin + f + 8];
        }
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            if (nt >= ntiles) break;
            const uint32_t b0 = dZ[p0 * Fout + nt * 8 + g], b1 = dZ[p1 * Fout + nt * 8 + g];
            mma16816(C[nt], a0, a1, a2, a3, b0, b1);
        }
    }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        if (nt >= ntiles) break;
        const int n0 = nt * 8 + 2 * i;
        if (biasTile) {
            if (g == 0) { atomicAdd(grads + pB + n0, C[nt][0]); atomicAdd(grads + pB + n0 + 1, C[nt][1]); }
        } else {
            const int m0 = mt * 16 + g;
            atomicAdd(grads + pW + m0 * Fout + n0, C[nt][0]);
            atomicAdd(grads + pW + m0 * Fout + n0 + 1, C[nt][1]);
            atomicAdd(grads + pW + (m0 + 8) * Fout + n0, C[nt][2]);
            atomicAdd(grads + pW + (m0 + 8) * Fout + n0 + 1, C[nt][3]);
        }
    }
}

// Parameter p's places in the bf16 weight block / bias vector.
__device__ __forceinline__ void publish(int p, float w, __nv_bfloat16* wbf, float* bias) {
    const __nv_bfloat16 b = __float2bfloat16(w);
    if (p < P_B1) {
        const int in = p / HID, out = p % HID;
        wbf[OFF_WT1 + out * RS1 + in] = b;
    } else if (p < P_W2) {
        bias[p - P_B1] = w;
    } else if (p < P_B4 + HID) {
        const int l = (p - P_W2) / (HID * HID + HID);           // 0..2 for W2..W4 (+ biases)
        const int r = (p - P_W2) - l * (HID * HID + HID);
        if (r < HID * HID) {
            const int in = r / HID, out = r % HID;
            const int wt = l == 0 ? OFF_WT2 : (l == 1 ? OFF_WT3 : OFF_WT4);
            const int wn = l == 0 ? OFF_WN2 : (l == 1 ? OFF_WN3 : OFF_WN4);
            wbf[wt + out * RSH + in] = b;
            wbf[wn + in * RSH + out] = b;
        } else {
            bias[(l + 1) * HID + (r - HID * HID)] = w;
        }
    } else if (p < P_B5) {
        const int in = (p - P_W5) / OUTN, out = (p - P_W5) % OUTN;
        wbf[OFF_WT5 + out * RSH + in] = b;
    } else {
        bias[4 * HID + (p - P_B5)] = w;
    }
}

// Adam (Kingma & Ba 2015) on the fp32 master parameters, then the bf16 / bias copies the kernels read.
__global__ void k_nsdf_adam(float* __restrict__ params, const float* __restrict__ grads, float* __restrict__ m,
                            float* __restrict__ v, int step, float lr, float gradScale, __nv_bfloat16* __restrict__ wbf,
                            float* __restrict__ bias) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NPARAM) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    float w = params[p];
    if (step > 0) {
        const float gr = grads[p] * gradScale;
        const float mm = b1 * m[p] + (1.0f - b1) * gr;
        const float vv = b2 * v[p] + (1.0f - b2) * gr * gr;
        m[p] = mm; v[p] = vv;
        const float mh = mm / (1.0f - powf(b1, (float)step)), vh = vv / (1.0f - powf(b2, (float)step));
        w -= lr * mh / (sqrtf(vh) + eps);
        // the padding rows of the first layer and the unused output columns stay zero
        const bool pad = (p < P_B1 && p / HID >= NFEAT) || (p >= P_W5 && p < P_B5 && (p - P_W5) % OUTN != 0) ||
                         (p >= P_B5 && p != P_B5);
        if (pad) w = 0.f;
        params[p] = w;
    }
    publish(p, w, wbf, bias);
}

// Uniform fan-in initialisation (He-style bound for SiLU), zero biases and padding.
__global__ void k_nsdf_init(float* __restrict__ params, uint32_t seed) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NPARAM) return;
    float w = 0.f;
    int fanIn = 0;
    if (p < P_B1) fanIn = p / HID < NFEAT ? NFEAT : 0;
    else if (p >= P_W2 && p < P_B4 + HID && ((p - P_W2) % (HID * HID + HID)) < HID * HID) fanIn = HID;
    else if (p >= P_W5 && p < P_B5 && (p - P_W5) % OUTN == 0) fanIn = HID;
    if (fanIn > 0) w = (2.0f * u01(hash32(seed ^ hash32((uint32_t)p))) - 1.0f) * sqrtf(6.0f / (float)fanIn);
    params[p] = w;
}

// ------------------------------------------------------------------------------------------ samples
__global__ void k_nsdf_sample(const float4* __restrict__ mesh, int nverts, const float* __restrict__ grid, SdfGrid g,
                              float band, float sigma, float3 sc, float sr, Pose pose, int count, uint32_t seed,
                              Sample* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    uint32_t h = hash32(seed ^ hash32((uint32_t)t * 0x9E3779B9u));
    auto next = [&]() { h = hash32(h + 0x6D2B79F5u); return u01(h); };
    float3 p;
    if (next() < 0.75f) {   // near the surface: a mesh vertex, moved along its normal and sideways
        const int v = min(nverts - 1, (int)(next() * (float)nverts));
        const float4 pos = mesh[2 * v], nrm = mesh[2 * v + 1];
        const float u1 = fmaxf(next(), 1e-7f), u2 = next(), u3 = fmaxf(next(), 1e-7f), u4 = next();
        const float r1 = sqrtf(-2.0f * __logf(u1)), r2 = sqrtf(-2.0f * __logf(u3));
        const float n0 = r1 * __cosf(6.2831853f * u2), n1 = r1 * __sinf(6.2831853f * u2), n2 = r2 * __cosf(6.2831853f * u4);
        const float along = n0 * sigma;
        p = mk3(pos.x + nrm.x * along + n1 * 0.5f * sigma, pos.y + nrm.y * along + n2 * 0.5f * sigma,
                pos.z + nrm.z * along + (n1 - n2) * 0.35f * sigma);
    } else {                // anywhere in the grid box
        p = mk3(g.ox + next() * g.nx * g.cell, g.oy + next() * g.ny * g.cell, g.oz + next() * g.nz * g.cell);
    }
    const float d = sdf_lookup(grid, g, p);
    Sample S;
    S.x = p.x; S.y = p.y; S.z = p.z;
    S.p0 = pose.a0; S.p1 = pose.a1; S.p2 = pose.a2;
    if (d == 1e10f) {
        const float dx = p.x - sc.x, dy = p.y - sc.y, dz = p.z - sc.z;
        const bool outside = dx * dx + dy * dy + dz * dz > sr * sr;
        S.target = band;
        S.weight = outside ? 1.0f : 0.0f;
    } else {
        S.target = fminf(fmaxf(d / g.cell, -band), band);
        S.weight = 1.0f;
    }
    out[t] = S;
}

}  // namespace

size_t acts_elements(int batch) { return (size_t)batch * (KIN + 8 * HID + OUTN); }

cudaError_t launch_query(const __nv_bfloat16* wbf, const float* bias, const Frame& fr, const float4* points, int count,
                         Pose pose, float* out, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k_nsdf_query<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)QUERY_SMEM);
    if (e != cudaSuccess) return e;
    const int tiles = (count + 31) / 32;
    const int blocks = std::min((tiles + QUERY_WARPS - 1) / QUERY_WARPS, sm_count() * 8);
    k_nsdf_query<false><<<blocks, QUERY_WARPS * 32, QUERY_SMEM, s>>>(wbf, bias, fr, points, nullptr, count, pose, out);
    return cudaGetLastError();
}

cudaError_t launch_query_samples(const __nv_bfloat16* wbf, const float* bias, const Frame& fr, const Sample* samples,
                                 int count, float* out, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k_nsdf_query<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)QUERY_SMEM);
    if (e != cudaSuccess) return e;
    const int tiles = (count + 31) / 32;
    const int blocks = std::min((tiles + QUERY_WARPS - 1) / QUERY_WARPS, sm_count() * 8);
    k_nsdf_query<true><<<blocks, QUERY_WARPS * 32, QUERY_SMEM, s>>>(wbf, bias, fr, nullptr, samples, count, Pose{0, 0, 0},
                                                                    out);
    return cudaGetLastError();
}

cudaError_t launch_train_step(const __nv_bfloat16* wbf, const float* bias, const Frame& fr, const Sample* pool,
                              long long poolSize, int batch, uint32_t seed, __nv_bfloat16* acts, float* grads,
                              float* lossSum, cudaStream_t s) {
    if (batch <= 0 || batch % WG_CHUNK != 0 || poolSize <= 0) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(k_nsdf_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TRAIN_SMEM);
    if (e != cudaSuccess) return e;
    const int tiles = batch / 16;
    const int blocks = std::min((tiles + TRAIN_WARPS - 1) / TRAIN_WARPS, sm_count() * 2);
    k_nsdf_train<<<blocks, TRAIN_WARPS * 32, TRAIN_SMEM, s>>>(wbf, bias, fr, pool, poolSize, batch, seed,
                                                             reinterpret_cast<uint32_t*>(acts), lossSum);
    e = cudaMemsetAsync(grads, 0, sizeof(float) * NPARAM, s);
    if (e != cudaSuccess) return e;
    const int warps = (batch / WG_CHUNK) * (8 + 4 * 5);
    k_nsdf_wgrad<<<(warps + 3) / 4, 128, 0, s>>>(reinterpret_cast<const uint32_t*>(acts), batch, grads);
    return cudaGetLastError();
}

cudaError_t launch_adam(float* params, const float* grads, float* m, float* v, int step, float lr, float gradScale,
                        __nv_bfloat16* wbf, float* bias, cudaStream_t s) {
    k_nsdf_adam<<<(NPARAM + 255) / 256, 256, 0, s>>>(params, grads, m, v, step, lr, gradScale, wbf, bias);
    return cudaGetLastError();
}

cudaError_t launch_init_params(float* params, uint32_t seed, __nv_bfloat16* wbf, float* bias, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(wbf, 0, sizeof(__nv_bfloat16) * WBF_ALL, s);
    if (e != cudaSuccess) return e;
    k_nsdf_init<<<(NPARAM + 255) / 256, 256, 0, s>>>(params, seed);
    k_nsdf_adam<<<(NPARAM + 255) / 256, 256, 0, s>>>(params, nullptr, nullptr, nullptr, 0, 0.f, 0.f, wbf, bias);
    return cudaGetLastError();
}

cudaError_t launch_sample(const float4* mesh, int nverts, const float* grid, const SdfGrid& g, float band, float sigma,
                          float3 sphereCentre, float sphereRadius, Pose pose, int count, uint32_t seed, Sample* out,
                          cudaStream_t s) {
    if (count <= 0 || nverts <= 0) return cudaSuccess;
    k_nsdf_sample<<<(count + 255) / 256, 256, 0, s>>>(mesh, nverts, grid, g, band, sigma, sphereCentre, sphereRadius, pose,
                                                      count, seed, out);
    return cudaGetLastError();
}

}  // namespace nsdf
}  // namespace tfx

// ================================================================================================
// collision with the proxy
namespace tfx {
namespace nsdf {
namespace {

__device__ __forceinline__ void mark_block(uint32_t* marks, const SdfGrid& g, int3 c) {
    for (int dz = 0; dz < 3; ++dz)
        for (int dy = 0; dy < 3; ++dy)
            for (int dx = 0; dx < 3; ++dx) {
                const int x = c.x + dx, y = c.y + dy, z = c.z + dz;
                if (x < 0 || y < 0 || z < 0 || x >= g.nx || y >= g.ny || z >= g.nz) continue;
                const long long cell = ((long long)z * g.ny + y) * g.nx + x;
                atomicOr(marks + (cell >> 5), 1u << (cell & 31));
            }
}

__global__ void __launch_bounds__(QUERY_WARPS * 32) k_nsdf_classify(CollideArgs a) {
    extern __shared__ uint4 smem_c[];
    __nv_bfloat16* sW = reinterpret_cast<__nv_bfloat16*>(smem_c);
    float* sB = reinterpret_cast<float*>(sW + WBF_FWD);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __nv_bfloat16* sF = reinterpret_cast<__nv_bfloat16*>(sB + NBIAS) + warp * 32 * RS1;
    stage_weights<FWD_U4>(smem_c, a.wbf, sB, a.bias);
    __syncthreads();
    const Frame fr = a.fr;
    const int g = lane >> 2, i = lane & 3;
    const long long nw = (long long)gridDim.x * QUERY_WARPS;
    const float limit = a.margin / fr.cell + a.slackCells;   // band: network distance below margin + slack
    for (long long tile = (long long)blockIdx.x * QUERY_WARPS + warp; tile * 32 < a.vtot; tile += nw) {
        const long long v = tile * 32 + lane;
        const bool valid = v < a.vtot;
        const float4 P = valid ? a.pos[v] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float ux = (P.x - fr.cx) * fr.ihx, uy = (P.y - fr.cy) * fr.ihy, uz = (P.z - fr.cz) * fr.ihz;
        const float p0 = a.pose.a0 * fr.poseScale, p1 = a.pose.a1 * fr.poseScale, p2 = a.pose.a2 * fr.poseScale;
        write_features(sF, lane, 0, ux, uy, uz, p0, p1, p2, valid);
        write_features(sF, lane, 1, ux, uy, uz, p0, p1, p2, valid);
        __syncwarp();
        float y[4];
        mlp_forward32(sW, sB, sF, lane, y);
        __syncwarp();
        if (i == 0) {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const long long vr = tile * 32 + (r >> 1) * 16 + g + 8 * (r & 1);
                if (vr >= a.vtot || (int)(vr % a.n) < 2 || !(y[r] < limit)) continue;
                a.bandList[atomicAdd(a.bandCount, 1)] = (int)vr;
                const float4 pv = a.pos[vr];
                mark_block(a.marks, a.grid, sdf_coords(a.grid, mk3(pv.x, pv.y, pv.z)));
            }
        }
    }
}

// Words of the per-cell marks (the coarse map of 4x4x4-cell blocks follows them).
__host__ __device__ __forceinline__ long long mark_words(long long cells) { return (cells + 31) / 32; }
__host__ __device__ __forceinline__ int coarse_dim(int n) { return (n + 3) >> 2; }

// The words' initial value, and the coarse map: the block of every marked cell.
__global__ void __launch_bounds__(256) k_gated_init(uint32_t* __restrict__ w, const uint32_t* __restrict__ marks,
                                                    uint32_t* __restrict__ coarse, SdfGrid g, const int* __restrict__ count) {
    if (*count == 0) return;
    const uint32_t v = float_flip3(1e10f);
    const long long cells = (long long)g.nx * g.ny * g.nz;
    const int cbx = coarse_dim(g.nx), cby = coarse_dim(g.ny);
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < cells; c += (long long)gridDim.x * blockDim.x) {
        w[c] = v;
        if ((__ldg(marks + (c >> 5)) >> (c & 31)) & 1u) {
            const long long nxy = (long long)g.nx * g.ny;
            const int z = (int)(c / nxy);
            const long long r = c - (long long)z * nxy;
            const int y = (int)(r / g.nx), x = (int)(r - (long long)y * g.nx);
            const int b = ((z >> 2) * cby + (y >> 2)) * cbx + (x >> 2);
            atomicOr(coarse + (b >> 5), 1u << (b & 31));
        }
    }
}

// ConstructSignedDistanceField (TressFXSDFCollision.hlsl:329-397) restricted to marked cells: every
// (triangle, cell) pair of a marked cell is evaluated, so each marked cell gets its exact value.  A
// warp takes a triangle, its lanes test the 4x4x4-cell blocks the reference's cell box overlaps, and a
// triangle whose box holds no marked cell is left at once (it contributes to no marked cell).  Box
// coordinates use the float reciprocal only below 2^22 cells, where it gives the integer quotient
// (as in the full construct).
__global__ void __launch_bounds__(256) k_gated_construct(CollideArgs a) {
    if (*a.bandCount == 0) return;
    const SdfGrid g = a.grid;
    const int lane = threadIdx.x & 31;
    const int warpsTotal = gridDim.x * (blockDim.x >> 5);
    const long long cells = (long long)g.nx * g.ny * g.nz;
    const uint32_t* coarse = a.marks + mark_words(cells);
    const int cbx = coarse_dim(g.nx), cby = coarse_dim(g.ny);
    for (int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < a.ntri; t += warpsTotal) {
        const float3 x0 = xyz(__ldg(a.mesh + 2 * (size_t)__ldg(a.indices + 3 * t + 0)));
        const float3 x1 = xyz(__ldg(a.mesh + 2 * (size_t)__ldg(a.indices + 3 * t + 1)));
        const float3 x2 = xyz(__ldg(a.mesh + 2 * (size_t)__ldg(a.indices + 3 * t + 2)));
        int3 lo, hi;
        tri_cell_box(g, x0, x1, x2, lo, hi);
        const int bx0 = lo.x >> 2, by0 = lo.y >> 2, bz0 = lo.z >> 2;
        const int nbx = (hi.x >> 2) - bx0 + 1, nby = (hi.y >> 2) - by0 + 1, nbz = (hi.z >> 2) - bz0 + 1;
        const int nb = nbx * nby * nbz;
        bool any = false;
        for (int k = lane; k < nb && !any; k += 32) {
            const int kz = k / (nbx * nby), kr = k - kz * nbx * nby, ky = kr / nbx, kx = kr - ky * nbx;
            const int b = ((bz0 + kz) * cby + (by0 + ky)) * cbx + (bx0 + kx);
            any = (__ldg(coarse + (b >> 5)) >> (b & 31)) & 1u;
        }
        if (!__any_sync(0xffffffffu, any)) continue;
        const int nx = hi.x - lo.x + 1, ny = hi.y - lo.y + 1, nz = hi.z - lo.z + 1;
        const int nxy = nx * ny, vol = nxy * nz;
        const bool floatIdx = vol < (1 << 22);
        const float inxy = 1.0f / (float)nxy, inx = 1.0f / (float)nx;
        const TriPre P = tri_pre(x0, x1, x2);
        for (int c = lane; c < vol; c += 32) {
            int cz, r, cy;
            if (floatIdx) {
                cz = (int)(((float)c + 0.5f) * inxy);
                r = c - cz * nxy;
                cy = (int)(((float)r + 0.5f) * inx);
            } else {
                cz = c / nxy;
                r = c - cz * nxy;
                cy = r / nx;
            }
            const int x = lo.x + (r - cy * nx), y = lo.y + cy, z = lo.z + cz;
            const long long cell = ((long long)z * g.ny + y) * g.nx + x;
            if (!((__ldg(a.marks + (cell >> 5)) >> (cell & 31)) & 1u)) continue;
            atomicMin(a.words + cell, float_flip3(signed_dist_pre(sdf_cell_pos(g, x, y, z), P)));
        }
    }
}

__global__ void __launch_bounds__(256) k_gated_finalize(uint32_t* __restrict__ w, long long cells, const int* __restrict__ count) {
    if (*count == 0) return;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < cells; c += (long long)gridDim.x * blockDim.x)
        w[c] = ifloat_flip3(w[c]);
}

__global__ void __launch_bounds__(256) k_band_collide(CollideArgs a) {
    const int cnt = *a.bandCount;
    const float* sdf = reinterpret_cast<const float*>(a.words);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x) {
        const int v = a.bandList[k];
        const float4 p = a.pos[v];
        float3 proj;
        if (sdf_collide_point(sdf, a.grid, a.margin, xyz(p), proj)) {
            a.pos[v] = with_xyz(p, proj);
            a.prev[v] = with_xyz(a.prev[v], proj);
        }
    }
}

}  // namespace

cudaError_t launch_collide(const CollideArgs& a, cudaStream_t s) {
    if (a.vtot <= 0) return cudaSuccess;
    const long long cells = (long long)a.grid.nx * a.grid.ny * a.grid.nz;
    cudaError_t e = cudaMemsetAsync(a.bandCount, 0, sizeof(int), s);
    const long long coarseBits = (long long)coarse_dim(a.grid.nx) * coarse_dim(a.grid.ny) * coarse_dim(a.grid.nz);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(a.marks, 0, sizeof(uint32_t) * (size_t)(mark_words(cells) + (coarseBits + 31) / 32), s);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_nsdf_classify, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)QUERY_SMEM);
    if (e != cudaSuccess) return e;
    if (a.wtc) {   // the network on the tcgen05 path
        TcArgs t{};
        t.wtc = a.wtc; t.fr = a.fr; t.pose = a.pose; t.pts = a.pos; t.err = a.err;
        t.vtot = a.vtot; t.n = a.n; t.margin = a.margin; t.slackCells = a.slackCells; t.grid = a.grid;
        t.bandList = a.bandList; t.bandCount = a.bandCount; t.marks = a.marks;
        e = launch_classify_tc(t, s);
        if (e != cudaSuccess) return e;
    } else {
        const long long tiles = (a.vtot + 31) / 32;
        const int blocks = (int)std::min<long long>((tiles + QUERY_WARPS - 1) / QUERY_WARPS, sm_count() * 8);
        k_nsdf_classify<<<blocks, QUERY_WARPS * 32, QUERY_SMEM, s>>>(a);
    }
    const unsigned gc = (unsigned)std::min<long long>((cells + 255) / 256, (long long)sm_count() * 16);
    k_gated_init<<<gc, 256, 0, s>>>(a.words, a.marks, a.marks + mark_words(cells), a.grid, a.bandCount);
    if (a.ntri > 0) k_gated_construct<<<(unsigned)std::min(( a.ntri + 7) / 8, sm_count() * 32), 256, 0, s>>>(a);
    k_gated_finalize<<<gc, 256, 0, s>>>(a.words, cells, a.bandCount);
    k_band_collide<<<sm_count() * 4, 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace nsdf
}  // namespace tfx
