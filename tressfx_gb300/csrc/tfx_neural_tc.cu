// Inference of the learned collision proxy (tfx_neural.cuh) on the fifth-generation tensor cores.
//
// A block holds the packed weights once in shared memory and runs TC_NWG warpgroups, each carrying
// its own tiles of 128 points through the network, so that one warpgroup's feature and activation
// arithmetic overlaps the other warpgroups' MMAs.  Both operands a warpgroup produces live in its
// 128 tensor-memory columns: the fp32 accumulator D (columns 0-63) and the bf16 A operand (columns
// 64-119, two bf16 per column, row r in lane r), so shared memory carries only the weights (the B
// operands).  In a warpgroup, thread r computes point r's 102 features and stores them as row r of A
// (tcgen05.st); one thread issues the layer's tcgen05.mma (kind::f16, A from tensor memory, B from
// shared memory, bf16 x bf16 -> f32, M = 128 points, N = 64 neurons, K = 16 per instruction);
// tcgen05.commit signals the warpgroup's mbarrier when the layer's MMAs are done.  Thread r then reads
// row r of D (tcgen05.ld), applies SiLU and stores the bf16 activations as row r of the next layer's A.
// The output layer (64 -> 1) is one more MMA (N = 16, weights in column 0), read back as one column,
// plus the fp32 bias.  Each thread loads its point of the warpgroup's next tile while the current
// tile's layers run.  Warpgroups synchronise on their own named barriers (ids 1..TC_NWG).
//
// Weight layout (B, shared memory): K-major, no swizzle, 8-row x 16-byte core matrices; the core matrix
// of row group R and column group C of a matrix with K columns starts at byte (R * K / 8 + C) * 128, so
// the descriptor of a 16-column step has a leading-dimension offset (between the two column groups) of
// 128 bytes and a stride offset (between row groups) of K * 16 bytes.
//
// Numerics are those of the mma.sync path: weights and activations in bf16, fp32 accumulation,
// SiLU(z) = h + h tanh(h) with h = z / 2 evaluated as bf16 pairs with the hardware tanh, the output
// bias added in fp32.  Two differences: the factor 1/2 is folded into the packed hidden weights and
// biases (exact, a power of two), and the hidden biases enter through the MMA as two extra input
// columns of ones whose weights are the bias's bf16 high part and the bf16 rounding of the remainder
// (about 16 significant bits).
#include "tfx_bulk.cuh"
#include "tfx_neural.cuh"
#include "tfx_sdf_math.cuh"

namespace tfx {
namespace nsdf {

namespace {

constexpr int TC_M = 128;                  // points per tile
// layer 1 (K = TC_K1): 102 features, ones in columns 102 (bias high part) and 103 (remainder);
// layers 2-4 (K = TC_KH): 64 activations, ones in columns 64 and 65
constexpr int TC_COLS = 128;               // tensor-memory columns of a warpgroup: D at 0 (64), A at TC_ACOL
constexpr int TC_ACOL = 64;                // A: TC_K1 / 2 = 56 columns (layer 1), TC_KH / 2 = 40 (the others)
static_assert(TC_ACOL + TC_K1 / 2 <= TC_COLS, "the A operand does not fit beside the accumulator");
// tensor-memory columns a block allocates: a power of two >= 32 covering every warpgroup's columns
constexpr int TC_TMEM_COLS = TC_NWG * TC_COLS <= 32 ? 32 : TC_NWG * TC_COLS <= 64 ? 64 : TC_NWG * TC_COLS <= 128 ? 128
                             : TC_NWG * TC_COLS <= 256 ? 256 : 512;
static_assert(TC_NWG * TC_COLS <= 512, "the warpgroups' columns exceed the tensor memory of an SM");
// instruction descriptor of kind::f16 with bf16 A and B (K-major, no negation) and an f32 D, for N columns
constexpr uint32_t tc_idesc(int n) {
    return (1u << 4)                          // D format f32
           | (1u << 7)                        // A format bf16
           | (1u << 10)                       // B format bf16
           | ((uint32_t)(n >> 3) << 17)       // N / 8
           | ((uint32_t)(TC_M >> 4) << 24);   // M / 16
}
constexpr uint32_t TC_IDESC = tc_idesc(HID);
constexpr uint32_t TC_IDESC5 = tc_idesc(TC_N5);
constexpr int TC_WAIT_POLLS = 1 << 20;
constexpr uint32_t BF16_ONES = 0x3F803F80u;   // two bf16 1.0

__host__ __device__ constexpr int kmajor_off(int row, int k, int kt) {
    return (((row >> 3) * (kt >> 3) + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1);
}

// ---- PTX wrappers (tcgen05, sm_100 family)
__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(cols) : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_barrier_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// A from tensor memory (taddr), B from shared memory (descriptor)
__device__ __forceinline__ void tc_mma_ts(uint32_t dtmem, uint32_t atmem, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "r"(atmem), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
          "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr)
        : "memory");
}
__device__ __forceinline__ void tc_ld1(uint32_t taddr, uint32_t& v) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];" : "=r"(v) : "r"(taddr) : "memory");
}
// this warp's 32 lanes, N consecutive columns from taddr (thread i: lane i)
__device__ __forceinline__ void tc_st8(uint32_t taddr, const uint32_t* v) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr), "r"(v[0]),
                 "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
                 : "memory");
}
__device__ __forceinline__ void tc_st16(uint32_t taddr, const uint32_t* v) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16};" ::"r"(taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]), "r"(v[9]),
        "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
        : "memory");
}
__device__ __forceinline__ void tc_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// named barrier of the warpgroup (id 1 + wg; id 0 is __syncthreads)
__device__ __forceinline__ void wg_sync(int wg) { asm volatile("bar.sync %0, 128;" ::"r"(wg + 1) : "memory"); }
// barrier of the warpgroup that also ORs a predicate over its 128 threads
__device__ __forceinline__ bool wg_sync_or(int wg, bool p) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred q, o;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.or.pred o, %2, 128, q;\n\tselp.u32 %0, 1, 0, o;\n\t}\n"
        : "=r"(r)
        : "r"((uint32_t)p), "r"(wg + 1)
        : "memory");
    return r != 0;
}


// SiLU of a pair of accumulator words holding h = z / 2: h + h tanh(h), as a bf16 pair.
__device__ __forceinline__ uint32_t silu_half2(uint32_t x, uint32_t y) {
    __nv_bfloat162 h = __floats2bfloat162_rn(__uint_as_float(x), __uint_as_float(y));
    uint32_t t;
    asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t) : "r"(*reinterpret_cast<uint32_t*>(&h)));
    const __nv_bfloat162 r = __hfma2(h, *reinterpret_cast<__nv_bfloat162*>(&t), h);
    return *reinterpret_cast<const uint32_t*>(&r);
}

__device__ __forceinline__ uint32_t bf16_pair(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// sin(pi x), cos(pi x) with x reduced exactly to [-1, 1] (as the mma.sync path computes them).
__device__ __forceinline__ void sincospi_r(float x, float& s, float& c) {
    const float r = x - 2.0f * rintf(0.5f * x);
    const float a = 3.14159265358979f * r;
    s = __sinf(a);
    c = __cosf(a);
}

// The 112 input columns of one point as 56 bf16 pairs: xyz, pose, then (sin, cos) of pi f_k u_d for
// k = 0..15, d = 0..2 at columns 6 + 6k + 2d, the frequencies 2^(k/3) with f_{k+3} = 2 f_k from the
// double-angle formulas; ones in columns 102, 103 (the bias inputs); zeros after.
__device__ __forceinline__ void point_features(float ux, float uy, float uz, float p0, float p1, float p2, bool valid,
                                               uint32_t (&w)[56]) {
    const float f0 = 1.0f, f1 = 1.2599210498948732f, f2 = 1.5874010519681994f;   // 2^(0/3), 2^(1/3), 2^(2/3)
    w[0] = bf16_pair(valid ? ux : 0.f, valid ? uy : 0.f);
    w[1] = bf16_pair(valid ? uz : 0.f, valid ? p0 : 0.f);
    w[2] = bf16_pair(valid ? p1 : 0.f, valid ? p2 : 0.f);
    const float u[3] = {ux, uy, uz};
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const int k0 = half * 8;
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            // base frequency 2^((k0 + b) / 3), exact powers of two times 1, 2^(1/3) or 2^(2/3)
            const int kb = k0 + b;
            const float fb = (kb % 3 == 0 ? f0 : (kb % 3 == 1 ? f1 : f2)) * (float)(1 << (kb / 3));
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                float sn = 0.f, cs = 0.f;
                if (valid) sincospi_r(fb * u[d], sn, cs);
#pragma unroll
                for (int k = kb; k < k0 + 8; k += 3) {
                    w[3 + 3 * k + d] = bf16_pair(sn, cs);
                    const float s2 = 2.0f * sn * cs, c2 = 1.0f - 2.0f * sn * sn;
                    sn = s2;
                    cs = c2;
                }
            }
        }
    }
    w[51] = BF16_ONES;
#pragma unroll
    for (int k = 52; k < 56; ++k) w[k] = 0u;
}

__device__ __forceinline__ void mark_block_tc(uint32_t* marks, const SdfGrid& g, int3 c) {
    for (int dz = 0; dz < 3; ++dz)
        for (int dy = 0; dy < 3; ++dy)
            for (int dx = 0; dx < 3; ++dx) {
                const int x = c.x + dx, y = c.y + dy, z = c.z + dz;
                if (x < 0 || y < 0 || z < 0 || x >= g.nx || y >= g.ny || z >= g.nz) continue;
                const long long cell = ((long long)z * g.ny + y) * g.nx + x;
                atomicOr(marks + (cell >> 5), 1u << (cell & 31));
            }
}

}  // namespace

// Packed weights for the tensor-core forward pass from the fp32 master parameters: W1..W4 transposed
// into K-major bf16 operands with the halved bias as two extra input columns (high part, remainder),
// then w5 as the bf16 K-major operand of an N = 16 MMA (row 0) and b5 (fp32).
__global__ void k_nsdf_pack_tc(const float* __restrict__ params, uint8_t* __restrict__ wtc) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int n1 = HID * TC_K1, nh = HID * TC_KH;
    auto split = [](float x, int part) {   // part 0: bf16 of x; part 1: bf16 of the remainder
        const __nv_bfloat16 hi = __float2bfloat16(x);
        return part == 0 ? hi : __float2bfloat16(x - __bfloat162float(hi));
    };
    if (t < n1) {
        const int n = t / TC_K1, k = t - n * TC_K1;
        __nv_bfloat16 v = __float2bfloat16(0.f);
        if (k < NFEAT) v = __float2bfloat16(0.5f * params[P_W1 + k * HID + n]);
        else if (k == NFEAT || k == NFEAT + 1) v = split(0.5f * params[P_B1 + n], k - NFEAT);
        *reinterpret_cast<__nv_bfloat16*>(wtc + TC_OFF_W1 + kmajor_off(n, k, TC_K1)) = v;
        return;
    }
    int u = t - n1;
    if (u < 3 * nh) {
        const int l = u / nh, r = u - l * nh;
        const int n = r / TC_KH, k = r - n * TC_KH;
        const int pw = l == 0 ? P_W2 : (l == 1 ? P_W3 : P_W4), pb = l == 0 ? P_B2 : (l == 1 ? P_B3 : P_B4);
        __nv_bfloat16 v = __float2bfloat16(0.f);
        if (k < HID) v = __float2bfloat16(0.5f * params[pw + k * HID + n]);
        else if (k == HID || k == HID + 1) v = split(0.5f * params[pb + n], k - HID);
        *reinterpret_cast<__nv_bfloat16*>(wtc + TC_OFF_W2 + l * TC_WH_BYTES + kmajor_off(n, k, TC_KH)) = v;
        return;
    }
    u -= 3 * nh;
    if (u < TC_N5 * TC_KH) {   // row 0: bf16 w5 (as the mma.sync path rounds it); the other rows zero
        const int n = u / TC_KH, k = u - n * TC_KH;
        const __nv_bfloat16 v = __float2bfloat16(n == 0 && k < HID ? params[P_W5 + k * OUTN] : 0.f);
        *reinterpret_cast<__nv_bfloat16*>(wtc + TC_OFF_W5 + kmajor_off(n, k, TC_KH)) = v;
        return;
    }
    u -= TC_N5 * TC_KH;
    if (u < 4) reinterpret_cast<float*>(wtc + TC_OFF_B5)[u] = u == 0 ? params[P_B5] : 0.f;
}

template <int MODE>
__global__ void __launch_bounds__(TC_M * TC_NWG, 1) k_nsdf_mlp_tc(TcArgs a) {
    extern __shared__ __align__(128) uint8_t smem_tc[];
    uint8_t* sW = smem_tc;
    const int wg = threadIdx.x >> 7, tid = threadIdx.x & (TC_M - 1), warp = tid >> 5;   // warpgroup, row, warp in it
    const uint32_t uW = smem_u32(sW);
    const uint32_t bars = smem_u32(smem_tc + TC_WBYTES);
    const uint32_t bar = bars + 8u * wg;
    uint32_t* slot = reinterpret_cast<uint32_t*>(smem_tc + TC_WBYTES + 8 * TC_NWG);

    for (int i = threadIdx.x; i < TC_WBYTES / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(sW)[i] = reinterpret_cast<const uint4*>(a.wtc)[i];
    if (threadIdx.x == 0) {
        for (int g = 0; g < TC_NWG; ++g) mbar_init(bars + 8u * g, 1);
        fence_barrier_init();
    }
    if (threadIdx.x < 32) {
        tmem_alloc(smem_u32(slot), TC_TMEM_COLS);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const float b5 = reinterpret_cast<const float*>(sW + TC_OFF_B5)[0];   // staged above
    const uint32_t tD = *slot + (uint32_t)(wg * TC_COLS);             // this warpgroup's accumulator
    const uint32_t tA = tD + TC_ACOL;                                 // and its A operand
    const uint32_t lanes = (uint32_t)(warp * 32) << 16;               // this warp's 32 rows
    const Frame fr = a.fr;
    const long long total = MODE == TC_CLASSIFY ? a.vtot : (long long)a.count;
    const float limit = a.margin / fr.cell + a.slackCells;
    uint32_t parity = 0;

    // waits for the layer's MMAs; false (all threads alike) when the bounded wait gave up
    auto layer_done = [&]() -> bool {
        const bool ok = mbar_wait_bounded(bar, parity, TC_WAIT_POLLS);
        if (wg_sync_or(wg, !ok)) {
            if (tid == 0) atomicOr(a.err, 1);
            mbar_wait_bounded(bar, parity, TC_WAIT_POLLS);   // let the MMAs in flight finish
            return false;
        }
        parity ^= 1u;
        tc_fence_after();
        return true;
    };
    // one layer: K/16 MMAs of A (tensor memory, 8 columns per step) against weights at byte offset wOff
    auto issue = [&](int kt, int wOff, uint32_t idesc) {
        if (tid == 0) {
            tc_fence_after();
            const uint32_t sbo = (uint32_t)kt * 16u;
            for (int j = 0; j < kt / 16; ++j)
                tc_mma_ts(tD, tA + 8u * j, smem_desc(uW + wOff + 256u * j, 128u, sbo), idesc, j > 0);
            tc_commit(bar);
        }
    };
    // A written by every thread of the warpgroup: make it visible to the MMA issued after the barrier
    auto publish_a = [&]() {
        tc_wait_st();
        tc_fence_before();
        wg_sync(wg);
    };
    // row `tid` of the accumulator through SiLU into row `tid` of the next A (K = TC_KH: 64 activations,
    // then the bias columns of ones and zeros)
    auto hidden_epilogue = [&]() {
        uint32_t v[32], u[32];
        tc_ld32(tD + lanes + 0, v);
        tc_ld32(tD + lanes + 32, u);
        tc_wait_ld();
        uint32_t h[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) h[c] = silu_half2(v[2 * c], v[2 * c + 1]);
        tc_st16(tA + lanes + 0, h);
#pragma unroll
        for (int c = 0; c < 16; ++c) h[c] = silu_half2(u[2 * c], u[2 * c + 1]);
        tc_st16(tA + lanes + 16, h);
        const uint32_t ones[8] = {BF16_ONES, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
        tc_st8(tA + lanes + 32, ones);
        publish_a();
    };

    // this thread's point of a tile (the query pose for points, the sample's own pose for samples)
    float qx = 0.f, qy = 0.f, qz = 0.f, q0 = a.pose.a0, q1 = a.pose.a1, q2 = a.pose.a2;
    auto fetch = [&](long long t) {
        const long long i = t * TC_M + tid;
        if (i < total) {
            if constexpr (MODE == TC_SAMPLES) {
                const Sample S = a.samples[i];
                qx = S.x; qy = S.y; qz = S.z; q0 = S.p0; q1 = S.p1; q2 = S.p2;
            } else {
                const float4 P = a.pts[i];
                qx = P.x; qy = P.y; qz = P.z;
            }
        }
    };
    const long long tileStride = (long long)gridDim.x * TC_NWG;
    fetch((long long)blockIdx.x * TC_NWG + wg);
    for (long long tile = (long long)blockIdx.x * TC_NWG + wg; tile * TC_M < total; tile += tileStride) {
        const long long idx = tile * TC_M + tid;
        const bool valid = idx < total;
        const float px = qx, py = qy, pz = qz, a0 = q0, a1 = q1, a2 = q2;
        fetch(tile + tileStride);   // in flight while this tile's layers run
        {
            uint32_t w[56];
            point_features((px - fr.cx) * fr.ihx, (py - fr.cy) * fr.ihy, (pz - fr.cz) * fr.ihz, a0 * fr.poseScale,
                           a1 * fr.poseScale, a2 * fr.poseScale, valid, w);
            tc_st16(tA + lanes + 0, w);
            tc_st16(tA + lanes + 16, w + 16);
            tc_st16(tA + lanes + 32, w + 32);
            tc_st8(tA + lanes + 48, w + 48);
        }
        publish_a();

        issue(TC_K1, TC_OFF_W1, TC_IDESC);
        if (!layer_done()) break;
        hidden_epilogue();
        issue(TC_KH, TC_OFF_W2, TC_IDESC);
        if (!layer_done()) break;
        hidden_epilogue();
        issue(TC_KH, TC_OFF_W3, TC_IDESC);
        if (!layer_done()) break;
        hidden_epilogue();
        issue(TC_KH, TC_OFF_W4, TC_IDESC);
        if (!layer_done()) break;
        hidden_epilogue();
        // output layer: y = b5 + sum_k w5[k] SiLU(z4)[k] (the ones columns meet zero weights)
        issue(TC_KH, TC_OFF_W5, TC_IDESC5);
        if (!layer_done()) break;
        uint32_t acc;
        tc_ld1(tD + lanes, acc);
        tc_wait_ld();
        const float y = b5 + __uint_as_float(acc);
        tc_fence_before();   // the next tile's stores and MMAs reuse the columns after the warpgroup's next barrier

        if (valid) {
            if constexpr (MODE == TC_CLASSIFY) {
                if ((int)(idx % a.n) >= 2 && y < limit) {
                    a.bandList[atomicAdd(a.bandCount, 1)] = (int)idx;
                    mark_block_tc(a.marks, a.grid, sdf_coords(a.grid, mk3(px, py, pz)));
                }
            } else {
                a.out[idx] = MODE == TC_SAMPLES ? y : y * fr.cell;
            }
        }
    }

    tc_fence_before();
    __syncthreads();
    if (threadIdx.x < 32) {
        tc_fence_after();
        tmem_dealloc(*slot, TC_TMEM_COLS);
    }
}

cudaError_t launch_pack_tc(const float* params, uint8_t* wtc, cudaStream_t s) {
    const int total = HID * TC_K1 + 3 * HID * TC_KH + TC_N5 * TC_KH + 4;
    k_nsdf_pack_tc<<<(total + 255) / 256, 256, 0, s>>>(params, wtc);
    return cudaGetLastError();
}

template <int MODE>
static cudaError_t launch_tc(const TcArgs& a, long long total, cudaStream_t s) {
    if (total <= 0) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k_nsdf_mlp_tc<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
    if (e != cudaSuccess) return e;
    // resident blocks per SM: tensor memory (512 columns per SM) and shared memory (the weights)
    // decide it
    int dev = 0, smemPerSM = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smemPerSM, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (e != cudaSuccess) return e;
    const int perSM = std::max(1, std::min(smemPerSM / (int)(TC_SMEM + 1024), 512 / TC_TMEM_COLS));
    const long long tiles = (total + TC_M - 1) / TC_M;
    const long long wanted = (tiles + TC_NWG - 1) / TC_NWG;
    const unsigned blocks = (unsigned)std::max<long long>(1, std::min<long long>(wanted, (long long)perSM * sm_count()));
    k_nsdf_mlp_tc<MODE><<<blocks, TC_M * TC_NWG, TC_SMEM, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_query_tc(const TcArgs& a, cudaStream_t s) { return launch_tc<TC_POINTS>(a, a.count, s); }
cudaError_t launch_query_samples_tc(const TcArgs& a, cudaStream_t s) { return launch_tc<TC_SAMPLES>(a, a.count, s); }
cudaError_t launch_classify_tc(const TcArgs& a, cudaStream_t s) { return launch_tc<TC_CLASSIFY>(a, a.vtot, s); }

}  // namespace nsdf
}  // namespace tfx
