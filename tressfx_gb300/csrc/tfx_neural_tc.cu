// Inference of the learned collision proxy (tfx_neural.cuh) on the fifth-generation tensor cores.
//
// A block holds the packed weights once in shared memory and runs TC_NWG warpgroups, each carrying
// its own tiles of 128 points through the network, so that one warpgroup's feature and activation
// arithmetic overlaps the other warpgroups' MMAs.  In a warpgroup, thread r computes point r's 102
// features into row r of the warpgroup's bf16 A operand; one thread issues the layer's tcgen05.mma
// (kind::f16, bf16 x bf16 -> f32, M = 128 points, N = 64 neurons, K = 16 per instruction) against the
// layer's weights; the accumulator lives in the warpgroup's 64 tensor-memory columns; tcgen05.commit
// signals the warpgroup's mbarrier when the layer's MMAs are done.  Thread r then reads row r of the
// accumulator (tcgen05.ld, 32 lanes x 32 columns per instruction), applies SiLU and writes the bf16
// activations back as row r of the next layer's A operand.  The output layer (64 -> 1) is one more
// MMA (N = 16, weights in column 0), read back as one tensor-memory column, plus the fp32 bias.  Each
// thread loads its point of the warpgroup's next tile while the current tile's layers run.
// Warpgroups synchronise on their own named barriers (ids 1..TC_NWG).
//
// Operand layout: K-major, no swizzle, 8-row x 16-byte core matrices; the core matrix of row group
// R and column group C of a matrix with K columns starts at byte (R * K / 8 + C) * 128, so the
// descriptor of a 16-column step has a leading-dimension offset (between the two column groups) of
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
constexpr int TC_COLS = 64;                // tensor-memory columns of one accumulator (N = 64, fp32)
// tensor-memory columns a block allocates: a power of two >= 32 covering every warpgroup's accumulator
constexpr int TC_TMEM_COLS = TC_NWG * TC_COLS <= 32 ? 32 : TC_NWG * TC_COLS <= 64 ? 64 : TC_NWG * TC_COLS <= 128 ? 128
                             : TC_NWG * TC_COLS <= 256 ? 256 : 512;
static_assert(TC_NWG * TC_COLS <= 512, "the warpgroups' accumulators exceed the tensor memory of an SM");
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
__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
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

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
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
    uint8_t* sA = smem_tc + TC_WBYTES + (size_t)wg * TC_ABYTES;
    const uint32_t uW = smem_u32(sW), uA = smem_u32(sA);
    const uint32_t bars = smem_u32(smem_tc + TC_WBYTES + (size_t)TC_NWG * TC_ABYTES);
    const uint32_t bar = bars + 8u * wg;
    uint32_t* slot = reinterpret_cast<uint32_t*>(smem_tc + TC_WBYTES + (size_t)TC_NWG * TC_ABYTES + 8 * TC_NWG);

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
    const uint32_t tmem = *slot + (uint32_t)(wg * TC_COLS);           // this warpgroup's accumulator
    const uint32_t myLanes = tmem + ((uint32_t)(warp * 32) << 16);   // this warp's 32 accumulator rows
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
    // one layer: K/16 MMAs of the A buffer (row stride kt columns) against weights at byte offset wOff
    auto issue = [&](int kt, int wOff, uint32_t idesc) {
        if (tid == 0) {
            tc_fence_after();
            const uint32_t sbo = (uint32_t)kt * 16u;
            for (int j = 0; j < kt / 16; ++j)
                tc_mma(tmem, smem_desc(uA + 256u * j, 128u, sbo), smem_desc(uW + wOff + 256u * j, 128u, sbo), idesc,
                       j > 0);
            tc_commit(bar);
        }
    };
    // row `tid` of the accumulator through SiLU into row `tid` of the next A operand (K = TC_KH)
    auto hidden_epilogue = [&](bool writeOnes) {
        uint32_t v[32], u[32];
        tc_ld32(myLanes + 0, v);
        tc_ld32(myLanes + 32, u);
        tc_wait_ld();
#pragma unroll
        for (int c = 0; c < 4; ++c)
            st_shared_v4(uA + kmajor_off(tid, 8 * c, TC_KH), silu_half2(v[8 * c], v[8 * c + 1]),
                         silu_half2(v[8 * c + 2], v[8 * c + 3]), silu_half2(v[8 * c + 4], v[8 * c + 5]),
                         silu_half2(v[8 * c + 6], v[8 * c + 7]));
#pragma unroll
        for (int c = 0; c < 4; ++c)
            st_shared_v4(uA + kmajor_off(tid, 32 + 8 * c, TC_KH), silu_half2(u[8 * c], u[8 * c + 1]),
                         silu_half2(u[8 * c + 2], u[8 * c + 3]), silu_half2(u[8 * c + 4], u[8 * c + 5]),
                         silu_half2(u[8 * c + 6], u[8 * c + 7]));
        if (writeOnes) {
            st_shared_v4(uA + kmajor_off(tid, HID, TC_KH), BF16_ONES, 0u, 0u, 0u);
            st_shared_v4(uA + kmajor_off(tid, HID + 8, TC_KH), 0u, 0u, 0u, 0u);
        }
        fence_proxy_async_smem();
        tc_fence_before();
        wg_sync(wg);
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
#pragma unroll
            for (int c = 0; c < TC_K1 / 8; ++c)
                st_shared_v4(uA + kmajor_off(tid, 8 * c, TC_K1), w[4 * c], w[4 * c + 1], w[4 * c + 2], w[4 * c + 3]);
        }
        fence_proxy_async_smem();
        wg_sync(wg);

        issue(TC_K1, TC_OFF_W1, TC_IDESC);
        if (!layer_done()) break;
        hidden_epilogue(true);
        issue(TC_KH, TC_OFF_W2, TC_IDESC);
        if (!layer_done()) break;
        hidden_epilogue(false);
        issue(TC_KH, TC_OFF_W3, TC_IDESC);
        if (!layer_done()) break;
        hidden_epilogue(false);
        issue(TC_KH, TC_OFF_W4, TC_IDESC);
        if (!layer_done()) break;
        hidden_epilogue(false);
        // output layer: y = b5 + sum_k w5[k] SiLU(z4)[k] (the ones columns meet zero weights)
        issue(TC_KH, TC_OFF_W5, TC_IDESC5);
        if (!layer_done()) break;
        uint32_t acc;
        tc_ld1(myLanes, acc);
        tc_wait_ld();
        const float y = b5 + __uint_as_float(acc);
        tc_fence_before();   // the next tile's MMAs overwrite the accumulator after the warpgroup's next barrier

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
    // resident blocks per SM: shared memory (each block holds the weights and one operand per
    // warpgroup) and tensor memory (512 columns per SM) decide it
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
