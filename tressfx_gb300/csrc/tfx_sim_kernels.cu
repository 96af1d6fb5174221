// Strand-simulation kernels of the plain path: one kernel per reference compute entry point of
// src/Shaders/TressFXSimulation.hlsl, launched once per object per stage in the reference's
// dispatch order (src/TressFX/TressFXSimulation.cpp:77-112).
//
// Work decomposition (sm_103a): 32-wide warps, no 64-wide groupshared emulation.
//   * vertex-parallel stages (integration, VSP, follow) use one thread per vertex, consecutive
//     threads on consecutive float4 of a strand (strand-major layout -> coalesced 16 B accesses);
//   * LocalShapeConstraints stages 32 strands per warp in shared memory (padded [vertex][strand]
//     layout, conflict-free) and runs the serial Gauss-Seidel sweep per strand from there;
//   * LengthConstriantsWindAndCollision keeps one strand segment in a warp's registers (one or two
//     vertices per lane) and does the red/black distance-constraint passes with warp shuffles.
// Every kernel reproduces the reference's per-vertex arithmetic in the same order (see
// tfx_device_math.cuh), so results match the FP32 oracle bit for bit.
#include "tfx_device_math.cuh"
#include "tfx_internal.h"

namespace tfx {

// --------------------------------------------------------------------------------------------
// IntegrationAndGlobalShapeConstraints, TressFXSimulation.hlsl:609-666.  One thread per guide vertex.
template <int N>
__global__ void __launch_bounds__(256) k_integrate(HairView h) {
    const DevSimConsts* __restrict__ c = h.consts;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= h.G * N) return;
    const int g = t / N, j = t % N;
    const int gs = g * (h.F + 1);
    const int gv = gs * N + j;

    float4 initialPos = __ldg(h.init + gv);
    float m[4][4];
    blend_bones(c->bones, __ldg(h.skin + 2 * gs), __ldg(h.skin + 2 * gs + 1), m);
    const float3 sk = xform_row(xyz(initialPos), 1.0f, m);
    initialPos.x = sk.x; initialPos.y = sk.y; initialPos.z = sk.z;

    float4 currentPos = h.pos[gv];
    float4 shared = currentPos;
    const float4 prevStored = h.prev[gv];
    float4 oldPos = prevStored;
    if (c->reset != 0.0f) { currentPos = initialPos; oldPos = initialPos; }

    if (currentPos.w > 0.0f) {
        // Integrate(), :440-446: cur + decay*(cur-old) + force*dt*dt, force = g*(0,-1,0)
        const float dt = c->timeStep;
        const float gx = c->gravity * 0.0f, gy = c->gravity * -1.0f;
        const float3 cur = xyz(currentPos), old = xyz(oldPos);
        const float3 force = mk3(gx, gy, gx);
        const float3 r = add(add(cur, mul(c->decay, sub(cur, old))), mul(mul(force, dt), dt));
        shared.x = r.x; shared.y = r.y; shared.z = r.z;
    } else {
        shared = initialPos;
    }

    const float kG = c->globalStiffness, range = c->globalRange;
    if (kG > 0.0f && range != 0.0f) {
        if (shared.w > 0.0f) {
            if ((float)j < range * (float)N) {
                const float3 del = mul(kG, sub(xyz(initialPos), xyz(shared)));
                shared.x = shared.x + del.x; shared.y = shared.y + del.y; shared.z = shared.z + del.z;
            }
        }
    }
    // UpdateFinalVertexPositions, :581-586
    h.prevprev[gv] = prevStored;
    h.prev[gv] = currentPos;
    h.pos[gv] = shared;
}

// --------------------------------------------------------------------------------------------
// CalculateStrandLevelData, TressFXSimulation.hlsl:677-728.  One thread per guide strand.
__global__ void __launch_bounds__(128) k_strand_level(HairView h) {
    const DevSimConsts* __restrict__ c = h.consts;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= h.G) return;
    const int gs = g * (h.F + 1);
    const int root = gs * h.n;
    const float4 oo1 = h.prevprev[root + 1];
    const float4 o0 = h.prev[root], o1 = h.prev[root + 1];
    const float4 n0 = h.pos[root], n1 = h.pos[root + 1];

    const float3 u = normalize(sub(xyz(o1), xyz(o0)));
    const float3 v = normalize(sub(xyz(n1), xyz(n0)));
    const Q4 rot = qfrom2(u, v);
    const float3 trans = sub(xyz(n0), qrot(rot, xyz(o0)));

    float vspCoeff = c->vspCoeff;
    const float ax = (n1.x - 2.0f * o1.x) + oo1.x;
    const float ay = (n1.y - 2.0f * o1.y) + oo1.y;
    const float az = (n1.z - 2.0f * o1.z) + oo1.z;
    const float aw = (n1.w - 2.0f * o1.w) + oo1.w;
    const float accel = sqrtf(ax * ax + ay * ay + az * az + aw * aw);
    if (accel > c->vspAccelThreshold) vspCoeff = 1.0f;

    float m[4][4];
    blend_bones(c->bones, __ldg(h.skin + 2 * gs), __ldg(h.skin + 2 * gs + 1), m);
    const Q4 bq = quat_from_matrix(m);

    h.sld[3 * gs + 0] = make_float4(bq.x, bq.y, bq.z, bq.w);
    h.sld[3 * gs + 1] = make_float4(rot.x, rot.y, rot.z, rot.w);
    h.sld[3 * gs + 2] = make_float4(trans.x, trans.y, trans.z, vspCoeff);
}

// --------------------------------------------------------------------------------------------
// VelocityShockPropagation, TressFXSimulation.hlsl:739-762.  One thread per guide vertex.
template <int N>
__global__ void __launch_bounds__(256) k_vsp(HairView h) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= h.G * N) return;
    const int g = t / N, j = t % N;
    if (j < 2) return;
    const int gs = g * (h.F + 1);
    const int gv = gs * N + j;
    const float4 qv = h.sld[3 * gs + 1];
    const float4 tv = h.sld[3 * gs + 2];
    const Q4 q{qv.x, qv.y, qv.z, qv.w};
    const float3 tr = xyz(tv);
    const float cf = tv.w;
    float4 pn = h.pos[gv];
    float4 po = h.prev[gv];
    const float3 a = add(mul(1.0f - cf, xyz(pn)), mul(cf, add(qrot(q, xyz(pn)), tr)));
    const float3 b = add(mul(1.0f - cf, xyz(po)), mul(cf, add(qrot(q, xyz(po)), tr)));
    h.pos[gv] = with_xyz(pn, a);
    h.prev[gv] = with_xyz(po, b);
}

// --------------------------------------------------------------------------------------------
// LocalShapeConstraints, TressFXSimulation.hlsl:773-829.  One warp = 32 strands; each lane owns
// one strand's serial sweep j = 1..n-2.  Positions and bind-pose positions (skinningQuat * rest)
// are staged in shared memory as [vertex][strand] rows padded to 33 entries.
template <int N>
__global__ void __launch_bounds__(32) k_local_shape(HairView h) {
    constexpr int S = 32, LD = S + 1;
    extern __shared__ float4 smem[];
    float4* P = smem;                        // [N][LD] positions
    float* BX = reinterpret_cast<float*>(P + N * LD);
    float* BY = BX + N * LD;
    float* BZ = BY + N * LD;                 // [N][LD] bind-pose positions, SoA

    const DevSimConsts* __restrict__ c = h.consts;
    const int lane = threadIdx.x;
    const int g0 = blockIdx.x * S;
    const int nstr = min(S, h.G - g0);
    const int stride = (h.F + 1) * N;

    for (int idx = lane; idx < nstr * N; idx += 32) {
        const int s = idx / N, j = idx % N;
        const int gs = (g0 + s) * (h.F + 1);
        const int gv = (g0 + s) * stride + j;
        P[j * LD + s] = h.pos[gv];
        const float4 bq4 = h.sld[3 * gs];
        const Q4 bq{bq4.x, bq4.y, bq4.z, bq4.w};
        const float3 b = qrot(bq, xyz(__ldg(h.init + gv)));
        BX[j * LD + s] = b.x; BY[j * LD + s] = b.y; BZ[j * LD + s] = b.z;
    }
    __syncwarp();

    if (lane < nstr) {
        const int s = lane;
        const float stiff = 0.5f * fminf(c->localStiffness, 0.95f);
        float4 pm1 = P[0 * LD + s];
        float4 pos = P[1 * LD + s];
        float3 bm1 = mk3(BX[s], BY[s], BZ[s]);
        float3 b0 = mk3(BX[LD + s], BY[LD + s], BZ[LD + s]);
#pragma unroll 4
        for (int j = 1; j < N - 1; ++j) {
            float4 pp1 = P[(j + 1) * LD + s];
            const float3 bp1 = mk3(BX[(j + 1) * LD + s], BY[(j + 1) * LD + s], BZ[(j + 1) * LD + s]);
            const float3 lastVec = sub(xyz(pos), xyz(pm1));
            const float3 vecBindPose = sub(bp1, b0);
            const float3 lastVecBindPose = sub(b0, bm1);
            const Q4 rg = qfrom2(normalize(lastVecBindPose), normalize(lastVec));
            const float3 org = add(qrot(rg, vecBindPose), xyz(pos));
            const float3 del = mul(stiff, sub(org, xyz(pp1)));
            if (pos.w > 0.0f) { pos.x = pos.x - del.x; pos.y = pos.y - del.y; pos.z = pos.z - del.z; }
            if (pp1.w > 0.0f) { pp1.x = pp1.x + del.x; pp1.y = pp1.y + del.y; pp1.z = pp1.z + del.z; }
            P[j * LD + s] = pos;
            pm1 = pos; pos = pp1; bm1 = b0; b0 = bp1;
        }
        P[(N - 1) * LD + s] = pos;
    }
    __syncwarp();

    for (int idx = lane; idx < nstr * N; idx += 32) {
        const int s = idx / N, j = idx % N;
        h.pos[(g0 + s) * stride + j] = P[j * LD + s];
    }
}

// --------------------------------------------------------------------------------------------
// LengthConstriantsWindAndCollision, TressFXSimulation.hlsl:875-975 (capsules compiled out).
// A strand occupies L = min(n,32) consecutive lanes; each lane holds VPL = n/L vertices.


template <int N>
__global__ void __launch_bounds__(256) k_length_wind(HairView h) {
    constexpr int L = N < 32 ? N : 32;
    constexpr int VPL = N / L;
    constexpr int SPW = 32 / L;
    const DevSimConsts* __restrict__ c = h.consts;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int q = lane % L;
    const int g = warp * SPW + lane / L;
    const bool active = g < h.G;
    const int gs = g * (h.F + 1);
    const int base = gs * N + q * VPL;

    float4 p[VPL];
    float len[VPL];
#pragma unroll
    for (int k = 0; k < VPL; ++k) {
        p[k] = active ? h.pos[base + k] : make_float4(0.f, 0.f, 0.f, 0.f);
        len[k] = active ? __ldg(h.rest + base + k) : 0.0f;
    }

    // ---- wind (all displacements from pre-wind positions)
    if (c->anyWind) {
        const float a = (float)(gs % 20) / 20.0f;
        const float3 w0 = xyz(c->wind[0]), w1 = xyz(c->wind[1]), w2 = xyz(c->wind[2]), w3 = xyz(c->wind[3]);
        const float3 w = add(add(add(mul(a, w0), mul(1.0f - a, w1)), mul(a, w2)), mul(1.0f - a, w3));
        const float dt = c->timeStep;
        float4 nxt[VPL];
        if constexpr (VPL == 1) {
            nxt[0] = shfl4_down(p[0], 1);
        } else {
            nxt[0] = p[1];
            nxt[1] = shfl4_down(p[0], 1);
        }
        float3 disp[VPL];
#pragma unroll
        for (int k = 0; k < VPL; ++k) {
            const int j = q * VPL + k;
            disp[k] = mk3(0.f, 0.f, 0.f);
            if (j >= 2 && j < N - 1) {
                const float3 v = sub(xyz(p[k]), xyz(nxt[k]));
                const float3 force = neg(cross(cross(v, w), v));
                disp[k] = mul(mul(force, dt), dt);
            }
        }
#pragma unroll
        for (int k = 0; k < VPL; ++k) {
            const int j = q * VPL + k;
            if (j >= 2 && j < N - 1) {
                p[k].x = p[k].x + disp[k].x; p[k].y = p[k].y + disp[k].y; p[k].z = p[k].z + disp[k].z;
            }
        }
    }

    // ---- length constraints: pass 1 on edges (2i, 2i+1), pass 2 on edges (2i+1, 2i+2)
    const int iters = c->lengthIterations;
    for (int it = 0; it < iters; ++it) {
        if constexpr (VPL == 1) {
            {
                const float4 o = shfl4(p[0], lane ^ 1);
                const float ol = __shfl_sync(FULL, len[0], lane ^ 1);
                const bool even = (q & 1) == 0;
                const DC r = even ? distance_constraint(p[0], o, len[0]) : distance_constraint(o, p[0], ol);
                p[0] = even ? r.p0 : r.p1;
            }
            {
                const bool odd = (q & 1) != 0;
                const int src = odd ? ((lane + 1) & 31) : ((lane + 31) & 31);
                const float4 o = shfl4(p[0], src);
                const float ol = __shfl_sync(FULL, len[0], src);
                if (odd && q <= N - 3) {
                    p[0] = distance_constraint(p[0], o, len[0]).p0;
                } else if (!odd && q >= 2) {
                    p[0] = distance_constraint(o, p[0], ol).p1;
                }
            }
        } else {
            {
                const DC r = distance_constraint(p[0], p[1], len[0]);
                p[0] = r.p0; p[1] = r.p1;
            }
            {
                const float4 nextFirst = shfl4_down(p[0], 1);
                const float4 prevLast = shfl4_up(p[1], 1);
                const float prevLen = __shfl_up_sync(FULL, len[1], 1);
                const float4 myLast = p[1];
                const float4 myFirst = p[0];
                if (q < L - 1) p[1] = distance_constraint(myLast, nextFirst, len[1]).p0;
                if (q >= 1) p[0] = distance_constraint(prevLast, myFirst, prevLen).p1;
            }
        }
    }

    // ---- tangents (from the constrained positions)
    float3 tng[VPL];
    if constexpr (VPL == 1) {
        const float4 nx = shfl4_down(p[0], 1);
        const float4 pv = shfl4_up(p[0], 1);
        tng[0] = (q == N - 1) ? sub(xyz(p[0]), xyz(pv)) : sub(xyz(nx), xyz(p[0]));
    } else {
        const float4 nx = shfl4_down(p[0], 1);
        tng[0] = sub(xyz(p[1]), xyz(p[0]));
        tng[1] = (q == L - 1) ? sub(xyz(p[1]), xyz(p[0])) : sub(xyz(nx), xyz(p[1]));
    }

    if (!active) return;
    const float clamp2 = c->clamp * c->clamp;
#pragma unroll
    for (int k = 0; k < VPL; ++k) {
        const int gv = base + k;
        const float4 oldPos = h.prev[gv];
        const float4 oldTan = h.tan[gv];
        h.tan[gv] = with_xyz(oldTan, normalize(tng[k]));
        float3 d = sub(xyz(p[k]), xyz(oldPos));
        const float speedSqr = dot(d, d);
        if (speedSqr > clamp2) {
            d = mul(d, clamp2 / speedSqr);
            h.prev[gv] = with_xyz(oldPos, sub(xyz(p[k]), d));
        }
        h.pos[gv] = p[k];
    }
}

// --------------------------------------------------------------------------------------------
// UpdateFollowHairVertices, TressFXSimulation.hlsl:978-1001.  One thread per follow vertex.
template <int N>
__global__ void __launch_bounds__(256) k_follow(HairView h) {
    const DevSimConsts* __restrict__ c = h.consts;
    const int per = h.F * N;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= h.G * per) return;
    const int g = t / per, r = t - g * per;
    const int i = r / N, j = r % N;
    const int sbase = g * (h.F + 1);
    const int gv = sbase * N + j;
    const int fv = sbase * N + N + r;
    const float4 p = h.pos[gv];
    const float4 tn = h.tan[gv];
    const float4 off = __ldg(h.followOffset + sbase + i + 1);
    const float factor = c->tipSeparation * ((float)j / (float)N) + 1.0f;
    const float4 old = h.pos[fv];
    h.pos[fv] = with_xyz(old, add(xyz(p), mul(factor, xyz(off))));
    h.tan[fv] = tn;
}

// --------------------------------------------------------------------------------------------
// launchers
#define TFX_SWITCH_N(n, CALL)                 \
    switch (n) {                              \
        case 4: { constexpr int NN = 4; CALL; } break;   \
        case 8: { constexpr int NN = 8; CALL; } break;   \
        case 16: { constexpr int NN = 16; CALL; } break; \
        case 32: { constexpr int NN = 32; CALL; } break; \
        case 64: { constexpr int NN = 64; CALL; } break; \
        default: return cudaErrorInvalidValue;           \
    }

static inline unsigned blocks_for(long long work, int threads) { return (unsigned)((work + threads - 1) / threads); }

cudaError_t launch_integrate(const HairView& h, cudaStream_t s) {
    if (h.G <= 0) return cudaSuccess;
    TFX_SWITCH_N(h.n, (k_integrate<NN><<<blocks_for((long long)h.G * NN, 256), 256, 0, s>>>(h)));
    return cudaGetLastError();
}

cudaError_t launch_strand_level(const HairView& h, cudaStream_t s) {
    if (h.G <= 0) return cudaSuccess;
    k_strand_level<<<blocks_for(h.G, 128), 128, 0, s>>>(h);
    return cudaGetLastError();
}

cudaError_t launch_vsp(const HairView& h, cudaStream_t s) {
    if (h.G <= 0) return cudaSuccess;
    TFX_SWITCH_N(h.n, (k_vsp<NN><<<blocks_for((long long)h.G * NN, 256), 256, 0, s>>>(h)));
    return cudaGetLastError();
}

template <int N>
static cudaError_t launch_local_shape_n(const HairView& h, cudaStream_t s) {
    const size_t smem = (size_t)N * 33 * (sizeof(float4) + 3 * sizeof(float));
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(k_local_shape<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    k_local_shape<N><<<blocks_for(h.G, 32), 32, smem, s>>>(h);
    return cudaGetLastError();
}

cudaError_t launch_local_shape(const HairView& h, cudaStream_t s) {
    if (h.G <= 0) return cudaSuccess;
    TFX_SWITCH_N(h.n, return launch_local_shape_n<NN>(h, s));
    return cudaSuccess;
}

template <int N>
static cudaError_t launch_length_wind_n(const HairView& h, cudaStream_t s) {
    constexpr int L = N < 32 ? N : 32;  // lanes per strand
    const long long lanes = (long long)((h.G + (32 / L) - 1) / (32 / L)) * 32;
    k_length_wind<N><<<blocks_for(lanes, 256), 256, 0, s>>>(h);
    return cudaGetLastError();
}

cudaError_t launch_length_wind(const HairView& h, cudaStream_t s) {
    if (h.G <= 0) return cudaSuccess;
    TFX_SWITCH_N(h.n, return launch_length_wind_n<NN>(h, s));
    return cudaSuccess;
}

cudaError_t launch_follow(const HairView& h, cudaStream_t s) {
    if (h.G <= 0 || h.F <= 0) return cudaSuccess;
    TFX_SWITCH_N(h.n, (k_follow<NN><<<blocks_for((long long)h.G * h.F * NN, 256), 256, 0, s>>>(h)));
    return cudaGetLastError();
}

}  // namespace tfx
