// C ABI of the library (include/tressfx_gb300.h): handles, device memory, validation, and the
// stream-ordered dispatch of the plain-path kernels.  It replaces the reference's Engine
// Interface compute subset (src/EngineInterface.h) and the per-object GPU state of
// TressFXHairObject / TressFXDynamicState / TressFXSDFCollision / TressFXBoneSkinning.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>

#include "tfx_handles.h"

using namespace tfx;

// ============================================================================ errors
static thread_local std::string g_last_error;

namespace tfx {
int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation) return fail(TFX_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    return fail(TFX_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

void context_retain(tfx_context c) { c->refs.fetch_add(1); }

void context_release(tfx_context c) {
    if (c->refs.fetch_sub(1) != 1) return;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (auto ev : c->stampEvents) cudaEventDestroy(ev);
    cudaStreamDestroy(c->stream);
    delete c;
}

void fill_consts_header(DevSimConsts* c, const tfx_sim_params* p, int cpuLocalIterations) {
    const float* w[4] = {p->wind, p->wind1, p->wind2, p->wind3};
    for (int i = 0; i < 4; ++i) c->wind[i] = make_float4(w[i][0], w[i][1], w[i][2], w[i][3]);
    c->damping = p->shape[0];
    c->localStiffness = p->shape[1];
    c->globalStiffness = p->shape[2];
    c->globalRange = p->shape[3];
    c->gravity = p->grav_time_tip[0];
    c->timeStep = p->grav_time_tip[1];
    c->tipSeparation = p->grav_time_tip[2];
    // exp(-dampingCoeff * g_TimeStep * 60.0f), TressFXSimulation.hlsl:444, once per upload
    const float arg = (-c->damping * c->timeStep) * 60.0f;
    c->decay = std::exp(arg);
    c->lengthIterations = p->sim_ints[0];
    c->localIterations = p->sim_ints[1];
    c->anyWind = (p->wind[0] != 0.0f || p->wind[1] != 0.0f || p->wind[2] != 0.0f) ? 1 : 0;
    c->reserved0 = cpuLocalIterations;
    c->vspCoeff = p->vsp[0];
    c->vspAccelThreshold = p->vsp[1];
    c->reset = p->reset_positions;
    c->clamp = p->clamp_position_delta;
}
}  // namespace tfx

extern "C" const char* tfx_status_string(int s) {
    switch (s) {
        case TFX_OK: return "TFX_OK";
        case TFX_ERR_INVALID_ARGUMENT: return "TFX_ERR_INVALID_ARGUMENT";
        case TFX_ERR_VERTS_PER_STRAND: return "TFX_ERR_VERTS_PER_STRAND";
        case TFX_ERR_BONE_INDEX: return "TFX_ERR_BONE_INDEX";
        case TFX_ERR_BONE_WEIGHTS: return "TFX_ERR_BONE_WEIGHTS";
        case TFX_ERR_CUDA: return "TFX_ERR_CUDA";
        case TFX_ERR_OUT_OF_MEMORY: return "TFX_ERR_OUT_OF_MEMORY";
        case TFX_ERR_TIMEOUT: return "TFX_ERR_TIMEOUT";
        case TFX_ERR_SIZE: return "TFX_ERR_SIZE";
        case TFX_ERR_MISMATCH: return "TFX_ERR_MISMATCH";
        case TFX_ERR_NO_DEVICE: return "TFX_ERR_NO_DEVICE";
        default: return "TFX_ERR_UNKNOWN";
    }
}
extern "C" const char* tfx_last_error(void) { return g_last_error.c_str(); }
extern "C" int tfx_abi_version(void) { return TFX_ABI_VERSION; }

// ============================================================================ context
extern "C" int tfx_context_create(int device, tfx_context* out) {
    if (!out) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_context_create: out is null");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count <= 0) return fail(TFX_ERR_NO_DEVICE, "tfx_context_create: no CUDA device (%s)", cudaGetErrorString(e));
    if (device < 0 || device >= count) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_context_create: device %d of %d", device, count);
    cudaDeviceProp prop;
    TFX_CUDA(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
    if (prop.major * 10 + prop.minor != 103)
        return fail(TFX_ERR_NO_DEVICE, "tfx_context_create: device %d is sm_%d%d; this library is built for sm_103a only", device,
                    prop.major, prop.minor);
    TFX_CUDA(cudaSetDevice(device), "cudaSetDevice");
    auto* c = new (std::nothrow) tfx_context_t();
    if (!c) return fail(TFX_ERR_OUT_OF_MEMORY, "tfx_context_create: host allocation");
    c->device = device;
    c->numSMs = prop.multiProcessorCount;
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete c; return cuda_fail(e, "cudaStreamCreateWithFlags"); }
    *out = c;
    return TFX_OK;
}

extern "C" int tfx_context_destroy(tfx_context c) {
    if (!c) return TFX_OK;
    context_release(c);
    return TFX_OK;
}

extern "C" int tfx_context_synchronize(tfx_context c) {
    if (!c) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_context_synchronize: null context");
    TFX_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    return TFX_OK;
}

extern "C" void* tfx_context_stream(tfx_context c) { return c ? (void*)c->stream : nullptr; }

extern "C" int tfx_context_timestamp(tfx_context c, const char* name) {
    if (!c || !name) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_context_timestamp: null argument");
    cudaEvent_t ev;
    TFX_CUDA(cudaEventCreate(&ev), "cudaEventCreate");
    cudaError_t e = cudaEventRecord(ev, c->stream);
    if (e != cudaSuccess) { cudaEventDestroy(ev); return cuda_fail(e, "cudaEventRecord"); }
    c->stampNames.emplace_back(name);
    c->stampEvents.push_back(ev);
    return TFX_OK;
}

extern "C" int tfx_context_timestamps(tfx_context c, char (*names)[64], float* ms, int max, int* count) {
    if (!c || !count) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_context_timestamps: null argument");
    TFX_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    int n = (int)c->stampEvents.size();
    int k = std::min(n, std::max(max, 0));
    for (int i = 0; i < k; ++i) {
        float t = 0.f;
        if (i > 0) cudaEventElapsedTime(&t, c->stampEvents[0], c->stampEvents[i]);
        if (ms) ms[i] = t;
        if (names) { std::strncpy(names[i], c->stampNames[i].c_str(), 63); names[i][63] = 0; }
    }
    *count = k;
    for (auto ev : c->stampEvents) cudaEventDestroy(ev);
    c->stampEvents.clear();
    c->stampNames.clear();
    return TFX_OK;
}

extern "C" int tfx_host_alloc(size_t bytes, void** out) {
    if (!out) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_host_alloc: out is null");
    *out = nullptr;
    TFX_CUDA(cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocPortable), "cudaHostAlloc");
    return TFX_OK;
}

extern "C" int tfx_host_free(void* p) {
    if (p) TFX_CUDA(cudaFreeHost(p), "cudaFreeHost");
    return TFX_OK;
}

// ============================================================================ hair object
static bool valid_n(int n) { return n == 4 || n == 8 || n == 16 || n == 32 || n == 64; }

// Bone indices / weights exactly as ApplyVertexBoneSkinning reads them (TressFXSimulation.hlsl:552-564):
// index 0 always, index i>0 only when its weight is > 0; the divisor is w0 + sum(w_i > 0).
// *maxBone receives the highest index read.
static int validate_skinning(const float* skin, int64_t count, int64_t stride_items, const char* who, int* maxBone) {
    int mb = 0;
    for (int64_t s = 0; s < count; ++s) {
        const float* idx = skin + 8 * s * stride_items;
        const float* w = idx + 4;
        float wsum = w[0];
        for (int i = 0; i < 4; ++i) {
            bool used = (i == 0) || (w[i] > 0.0f);
            if (!used) continue;
            if (!(idx[i] >= 0.0f) || !(idx[i] < (float)TFX_MAX_BONES))
                return fail(TFX_ERR_BONE_INDEX, "%s: item %lld bone index %g outside [0, %d)", who, (long long)s * stride_items,
                            (double)idx[i], TFX_MAX_BONES);
            mb = std::max(mb, (int)idx[i]);
            if (i > 0) wsum = wsum + w[i];
        }
        if (!(wsum > 0.0f) || !std::isfinite(wsum))
            return fail(TFX_ERR_BONE_WEIGHTS, "%s: item %lld bone weights sum to %g", who, (long long)s * stride_items, (double)wsum);
    }
    if (maxBone) *maxBone = mb;
    return TFX_OK;
}

static int validate_desc(const tfx_hair_desc* d, const float* bone_skinning, const char* who, int* maxBone) {
    if (!d || !bone_skinning) return fail(TFX_ERR_INVALID_ARGUMENT, "%s: null descriptor or skinning", who);
    if (!valid_n(d->verts_per_strand))
        return fail(TFX_ERR_VERTS_PER_STRAND, "%s: %d vertices per strand; must be 4, 8, 16, 32 or 64", who, d->verts_per_strand);
    if (d->num_guide_strands <= 0 || d->follow_hairs_per_guide < 0)
        return fail(TFX_ERR_INVALID_ARGUMENT, "%s: %d guide strands, %d follow hairs per guide", who, d->num_guide_strands,
                    d->follow_hairs_per_guide);
    const int64_t G = d->num_guide_strands, n = d->verts_per_strand, F = d->follow_hairs_per_guide;
    const int64_t Stot = G * (F + 1), Vtot = Stot * n;
    if (Vtot > (int64_t)std::numeric_limits<int32_t>::max() / 2 || 3 * Stot > (int64_t)std::numeric_limits<int32_t>::max())
        return fail(TFX_ERR_SIZE, "%s: %lld vertices exceed the 31-bit index space", who, (long long)Vtot);
    return validate_skinning(bone_skinning, G, F + 1, who, maxBone);
}

extern "C" int tfx_hair_validate(const tfx_hair_desc* d, const float* bone_skinning) {
    return validate_desc(d, bone_skinning, "tfx_hair_validate", nullptr);
}

static void hair_free(tfx_hair h) {
    if (h->arena) cudaFree(h->arena);
    for (int i = 0; i < 2; ++i) {
        if (h->staging[i]) cudaFreeHost(h->staging[i]);
        if (h->stagingDone[i]) cudaEventDestroy(h->stagingDone[i]);
    }
    if (h->ctx) context_release(h->ctx);
    delete h;
}

extern "C" int tfx_hair_create(tfx_context ctx, const tfx_hair_desc* d, const float* positions, const float* tangents,
                               const float* rest_lengths, const float* follow_root_offsets, const float* bone_skinning,
                               tfx_hair* out) {
    if (!out) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_hair_create: out is null");
    *out = nullptr;
    if (!ctx || !d || !positions || !rest_lengths || !bone_skinning)
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_hair_create: null context, descriptor, positions, rest lengths or skinning");
    int maxBone = 0;
    if (int r = validate_desc(d, bone_skinning, "tfx_hair_create", &maxBone)) return r;
    const int64_t G = d->num_guide_strands, n = d->verts_per_strand, F = d->follow_hairs_per_guide;
    const int64_t Stot = G * (F + 1), Vtot = Stot * n;

    TFX_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    auto* h = new (std::nothrow) tfx_hair_t();
    if (!h) return fail(TFX_ERR_OUT_OF_MEMORY, "tfx_hair_create: host allocation");
    h->ctx = ctx; h->G = (int)G; h->n = (int)n; h->F = (int)F; h->Vtot = Vtot; h->Stot = Stot; h->maxBone = maxBone;
    context_retain(ctx);

    const size_t v16 = 16 * (size_t)Vtot, s16 = 16 * (size_t)Stot;
    const size_t sizes[10] = {0, v16, v16, v16, v16, 3 * s16, v16, 4 * (size_t)Vtot, s16, 2 * s16};
    size_t offs[11];
    size_t total = 0;
    for (int b = 1; b <= 9; ++b) { offs[b] = total; total += align256(sizes[b]); }
    offs[10] = total;
    total += align256(sizeof(DevSimConsts));
    const size_t healthOff = total;   // tfx_hair_count_nonfinite's two counters
    total += align256(2 * sizeof(unsigned long long));

    cudaError_t e = cudaMalloc(&h->arena, total);
    if (e != cudaSuccess) { h->arena = nullptr; hair_free(h); return cuda_fail(e, "tfx_hair_create: cudaMalloc"); }
    h->arenaBytes = total;
    char* base = (char*)h->arena;
    for (int b = 1; b <= 9; ++b) h->bufs[b] = {base + offs[b], sizes[b]};
    h->consts = (DevSimConsts*)(base + offs[10]);
    h->health = (unsigned long long*)(base + healthOff);
    for (int i = 0; i < 2; ++i) {
        e = cudaMallocHost((void**)&h->staging[i], sizeof(DevSimConsts));
        if (e != cudaSuccess) { h->staging[i] = nullptr; hair_free(h); return cuda_fail(e, "tfx_hair_create: cudaMallocHost"); }
        std::memset(h->staging[i], 0, sizeof(DevSimConsts));
        e = cudaEventCreateWithFlags(&h->stagingDone[i], cudaEventDisableTiming);
        if (e != cudaSuccess) { h->stagingDone[i] = nullptr; hair_free(h); return cuda_fail(e, "cudaEventCreate"); }
    }
    cudaStream_t s = ctx->stream;
    // UploadGPUData (TressFXHairObject.cpp:528-558): Pos, Tan, Prev and PrevPrev from the asset;
    // InitialPosition / RestLength / RootOffset / SkinningData SRVs (:116-120).
    const void* src[10] = {nullptr, positions, positions, positions, tangents, nullptr, positions, rest_lengths,
                           follow_root_offsets, bone_skinning};
    e = cudaMemsetAsync(h->arena, 0, total, s);
    for (int b = 1; b <= 9 && e == cudaSuccess; ++b)
        if (src[b]) e = cudaMemcpyAsync(h->bufs[b].ptr, src[b], sizes[b], cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { hair_free(h); return cuda_fail(e, "tfx_hair_create: upload"); }

    HairView& v = h->view;
    v.pos = (float4*)h->bufs[TFX_BUF_POSITIONS].ptr;
    v.prev = (float4*)h->bufs[TFX_BUF_POSITIONS_PREV].ptr;
    v.prevprev = (float4*)h->bufs[TFX_BUF_POSITIONS_PREV_PREV].ptr;
    v.tan = (float4*)h->bufs[TFX_BUF_TANGENTS].ptr;
    v.sld = (float4*)h->bufs[TFX_BUF_STRAND_LEVEL_DATA].ptr;
    v.init = (const float4*)h->bufs[TFX_BUF_INITIAL_POSITIONS].ptr;
    v.rest = (const float*)h->bufs[TFX_BUF_REST_LENGTHS].ptr;
    v.followOffset = (const float4*)h->bufs[TFX_BUF_FOLLOW_ROOT_OFFSETS].ptr;
    v.skin = (const float4*)h->bufs[TFX_BUF_BONE_SKINNING].ptr;
    v.consts = h->consts;
    v.G = h->G; v.n = h->n; v.F = h->F;
    *out = h;
    return TFX_OK;
}

extern "C" int tfx_hair_destroy(tfx_hair h) {
    if (!h) return TFX_OK;
    cudaSetDevice(h->ctx->device);
    cudaStreamSynchronize(h->ctx->stream);
    hair_free(h);
    return TFX_OK;
}

extern "C" int tfx_hair_update_constants(tfx_hair h, const tfx_sim_params* p, int num_bones) {
    if (!h || !p) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_hair_update_constants: null argument");
    if (num_bones < 0 || num_bones > TFX_MAX_BONES)
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_hair_update_constants: %d bones (max %d)", num_bones, TFX_MAX_BONES);
    if (p->counts[0] != TFX_THREAD_GROUP_SIZE / h->n || p->counts[1] != h->F || p->counts[2] != h->n)
        return fail(TFX_ERR_MISMATCH, "tfx_hair_update_constants: counts (%d,%d,%d) but object has (%d,%d,%d)", p->counts[0],
                    p->counts[1], p->counts[2], TFX_THREAD_GROUP_SIZE / h->n, h->F, h->n);
    const int slot = h->stagingNext;
    h->stagingNext ^= 1;
    if (h->stagingUsed[slot]) TFX_CUDA(cudaEventSynchronize(h->stagingDone[slot]), "cudaEventSynchronize");
    DevSimConsts* c = h->staging[slot];
    fill_consts_header(c, p, 0);
    std::memcpy(c->bones, p->bone_matrices, (size_t)num_bones * 64);
    const size_t bytes = offsetof(DevSimConsts, bones) + (size_t)num_bones * 64;
    TFX_CUDA(cudaSetDevice(h->ctx->device), "cudaSetDevice");
    TFX_CUDA(cudaMemcpyAsync(h->consts, c, bytes, cudaMemcpyHostToDevice, h->ctx->stream), "tfx_hair_update_constants: copy");
    TFX_CUDA(cudaEventRecord(h->stagingDone[slot], h->ctx->stream), "cudaEventRecord");
    h->stagingUsed[slot] = true;
    return TFX_OK;
}

static int dispatch_one(tfx_hair h, int kernel) {
    cudaStream_t s = h->ctx->stream;
    cudaError_t e;
    switch (kernel) {
        case TFX_KERNEL_INTEGRATION_AND_GLOBAL_SHAPE: e = launch_integrate(h->view, s); break;
        case TFX_KERNEL_STRAND_LEVEL_DATA: e = launch_strand_level(h->view, s); break;
        case TFX_KERNEL_VELOCITY_SHOCK_PROPAGATION: e = launch_vsp(h->view, s); break;
        case TFX_KERNEL_LOCAL_SHAPE_CONSTRAINTS: e = launch_local_shape(h->view, s); break;
        case TFX_KERNEL_LENGTH_WIND_COLLISION: e = launch_length_wind(h->view, s); break;
        case TFX_KERNEL_UPDATE_FOLLOW_HAIR: e = launch_follow(h->view, s); break;
        default: return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_hair_dispatch: kernel %d is not a simulation kernel", kernel);
    }
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    return TFX_OK;
}

extern "C" int tfx_hair_dispatch(tfx_hair h, int kernel, int repeat) {
    if (!h || repeat < 0) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_hair_dispatch: null object or negative repeat");
    TFX_CUDA(cudaSetDevice(h->ctx->device), "cudaSetDevice");
    for (int r = 0; r < repeat; ++r)
        if (int st = dispatch_one(h, kernel)) return st;
    return TFX_OK;
}

extern "C" int tfx_hair_simulate(tfx_hair h, int cpu_local_iterations) {
    if (!h || cpu_local_iterations < 0) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_hair_simulate: bad argument");
    TFX_CUDA(cudaSetDevice(h->ctx->device), "cudaSetDevice");
    static const int order[] = {TFX_KERNEL_INTEGRATION_AND_GLOBAL_SHAPE, TFX_KERNEL_STRAND_LEVEL_DATA,
                                TFX_KERNEL_VELOCITY_SHOCK_PROPAGATION};
    for (int k : order)
        if (int st = dispatch_one(h, k)) return st;
    for (int i = 0; i < cpu_local_iterations; ++i)
        if (int st = dispatch_one(h, TFX_KERNEL_LOCAL_SHAPE_CONSTRAINTS)) return st;
    if (int st = dispatch_one(h, TFX_KERNEL_LENGTH_WIND_COLLISION)) return st;
    return dispatch_one(h, TFX_KERNEL_UPDATE_FOLLOW_HAIR);
}

static int hair_buf(tfx_hair h, int b, size_t bytes, const char* who) {
    if (!h || b < 1 || b > 9) return fail(TFX_ERR_INVALID_ARGUMENT, "%s: bad object or buffer id %d", who, b);
    if (bytes > h->bufs[b].bytes)
        return fail(TFX_ERR_SIZE, "%s: %zu bytes requested, buffer %d holds %zu", who, bytes, b, h->bufs[b].bytes);
    return TFX_OK;
}

extern "C" int tfx_hair_read_async(tfx_hair h, int b, void* dst, size_t bytes) {
    if (int r = hair_buf(h, b, bytes, "tfx_hair_read")) return r;
    if (!dst && bytes) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_hair_read: null destination");
    TFX_CUDA(cudaSetDevice(h->ctx->device), "cudaSetDevice");
    TFX_CUDA(cudaMemcpyAsync(dst, h->bufs[b].ptr, bytes, cudaMemcpyDeviceToHost, h->ctx->stream), "tfx_hair_read: copy");
    return TFX_OK;
}
extern "C" int tfx_hair_write_async(tfx_hair h, int b, const void* srcp, size_t bytes) {
    if (int r = hair_buf(h, b, bytes, "tfx_hair_write")) return r;
    if (!srcp && bytes) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_hair_write: null source");
    if (b == TFX_BUF_BONE_SKINNING)
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_hair_write: the skinning buffer is fixed at creation (validated there)");
    TFX_CUDA(cudaSetDevice(h->ctx->device), "cudaSetDevice");
    TFX_CUDA(cudaMemcpyAsync(h->bufs[b].ptr, srcp, bytes, cudaMemcpyHostToDevice, h->ctx->stream), "tfx_hair_write: copy");
    return TFX_OK;
}
extern "C" int tfx_hair_read(tfx_hair h, int b, void* dst, size_t bytes) {
    if (int r = tfx_hair_read_async(h, b, dst, bytes)) return r;
    TFX_CUDA(cudaStreamSynchronize(h->ctx->stream), "cudaStreamSynchronize");
    return TFX_OK;
}
extern "C" int tfx_hair_write(tfx_hair h, int b, const void* srcp, size_t bytes) {
    if (int r = tfx_hair_write_async(h, b, srcp, bytes)) return r;
    TFX_CUDA(cudaStreamSynchronize(h->ctx->stream), "cudaStreamSynchronize");
    return TFX_OK;
}
extern "C" int tfx_hair_get_buffer(tfx_hair h, int b, void** ptr, size_t* bytes) {
    if (int r = hair_buf(h, b, 0, "tfx_hair_get_buffer")) return r;
    if (ptr) *ptr = h->bufs[b].ptr;
    if (bytes) *bytes = h->bufs[b].bytes;
    return TFX_OK;
}
extern "C" int tfx_hair_get_counts(tfx_hair h, int32_t out[4]) {
    if (!h || !out) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_hair_get_counts: null argument");
    out[0] = (int32_t)h->Vtot; out[1] = (int32_t)h->Stot; out[2] = h->n; out[3] = h->F;
    return TFX_OK;
}

// ============================================================================ strand quads
extern "C" int tfx_hair_expand_strands(tfx_hair h, const tfx_strand_params* p, const float eye[3], const float win[2],
                                       const float vp[16], int shadow, void* out) {
    if (!h || !p || !eye || !win || !vp || !out) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_hair_expand_strands: null argument");
    if (p->num_vertices_per_strand != h->n)
        return fail(TFX_ERR_MISMATCH, "tfx_hair_expand_strands: %d vertices per strand, object has %d", p->num_vertices_per_strand, h->n);
    if (((uintptr_t)out & 15) != 0) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_hair_expand_strands: output not 16-byte aligned");
    ExpandParams P{};
    for (int k = 0; k < 4; ++k) { P.baseColor[k] = p->mat_base_color[k]; P.tipColor[k] = p->mat_tip_color[k]; }
    P.tipPercentage = p->tip_percentage; P.fiberRatio = p->fiber_ratio; P.fiberRadius = p->fiber_radius;
    P.n = h->n; P.enableThinTip = p->enable_thin_tip; P.shadow = shadow ? 1 : 0;
    for (int k = 0; k < 3; ++k) P.eye[k] = eye[k];
    P.winH = win[1];
    for (int k = 0; k < 16; ++k) P.viewProj[k] = vp[k];
    TFX_CUDA(cudaSetDevice(h->ctx->device), "cudaSetDevice");
    cudaError_t e = launch_expand_strands(h->view.pos, h->view.tan, h->Vtot, P, static_cast<float4*>(out), h->ctx->stream);
    return e == cudaSuccess ? TFX_OK : cuda_fail(e, "tfx_hair_expand_strands launch");
}

// ============================================================================ SDF
extern "C" int tfx_sdf_create(tfx_context ctx, int64_t alloc_cells, tfx_sdf* out) {
    if (!out) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_sdf_create: out is null");
    *out = nullptr;
    if (!ctx || alloc_cells <= 0) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_sdf_create: null context or %lld cells", (long long)alloc_cells);
    TFX_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    auto* s = new (std::nothrow) tfx_sdf_t();
    if (!s) return fail(TFX_ERR_OUT_OF_MEMORY, "tfx_sdf_create: host allocation");
    s->ctx = ctx;
    s->alloc = alloc_cells;
    cudaError_t e = cudaMalloc(&s->grid, align256(4 * (size_t)alloc_cells));
    if (e != cudaSuccess) { delete s; return cuda_fail(e, "tfx_sdf_create: cudaMalloc"); }
    e = cudaMemsetAsync(s->grid, 0, 4 * (size_t)alloc_cells, ctx->stream);
    if (e != cudaSuccess) { cudaFree(s->grid); delete s; return cuda_fail(e, "tfx_sdf_create: memset"); }
    context_retain(ctx);
    *out = s;
    return TFX_OK;
}

extern "C" int tfx_sdf_destroy(tfx_sdf s) {
    if (!s) return TFX_OK;
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    cudaFree(s->grid);
    context_release(s->ctx);
    delete s;
    return TFX_OK;
}

extern "C" int tfx_sdf_set_mesh(tfx_sdf s, const void* mesh, int nverts, const uint32_t* idx, int ntri) {
    if (!s || nverts < 0 || ntri < 0 || (ntri > 0 && (!mesh || !idx)))
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_sdf_set_mesh: bad argument");
    if (((uintptr_t)mesh & 15) != 0) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_sdf_set_mesh: mesh buffer not 16-byte aligned");
    s->mesh = (const float4*)mesh; s->nverts = nverts; s->idx = idx; s->ntri = ntri;
    return TFX_OK;
}

static int check_grid(tfx_sdf s, const tfx_sdf_grid* g, SdfGrid* out, const char* who) {
    if (!s || !g) return fail(TFX_ERR_INVALID_ARGUMENT, "%s: null argument", who);
    if (g->num_cells_x <= 0 || g->num_cells_y <= 0 || g->num_cells_z <= 0 || !(g->cell_size > 0.0f))
        return fail(TFX_ERR_INVALID_ARGUMENT, "%s: grid %dx%dx%d cell %g", who, g->num_cells_x, g->num_cells_y, g->num_cells_z,
                    (double)g->cell_size);
    const int64_t cells = (int64_t)g->num_cells_x * g->num_cells_y * g->num_cells_z;
    if (cells > s->alloc) return fail(TFX_ERR_SIZE, "%s: grid of %lld cells exceeds allocation of %lld", who, (long long)cells, (long long)s->alloc);
    *out = SdfGrid{g->origin[0], g->origin[1], g->origin[2], g->cell_size, g->num_cells_x, g->num_cells_y, g->num_cells_z, 0};
    return TFX_OK;
}

static int sdf_kernel(tfx_sdf s, int kernel, const SdfGrid& g) {
    const int64_t cells = (int64_t)g.nx * g.ny * g.nz;
    cudaError_t e;
    switch (kernel) {
        case TFX_KERNEL_SDF_INITIALIZE: e = launch_sdf_initialize(s->grid, cells, s->ctx->stream); break;
        case TFX_KERNEL_SDF_CONSTRUCT:
            if (s->ntri > 0 && !s->mesh) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_sdf: no collision mesh bound");
            e = launch_sdf_construct(s->grid, g, s->mesh, s->idx, s->ntri, s->ctx->stream);
            break;
        case TFX_KERNEL_SDF_FINALIZE: e = launch_sdf_finalize(s->grid, cells, s->ctx->stream); break;
        default: return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_sdf_dispatch: kernel %d is not an SDF build kernel", kernel);
    }
    if (e != cudaSuccess) return cuda_fail(e, "SDF kernel launch");
    return TFX_OK;
}

extern "C" int tfx_sdf_dispatch(tfx_sdf s, int kernel, const tfx_sdf_grid* grid) {
    SdfGrid g;
    if (int r = check_grid(s, grid, &g, "tfx_sdf_dispatch")) return r;
    TFX_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    return sdf_kernel(s, kernel, g);
}

extern "C" int tfx_sdf_update(tfx_sdf s, const tfx_sdf_grid* grid) {
    SdfGrid g;
    if (int r = check_grid(s, grid, &g, "tfx_sdf_update")) return r;
    TFX_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    if (int r = sdf_kernel(s, TFX_KERNEL_SDF_INITIALIZE, g)) return r;
    if (int r = sdf_kernel(s, TFX_KERNEL_SDF_CONSTRUCT, g)) return r;
    return sdf_kernel(s, TFX_KERNEL_SDF_FINALIZE, g);
}

extern "C" int tfx_sdf_collide(tfx_sdf s, tfx_hair h, const tfx_sdf_grid* grid, float margin_world) {
    SdfGrid g;
    if (int r = check_grid(s, grid, &g, "tfx_sdf_collide")) return r;
    if (!h) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_sdf_collide: null hair object");
    if (h->ctx != s->ctx) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_sdf_collide: hair and SDF live on different contexts");
    TFX_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    cudaError_t e = launch_sdf_collide(s->grid, g, margin_world, h->view.pos, h->view.prev, h->n, h->Vtot, s->ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "SDF collide launch");
    return TFX_OK;
}

extern "C" int tfx_sdf_collide_mixed(tfx_sdf s, tfx_hair h, const tfx_sdf_grid* grid, float margin_world) {
    SdfGrid g;
    if (int r = check_grid(s, grid, &g, "tfx_sdf_collide_mixed")) return r;
    if (!h) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_sdf_collide_mixed: null hair");
    TFX_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    cudaError_t e = launch_sdf_collide_mixed(s->grid, g, margin_world, h->view.pos, h->view.prev, h->Vtot, s->ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "SDF mixed collide launch");
    return TFX_OK;
}
extern "C" int tfx_sdf_read(tfx_sdf s, void* dst, size_t bytes) {
    if (!s || (!dst && bytes)) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_sdf_read: bad argument");
    if (bytes > 4 * (size_t)s->alloc) return fail(TFX_ERR_SIZE, "tfx_sdf_read: %zu bytes > allocation", bytes);
    TFX_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    TFX_CUDA(cudaMemcpyAsync(dst, s->grid, bytes, cudaMemcpyDeviceToHost, s->ctx->stream), "tfx_sdf_read");
    TFX_CUDA(cudaStreamSynchronize(s->ctx->stream), "cudaStreamSynchronize");
    return TFX_OK;
}
extern "C" int tfx_sdf_write(tfx_sdf s, const void* srcp, size_t bytes) {
    if (!s || (!srcp && bytes)) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_sdf_write: bad argument");
    if (bytes > 4 * (size_t)s->alloc) return fail(TFX_ERR_SIZE, "tfx_sdf_write: %zu bytes > allocation", bytes);
    TFX_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    TFX_CUDA(cudaMemcpyAsync(s->grid, srcp, bytes, cudaMemcpyHostToDevice, s->ctx->stream), "tfx_sdf_write");
    TFX_CUDA(cudaStreamSynchronize(s->ctx->stream), "cudaStreamSynchronize");
    return TFX_OK;
}
extern "C" int tfx_sdf_get_buffer(tfx_sdf s, void** ptr, size_t* bytes) {
    if (!s) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_sdf_get_buffer: null argument");
    if (ptr) *ptr = s->grid;
    if (bytes) *bytes = 4 * (size_t)s->alloc;
    return TFX_OK;
}

// ============================================================================ collision mesh
extern "C" int tfx_mesh_destroy(tfx_mesh m) {
    if (!m) return TFX_OK;
    cudaSetDevice(m->ctx->device);
    cudaStreamSynchronize(m->ctx->stream);
    if (m->arena) cudaFree(m->arena);
    for (int i = 0; i < 2; ++i) {
        if (m->staging[i]) cudaFreeHost(m->staging[i]);
        if (m->stagingDone[i]) cudaEventDestroy(m->stagingDone[i]);
    }
    context_release(m->ctx);
    delete m;
    return TFX_OK;
}

extern "C" int tfx_mesh_create(tfx_context ctx, const float* vertices, int nverts, const uint32_t* indices, int ntri,
                               const float* skinning, tfx_mesh* out) {
    if (!out) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mesh_create: out is null");
    *out = nullptr;
    if (!ctx || !vertices || !indices || !skinning || nverts <= 0 || ntri <= 0)
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mesh_create: bad argument");
    for (int64_t i = 0; i < 3 * (int64_t)ntri; ++i)
        if (indices[i] >= (uint32_t)nverts)
            return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mesh_create: index %u at %lld >= %d vertices", indices[i], (long long)i, nverts);
    int maxBone = 0;
    if (int r = validate_skinning(skinning, nverts, 1, "tfx_mesh_create", &maxBone)) return r;
    TFX_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    auto* m = new (std::nothrow) tfx_mesh_t();
    if (!m) return fail(TFX_ERR_OUT_OF_MEMORY, "tfx_mesh_create: host allocation");
    m->ctx = ctx; m->nverts = nverts; m->ntri = ntri; m->maxBone = maxBone;
    context_retain(ctx);
    const size_t vb = 32 * (size_t)nverts, ib = 12 * (size_t)ntri, bb = 64 * (size_t)TFX_MAX_BONES;
    const size_t total = 3 * align256(vb) + align256(ib) + align256(bb);
    cudaError_t e = cudaMalloc(&m->arena, total);
    if (e != cudaSuccess) { m->arena = nullptr; tfx_mesh_destroy(m); return cuda_fail(e, "tfx_mesh_create: cudaMalloc"); }
    char* b = (char*)m->arena;
    m->bind = (float4*)b; b += align256(vb);
    m->skinned = (float4*)b; b += align256(vb);
    m->skin = (float4*)b; b += align256(vb);
    m->idx = (uint32_t*)b; b += align256(ib);
    m->bones = (float4*)b;
    for (int i = 0; i < 2; ++i) {
        e = cudaMallocHost((void**)&m->staging[i], bb);
        if (e != cudaSuccess) { m->staging[i] = nullptr; tfx_mesh_destroy(m); return cuda_fail(e, "cudaMallocHost"); }
        e = cudaEventCreateWithFlags(&m->stagingDone[i], cudaEventDisableTiming);
        if (e != cudaSuccess) { m->stagingDone[i] = nullptr; tfx_mesh_destroy(m); return cuda_fail(e, "cudaEventCreate"); }
    }
    cudaStream_t s = ctx->stream;
    e = cudaMemsetAsync(m->bones, 0, bb, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(m->bind, vertices, vb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(m->skinned, vertices, vb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(m->skin, skinning, vb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(m->idx, indices, ib, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { tfx_mesh_destroy(m); return cuda_fail(e, "tfx_mesh_create: upload"); }
    *out = m;
    return TFX_OK;
}

extern "C" int tfx_mesh_skin(tfx_mesh m, const float* bone_matrices, int num_bones) {
    if (!m || num_bones < 0 || num_bones > TFX_MAX_BONES || (num_bones > 0 && !bone_matrices))
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mesh_skin: bad argument");
    TFX_CUDA(cudaSetDevice(m->ctx->device), "cudaSetDevice");
    if (num_bones > 0) {
        const int slot = m->stagingNext;
        m->stagingNext ^= 1;
        if (m->stagingUsed[slot]) TFX_CUDA(cudaEventSynchronize(m->stagingDone[slot]), "cudaEventSynchronize");
        std::memcpy(m->staging[slot], bone_matrices, 64 * (size_t)num_bones);
        TFX_CUDA(cudaMemcpyAsync(m->bones, m->staging[slot], 64 * (size_t)num_bones, cudaMemcpyHostToDevice, m->ctx->stream),
                 "tfx_mesh_skin: bone upload");
        TFX_CUDA(cudaEventRecord(m->stagingDone[slot], m->ctx->stream), "cudaEventRecord");
        m->stagingUsed[slot] = true;
    }
    cudaError_t e = launch_mesh_skin(m->skinned, m->bind, m->skin, m->bones, m->nverts, m->ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "BoneSkinning launch");
    return TFX_OK;
}

extern "C" int tfx_mesh_get_buffers(tfx_mesh m, void** skinned, void** indices, int32_t* nverts, int32_t* ntri) {
    if (!m) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mesh_get_buffers: null mesh");
    if (skinned) *skinned = m->skinned;
    if (indices) *indices = m->idx;
    if (nverts) *nverts = m->nverts;
    if (ntri) *ntri = m->ntri;
    return TFX_OK;
}

extern "C" int tfx_mesh_read_skinned(tfx_mesh m, float* dst, size_t bytes) {
    if (!m || (!dst && bytes)) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_mesh_read_skinned: bad argument");
    if (bytes > 32 * (size_t)m->nverts) return fail(TFX_ERR_SIZE, "tfx_mesh_read_skinned: %zu bytes too many", bytes);
    TFX_CUDA(cudaSetDevice(m->ctx->device), "cudaSetDevice");
    TFX_CUDA(cudaMemcpyAsync(dst, m->skinned, bytes, cudaMemcpyDeviceToHost, m->ctx->stream), "tfx_mesh_read_skinned");
    TFX_CUDA(cudaStreamSynchronize(m->ctx->stream), "cudaStreamSynchronize");
    return TFX_OK;
}
