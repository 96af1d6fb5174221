// C ABI of the batched path (tfx_batch_*): many hair objects and their SDFs advance one frame per
// tfx_batch_run, which is one CUDA-graph launch.
//
// Frame layout.  Everything a frame needs from the host (each object's simulation constants and
// bone matrices, each SDF's grid and margin, each collision mesh's bone matrices) lives in one
// "frame block".  The caller fills a host copy with tfx_batch_set_*; tfx_batch_run copies it into
// one of two pinned blocks and launches the graph that was captured for that block: its first
// node uploads the block, then come the mesh skinning, the SDF rebuild and one fused strand launch
// per vertices-per-strand class.  The two pinned blocks alternate, so the host can prepare frame
// f+1 while frame f runs; an event per block keeps a block from being rewritten before its upload
// has executed.
//
// Autotuning.  tfx_batch_autotune(b, frames) times the candidate launch shapes (vertices per lane
// and warps per block of every fused class, the form of its follow/collide kernel, block size of the
// SDF construct) on the real objects,
// restores every state buffer it touched, and recaptures the graphs with the fastest shape of each
// part.  All shapes give the same bits; only the speed differs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "tfx_batch.h"
#include "tfx_handles.h"

using namespace tfx;

struct BatchClass {
    int n = 0;
    int vpl = 2, warps = 4, blocks = 1;
    int perSMCap = 0;            // resident strand blocks per SM allowed (0 = as many as fit)
    int followBlocks = 1;        // grid of k_follow_collide (persistent over the chunks)
    int followChunks = 1;        // chunks per group in k_follow_collide
    int followMode = 0;          // FollowLaunch::queued.  Default, from measurements: 1 when an object of the
                                 // class has follow hairs, else 2 at n >= 64 (long strands: lanes of one warp
                                 // reach both surface and far vertices), else 0; the autotuner tries the others
    bool splitSweeps = false;    // local-shape sweeps in k_local_sweep between two strand passes
    bool noFollow = false;       // no object of the class has follow hairs
    std::vector<WorkItem> hostItems;
    WorkItem* items = nullptr;  // device
    int numItems = 0;
};

// Frames tfx_batch_run can queue ahead of the GPU (pinned frame blocks and graph instances).
constexpr int kFrameSlots = 8;

struct tfx_batch_t {
    tfx_context ctx = nullptr;
    std::vector<tfx_hair> hairs;
    std::vector<int> hairSdf;
    std::vector<std::vector<int>> hairMoreSdf;   // per hair object: further SDFs, in collision order
    std::vector<BatchCollide*> levelPairs;       // per collision level: its pairs on the device
    std::vector<int> levelCount;
    std::vector<long long> levelVertices;
    std::vector<bool> hairSet;
    std::vector<tfx_sdf> sdfs;
    std::vector<tfx_mesh> sdfMesh;
    std::vector<int> sdfDims;  // 3 per SDF
    std::vector<bool> sdfSet;
    bool built = false;

    // frame block
    size_t blockBytes = 0;
    std::vector<size_t> objOff, sdfOff, meshOff;
    std::vector<int> objBones, meshBones;
    std::vector<char> staging;
    // kFrameSlots frame blocks in pinned memory, each with its graph instance: tfx_batch_run may run
    // that many frames ahead of the GPU, so a pause of the calling thread shorter than the frames
    // already queued leaves the GPU busy
    char* pinned[kFrameSlots] = {};
    char* devBlock = nullptr;
    cudaEvent_t done[kFrameSlots] = {};
    bool used[kFrameSlots] = {};
    int slot = 0;

    // device tables
    void* devArena = nullptr;
    void* expandedArena = nullptr;   // corner-expanded copies of the SDF grids
    int expandMode = 2;              // TFX_BATCH_EXPANDED_GRIDS: 0 never, 1 always, 2 where lookups >= 4 per cell
    std::vector<float4*> sdfExpanded;   // per SDF: its slot in expandedArena
    void* expTable = nullptr;        // SdfBatchLaunch::expSdf / expFirst
    BatchObject* objTable = nullptr;
    BatchMesh* meshTable = nullptr;
    BatchSdf* sdfTable = nullptr;
    int nmeshes = 0, totalMeshVerts = 0;
    std::vector<BatchClass> classes;
    SdfBatchLaunch sdfL{};
    SdfTileLaunch sdfT{};           // the tiled construct's tables
    void* tileArena = nullptr;
    int sdfForm = 0;                // TFX_BATCH_SDF_FORM: 0 one warp per triangle, 1 tiles (when the grids allow)
    bool tilesAvailable = false;

    cudaStream_t side = nullptr;             // second capture branch: mesh skinning + SDF build
    bool overlap = true;                     // capture the SDF branch on `side`
    cudaEvent_t evFork = nullptr, evJoin = nullptr;
    // with `overlap`, each n class's strand and follow/collide kernels form their own branch too (the
    // classes touch disjoint objects), so one class's last blocks run beside the next class's
    cudaStream_t classStream[5] = {};
    cudaEvent_t evClasses = nullptr, evClassDone[5] = {};
    int* devErr = nullptr;      // fused kernel: a block gave up waiting for its bulk copies
    int* pinnedErr = nullptr;   // its copy at the end of each frame, one word per slot
    int waitPolls = kFusedWaitPollsDefault;   // TFX_BATCH_WAIT_POLLS

    cudaGraphExec_t graph[kFrameSlots] = {};
    int launchesPerFrame = 0;
    std::string description;

    // tfx_batch_readback: two device snapshots of every object's positions, copied to the host on
    // `copy` while the next frames run
    cudaStream_t copy = nullptr;
    char* snap[2] = {nullptr, nullptr};
    std::vector<long long> snapFirst;  // per hair object: its first vertex in a snapshot
    long long* devFirst = nullptr;     // the same, on the device
    long long snapVerts = 0;
    cudaEvent_t snapDone[2] = {nullptr, nullptr}, copyDone[2] = {nullptr, nullptr};
    bool copyUsed[2] = {false, false};
    int64_t nextTicket = 0;
};

static int batch_fail_built(const char* who) { return fail(TFX_ERR_INVALID_ARGUMENT, "%s: the batch is already built", who); }

// A frame's fused strand kernel gave up waiting for its bulk copies: waits for the frames queued so
// far, clears the device flag and both frames' copies of it (so the report is made once), and
// returns TFX_ERR_TIMEOUT.  The state of the failed frame is undefined; the caller restores it
// (tfx_hair_write) or resets the objects.
static int report_timeout(tfx_batch b) {
    cudaSetDevice(b->ctx->device);
    cudaError_t e = cudaStreamSynchronize(b->ctx->stream);
    if (e == cudaSuccess) e = cudaMemset(b->devErr, 0, sizeof(int));
    if (e != cudaSuccess) return cuda_fail(e, "tfx_batch: clearing the error flag");
    for (int i = 0; i < kFrameSlots; ++i) b->pinnedErr[i] = 0;
    return fail(TFX_ERR_TIMEOUT, "tfx_batch: a fused strand block gave up waiting for its bulk copies");
}

extern "C" int tfx_batch_create(tfx_context ctx, tfx_batch* out) {
    if (!out || !ctx) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_create: null argument");
    auto* b = new (std::nothrow) tfx_batch_t();
    if (!b) return fail(TFX_ERR_OUT_OF_MEMORY, "tfx_batch_create: host allocation");
    b->ctx = ctx;
    context_retain(ctx);
    *out = b;
    return TFX_OK;
}

extern "C" int tfx_batch_destroy(tfx_batch b) {
    if (!b) return TFX_OK;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    for (int i = 0; i < kFrameSlots; ++i) {
        if (b->graph[i]) cudaGraphExecDestroy(b->graph[i]);
        if (b->pinned[i]) cudaFreeHost(b->pinned[i]);
        if (b->done[i]) cudaEventDestroy(b->done[i]);
    }
    if (b->copy) cudaStreamSynchronize(b->copy);
    for (int i = 0; i < 2; ++i) {
        if (b->snap[i]) cudaFree(b->snap[i]);
        if (b->snapDone[i]) cudaEventDestroy(b->snapDone[i]);
        if (b->copyDone[i]) cudaEventDestroy(b->copyDone[i]);
    }
    if (b->copy) cudaStreamDestroy(b->copy);
    if (b->devFirst) cudaFree(b->devFirst);
    if (b->pinnedErr) cudaFreeHost(b->pinnedErr);
    if (b->evFork) cudaEventDestroy(b->evFork);
    if (b->evJoin) cudaEventDestroy(b->evJoin);
    if (b->side) cudaStreamDestroy(b->side);
    for (int i = 0; i < 5; ++i) {
        if (b->classStream[i]) cudaStreamDestroy(b->classStream[i]);
        if (b->evClassDone[i]) cudaEventDestroy(b->evClassDone[i]);
    }
    if (b->evClasses) cudaEventDestroy(b->evClasses);
    if (b->devBlock) cudaFree(b->devBlock);
    if (b->devArena) cudaFree(b->devArena);
    if (b->expandedArena) cudaFree(b->expandedArena);
    if (b->expTable) cudaFree(b->expTable);
    if (b->tileArena) cudaFree(b->tileArena);
    for (auto t : b->levelPairs)
        if (t) cudaFree(t);
    for (auto& c : b->classes)
        if (c.items) cudaFree(c.items);
    for (auto h : b->hairs) context_release(h->ctx);
    for (auto s : b->sdfs) context_release(s->ctx);
    for (auto m : b->sdfMesh)
        if (m) context_release(m->ctx);
    context_release(b->ctx);
    delete b;
    return TFX_OK;
}

extern "C" int tfx_batch_add_sdf(tfx_batch b, tfx_sdf sdf, tfx_mesh mesh, int nx, int ny, int nz, int* index) {
    if (!b || !sdf) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_add_sdf: null argument");
    if (b->built) return batch_fail_built("tfx_batch_add_sdf");
    if (sdf->ctx != b->ctx || (mesh && mesh->ctx != b->ctx))
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_add_sdf: objects of another context");
    if (nx <= 0 || ny <= 0 || nz <= 0 || (int64_t)nx * ny * nz > sdf->alloc)
        return fail(TFX_ERR_SIZE, "tfx_batch_add_sdf: grid %dx%dx%d does not fit the SDF allocation", nx, ny, nz);
    if (!mesh && (!sdf->mesh || sdf->ntri <= 0))
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_add_sdf: no mesh given and none bound to the SDF");
    for (auto s : b->sdfs)
        if (s == sdf) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_add_sdf: SDF added twice");
    context_retain(sdf->ctx);
    if (mesh) context_retain(mesh->ctx);
    b->sdfs.push_back(sdf);
    b->sdfMesh.push_back(mesh);
    b->sdfDims.insert(b->sdfDims.end(), {nx, ny, nz});
    b->sdfSet.push_back(false);
    if (index) *index = (int)b->sdfs.size() - 1;
    return TFX_OK;
}

extern "C" int tfx_batch_add_hair(tfx_batch b, tfx_hair hair, int sdf_index, int* index) {
    if (!b || !hair) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_add_hair: null argument");
    if (b->built) return batch_fail_built("tfx_batch_add_hair");
    if (hair->ctx != b->ctx) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_add_hair: object of another context");
    if (sdf_index < -1 || sdf_index >= (int)b->sdfs.size())
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_add_hair: SDF index %d of %zu", sdf_index, b->sdfs.size());
    for (auto h : b->hairs)
        if (h == hair) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_add_hair: object added twice");
    context_retain(hair->ctx);
    b->hairs.push_back(hair);
    b->hairSdf.push_back(sdf_index);
    b->hairMoreSdf.emplace_back();
    b->hairSet.push_back(false);
    if (index) *index = (int)b->hairs.size() - 1;
    return TFX_OK;
}

extern "C" int tfx_batch_add_hair_collision(tfx_batch b, int hair_index, int sdf_index) {
    if (!b) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_add_hair_collision: null batch");
    if (b->built) return batch_fail_built("tfx_batch_add_hair_collision");
    if (hair_index < 0 || hair_index >= (int)b->hairs.size())
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_add_hair_collision: hair index %d of %zu", hair_index,
                    b->hairs.size());
    if (sdf_index < 0 || sdf_index >= (int)b->sdfs.size())
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_add_hair_collision: SDF index %d of %zu", sdf_index,
                    b->sdfs.size());
    if (b->hairSdf[hair_index] < 0)
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_add_hair_collision: hair object %d was added without an SDF",
                    hair_index);
    auto& more = b->hairMoreSdf[hair_index];
    if (sdf_index == b->hairSdf[hair_index] || std::find(more.begin(), more.end(), sdf_index) != more.end())
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_add_hair_collision: hair object %d already collides with SDF %d",
                    hair_index, sdf_index);
    more.push_back(sdf_index);
    return TFX_OK;
}

// ---------------------------------------------------------------------------------------------
static size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

static void describe(tfx_batch b) {
    char buf[1024];
    int k = b->sdfForm == 1 ? snprintf(buf, sizeof(buf), "sdf construct on 8x8x4-cell tiles (a warp per 4x4x2 brick), %d blocks;", b->sdfT.blocks)
                            : snprintf(buf, sizeof(buf), "sdf construct %d threads/block;", b->sdfL.constructThreads);
    for (auto& c : b->classes)
        k += snprintf(buf + k, sizeof(buf) - k, " n=%d: %d vertices/lane, %d warps/block, %d blocks, %d groups of %d%s%s;",
                      c.n, c.vpl, c.warps, c.blocks, c.numItems, fused_group_size(c.n),
                      c.splitSweeps ? ", sweeps in their own launch" : "",
                      c.followMode == 1 ? ", collide on per-warp lookup queues"
                                         : c.followMode == 2 ? ", gradient lookups on per-warp queues" : "");
    k += snprintf(buf + k, sizeof(buf) - k, " SDF build %s the strand kernels%s;",
                  b->overlap ? "concurrent with" : "before", b->sdfL.expand ? ", lookups on corner-expanded grids" : "");
    b->description = buf;
}

static void make_items(tfx_batch b, BatchClass& c) {
    c.hostItems.clear();
    c.followMode = c.n >= 64 ? 2 : 0;
    c.noFollow = true;
    for (int o = 0; o < (int)b->hairs.size(); ++o) {
        tfx_hair h = b->hairs[o];
        if (h->n != c.n) continue;
        if (h->F > 0) { c.followMode = 1; c.noFollow = false; }
        const int gsz = fused_group_size(c.n);
        for (int g = 0; g < h->G; g += gsz) c.hostItems.push_back(WorkItem{o, g, std::min(gsz, h->G - g), 0});
    }
    c.numItems = (int)c.hostItems.size();
}

static int upload_items(BatchClass& c) {
    if (c.items) { cudaFree(c.items); c.items = nullptr; }
    if (c.numItems == 0) return TFX_OK;
    TFX_CUDA(cudaMalloc(&c.items, sizeof(WorkItem) * c.numItems), "tfx_batch: cudaMalloc items");
    TFX_CUDA(cudaMemcpy(c.items, c.hostItems.data(), sizeof(WorkItem) * c.numItems, cudaMemcpyHostToDevice),
             "tfx_batch: upload items");
    return TFX_OK;
}

// Grid of a fused class: as many resident blocks as fit (persistent), no more than groups.
static int size_class(tfx_batch b, BatchClass& c) {
    int perSM = fused_blocks_per_sm(c.n, c.vpl, c.warps);
    if (perSM <= 0)
        return fail(TFX_ERR_CUDA, "tfx_batch: fused kernel n=%d vpl=%d with %d warps cannot be resident", c.n, c.vpl, c.warps);
    if (c.perSMCap > 0) perSM = std::min(perSM, c.perSMCap);
    c.blocks = std::max(1, std::min(perSM * b->ctx->numSMs, c.numItems));
    // follow/collide: whole groups when every resident block gets at least four, else the smallest chunks
    const int fResident = std::max(1, follow_blocks_per_sm(c.n, c.followMode, c.noFollow)) * b->ctx->numSMs;
    c.followChunks = c.numItems >= 4 * fResident ? 1 : follow_max_chunks_per_item(c.n);
    c.followBlocks = std::max(1, std::min(fResident, c.numItems * c.followChunks));
    return TFX_OK;
}

static int launch_sdf_part(tfx_batch b, cudaStream_t s) {
    if (b->totalMeshVerts > 0) {
        cudaError_t e = launch_batch_mesh_skin(b->meshTable, b->nmeshes, b->totalMeshVerts, s);
        if (e != cudaSuccess) return cuda_fail(e, "tfx_batch: mesh skinning launch");
    }
    if (!b->sdfs.empty()) {
        cudaError_t e;
        if (b->sdfForm == 1) {
            e = launch_sdf_tiles(b->sdfT, s);
            if (e == cudaSuccess) e = launch_batch_sdf_expand(b->sdfL, s);
        } else {
            e = launch_batch_sdf(b->sdfL, s);
        }
        if (e != cudaSuccess) return cuda_fail(e, "tfx_batch: SDF launch");
    }
    return TFX_OK;
}

static int launch_strands(tfx_batch b, BatchClass& c, cudaStream_t s) {
    FusedLaunch fl{c.n, c.vpl, c.warps, c.blocks, b->objTable, c.items, c.numItems, b->devErr, 0, b->waitPolls};
    cudaError_t e;
    if (!c.splitSweeps) {
        e = launch_fused_strands(fl, s);
    } else {   // the sweeps as their own launch, between the two halves of the strand kernel
        fl.mode = 1;
        e = launch_fused_strands(fl, s);
        if (e == cudaSuccess) e = launch_local_sweep(fl, s);
        fl.mode = 2;
        if (e == cudaSuccess) e = launch_fused_strands(fl, s);
    }
    return e == cudaSuccess ? TFX_OK : cuda_fail(e, "tfx_batch: fused strand launch");
}

static int launch_follows(tfx_batch b, BatchClass& c, cudaStream_t s) {
    FollowLaunch fl{c.n, c.followBlocks, b->objTable, c.items, c.numItems, c.followChunks, c.followMode,
                    c.noFollow ? 1 : 0};
    cudaError_t e = launch_follow_collide(fl, s);
    return e == cudaSuccess ? TFX_OK : cuda_fail(e, "tfx_batch: follow/collide launch");
}

// The objects' further SDFs, level by level, after every follow/collide launch.
static int launch_collide_levels(tfx_batch b, cudaStream_t s) {
    for (size_t k = 0; k < b->levelPairs.size(); ++k) {
        cudaError_t e = launch_collide_level(b->objTable, b->sdfTable, b->levelPairs[k], b->levelCount[k],
                                             b->levelVertices[k], s);
        if (e != cudaSuccess) return cuda_fail(e, "tfx_batch: collision level launch");
    }
    return TFX_OK;
}

// One frame as direct launches, in dependency order on one stream, with an event after each part:
// part 0 = mesh skinning + SDF build, then one part per class for k_fused_strands, then one per
// class for k_follow_collide (used by profiling).
static int launch_frame_direct(tfx_batch b, cudaStream_t s, std::vector<float>* partMs) {
    std::vector<cudaEvent_t> ev;
    auto mark = [&]() {
        if (!partMs) return;
        cudaEvent_t e;
        cudaEventCreate(&e);
        cudaEventRecord(e, s);
        ev.push_back(e);
    };
    mark();
    if (int r = launch_sdf_part(b, s)) return r;
    mark();
    for (auto& c : b->classes) {
        if (c.numItems == 0) continue;
        if (int r = launch_strands(b, c, s)) return r;
        mark();
    }
    for (auto& c : b->classes) {
        if (c.numItems == 0) continue;
        if (int r = launch_follows(b, c, s)) return r;
        mark();
    }
    if (!b->levelPairs.empty()) {
        if (int r = launch_collide_levels(b, s)) return r;
        mark();
    }
    if (partMs) {
        cudaEventSynchronize(ev.back());
        int flag = 0;
        cudaMemcpy(&flag, b->devErr, sizeof(int), cudaMemcpyDeviceToHost);
        if (flag) {
            for (auto e : ev) cudaEventDestroy(e);
            return report_timeout(b);
        }
        partMs->clear();
        for (size_t i = 1; i < ev.size(); ++i) {
            float t = 0.f;
            cudaEventElapsedTime(&t, ev[i - 1], ev[i]);
            partMs->push_back(t);
        }
        for (auto e : ev) cudaEventDestroy(e);
    }
    return TFX_OK;
}

// The frame body as captured into the graph: the SDF branch (mesh skinning + SDF build) on the side
// stream runs concurrently with the strand kernels, which need no SDF; k_follow_collide waits for both.
// With `overlap` every n class is a branch of its own (its strand kernel, then, once the SDFs are
// built, its follow/collide kernel); the further-mesh levels follow all of them.
static int launch_frame_forked(tfx_batch b, cudaStream_t s) {
    const bool fork = b->overlap && b->side && !b->sdfs.empty();
    if (fork) {
        TFX_CUDA(cudaEventRecord(b->evFork, s), "tfx_batch: fork");
        TFX_CUDA(cudaStreamWaitEvent(b->side, b->evFork, 0), "tfx_batch: fork");
        if (int r = launch_sdf_part(b, b->side)) return r;
        TFX_CUDA(cudaEventRecord(b->evJoin, b->side), "tfx_batch: join");
    } else if (int r = launch_sdf_part(b, s)) {
        return r;
    }
    if (!b->overlap) {
        for (auto& c : b->classes)
            if (c.numItems > 0)
                if (int r = launch_strands(b, c, s)) return r;
        for (auto& c : b->classes)
            if (c.numItems > 0)
                if (int r = launch_follows(b, c, s)) return r;
        return launch_collide_levels(b, s);
    }
    TFX_CUDA(cudaEventRecord(b->evClasses, s), "tfx_batch: class fork");
    int k = 0;
    for (auto& c : b->classes) {
        if (c.numItems == 0) continue;
        cudaStream_t cs = k == 0 ? s : b->classStream[k];
        if (k > 0) TFX_CUDA(cudaStreamWaitEvent(cs, b->evClasses, 0), "tfx_batch: class fork");
        if (int r = launch_strands(b, c, cs)) return r;
        if (fork) TFX_CUDA(cudaStreamWaitEvent(cs, b->evJoin, 0), "tfx_batch: join");
        if (int r = launch_follows(b, c, cs)) return r;
        if (k > 0) TFX_CUDA(cudaEventRecord(b->evClassDone[k], cs), "tfx_batch: class join");
        ++k;
    }
    if (k == 0 && fork) TFX_CUDA(cudaStreamWaitEvent(s, b->evJoin, 0), "tfx_batch: join");
    for (int i = 1; i < k; ++i) TFX_CUDA(cudaStreamWaitEvent(s, b->evClassDone[i], 0), "tfx_batch: class join");
    return launch_collide_levels(b, s);
}

static int capture_graphs(tfx_batch b) {
    cudaStream_t s = b->ctx->stream;
    for (int slot = 0; slot < kFrameSlots; ++slot) {
        if (b->graph[slot]) { cudaGraphExecDestroy(b->graph[slot]); b->graph[slot] = nullptr; }
        cudaGraph_t g = nullptr;
        TFX_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
        cudaError_t e = cudaMemcpyAsync(b->devBlock, b->pinned[slot], b->blockBytes, cudaMemcpyHostToDevice, s);
        int r = TFX_OK;
        if (e != cudaSuccess) r = cuda_fail(e, "tfx_batch: capture upload");
        if (r == TFX_OK) r = launch_frame_forked(b, s);
        if (r == TFX_OK) {
            e = cudaMemcpyAsync(b->pinnedErr + slot, b->devErr, sizeof(int), cudaMemcpyDeviceToHost, s);
            if (e != cudaSuccess) r = cuda_fail(e, "tfx_batch: capture error-flag copy");
        }
        cudaError_t ee = cudaStreamEndCapture(s, &g);
        if (r != TFX_OK) { if (g) cudaGraphDestroy(g); return r; }
        if (ee != cudaSuccess) return cuda_fail(ee, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&b->graph[slot], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    }
    int sdfLaunches = 0;
    if (!b->sdfs.empty()) {
        if (b->sdfForm == 1) sdfLaunches = (b->sdfT.totalTris > 0 ? 5 : 1) + (b->sdfL.expand ? 1 : 0);
        else sdfLaunches = (b->sdfL.totalTris > 0 ? 3 : 2) + (b->sdfL.expand ? 1 : 0);
    }
    int launches = (b->totalMeshVerts > 0 ? 1 : 0) + sdfLaunches;
    for (auto& c : b->classes) launches += c.numItems > 0 ? (c.splitSweeps ? 4 : 2) : 0;
    for (size_t k = 0; k < b->levelPairs.size(); ++k) launches += b->levelVertices[k] > 0 ? 1 : 0;
    b->launchesPerFrame = launches;
    return TFX_OK;
}

// State snapshot for the autotuner: every buffer a frame writes.
struct Snapshot {
    void* mem = nullptr;
    std::vector<std::pair<void*, size_t>> regions;
};

static int snapshot_take(tfx_batch b, Snapshot& sn, cudaStream_t s) {
    size_t total = 0;
    sn.regions.clear();
    for (auto h : b->hairs)
        for (int k = TFX_BUF_POSITIONS; k <= TFX_BUF_STRAND_LEVEL_DATA; ++k) {
            sn.regions.push_back({h->bufs[k].ptr, h->bufs[k].bytes});
            total += align256(h->bufs[k].bytes);
        }
    for (size_t i = 0; i < b->sdfs.size(); ++i) {
        sn.regions.push_back({b->sdfs[i]->grid, 4 * (size_t)b->sdfs[i]->alloc});
        total += align256(4 * (size_t)b->sdfs[i]->alloc);
        if (b->sdfMesh[i]) {
            sn.regions.push_back({b->sdfMesh[i]->skinned, 32 * (size_t)b->sdfMesh[i]->nverts});
            total += align256(32 * (size_t)b->sdfMesh[i]->nverts);
        }
    }
    TFX_CUDA(cudaMalloc(&sn.mem, total ? total : 256), "tfx_batch: snapshot allocation");
    char* p = (char*)sn.mem;
    for (auto& r : sn.regions) {
        TFX_CUDA(cudaMemcpyAsync(p, r.first, r.second, cudaMemcpyDeviceToDevice, s), "tfx_batch: snapshot");
        p += align256(r.second);
    }
    return TFX_OK;
}

static int snapshot_restore(Snapshot& sn, cudaStream_t s) {
    char* p = (char*)sn.mem;
    for (auto& r : sn.regions) {
        TFX_CUDA(cudaMemcpyAsync(r.first, p, r.second, cudaMemcpyDeviceToDevice, s), "tfx_batch: restore");
        p += align256(r.second);
    }
    TFX_CUDA(cudaStreamSynchronize(s), "tfx_batch: restore sync");
    cudaFree(sn.mem);
    sn.mem = nullptr;
    return TFX_OK;
}

// Time per frame of the frame graph captured for the current shapes: the graph is uploaded and
// launched twice untimed, then the mean over max(frames, 6) launches is taken three times and the
// smallest kept (a freshly instantiated graph's first launches carry one-off costs).
static int time_graph_frames(tfx_batch b, int frames, float* ms) {
    if (int r = capture_graphs(b)) return r;
    cudaStream_t s = b->ctx->stream;
    const int n = std::max(frames, 6);
    cudaEvent_t e0, e1;
    TFX_CUDA(cudaEventCreate(&e0), "cudaEventCreate");
    TFX_CUDA(cudaEventCreate(&e1), "cudaEventCreate");
    cudaError_t e = cudaGraphUpload(b->graph[0], s);
    for (int w = 0; w < 2 && e == cudaSuccess; ++w) e = cudaGraphLaunch(b->graph[0], s);
    float best = 1e30f;
    for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
        e = cudaEventRecord(e0, s);
        for (int f = 0; f < n && e == cudaSuccess; ++f) e = cudaGraphLaunch(b->graph[0], s);
        if (e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float t = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
        if (e == cudaSuccess) best = std::min(best, t / (float)n);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cuda_fail(e, "tfx_batch: autotune frames");
    int flag = 0;
    TFX_CUDA(cudaMemcpy(&flag, b->devErr, sizeof(int), cudaMemcpyDeviceToHost), "tfx_batch: error flag");
    if (flag) return report_timeout(b);
    *ms = best;
    return TFX_OK;
}

// Coordinate descent over the launch shapes, each candidate timed as whole frames of the graph
// (the SDF branch overlaps the strand kernels, so a part cannot be timed alone): the SDF construct's
// block size, then per class the vertices per lane, warps per block, resident blocks per SM and the
// form of the follow/collide kernel.
static int autotune(tfx_batch b, int frames) {
    cudaStream_t s = b->ctx->stream;
    for (int i = 0; i < kFrameSlots; ++i) std::memcpy(b->pinned[i], b->staging.data(), b->blockBytes);
    Snapshot sn;
    if (int r = snapshot_take(b, sn, s)) return r;
    int rc = TFX_OK;
    float best = 1e30f;
    if ((rc = time_graph_frames(b, frames, &best))) { snapshot_restore(sn, s); return rc; }
    if (!b->sdfs.empty() && b->sdfL.totalTris > 0) {
        // the construct's form (tiles, or one warp per triangle at 64 / 128 / 256 threads per block)
        int bestForm = b->sdfForm, bestThreads = b->sdfL.constructThreads;
        for (int form = 0; form < 2 && rc == TFX_OK; ++form) {
            if (form == 1 && !b->tilesAvailable) continue;
            for (int th : {64, 128, 256}) {
                if (form == 1 && th != 128) continue;   // the tiled form has no block-size choice
                if (form == bestForm && (form == 1 || th == bestThreads)) continue;
                b->sdfForm = form;
                b->sdfL.constructThreads = th;
                float ms;
                if ((rc = time_graph_frames(b, frames, &ms))) break;
                if (ms < best) { best = ms; bestForm = form; bestThreads = th; }
            }
        }
        b->sdfForm = bestForm;
        b->sdfL.constructThreads = bestThreads;
    }
    for (size_t ci = 0; ci < b->classes.size() && rc == TFX_OK; ++ci) {
        BatchClass& c = b->classes[ci];
        if (c.numItems == 0) continue;
        int bestV = c.vpl, bestW = c.warps, bestCap = c.perSMCap;
        bool bestSplit = c.splitSweeps;
        for (int split = 0; split < 2 && rc == TFX_OK; ++split) {   // sweeps inside, or their own launch
            for (int vpl : {1, 2, 4}) {
                if (!fused_config_valid(c.n, vpl)) continue;
                for (int warps : {4, 8}) {
                    const int perSM = fused_blocks_per_sm(c.n, vpl, warps);
                    if (perSM <= 0) continue;
                    for (int cap = perSM; cap >= std::max(1, perSM - 1); --cap) {
                        if ((split != 0) == bestSplit && vpl == bestV && warps == bestW &&
                            (cap == perSM ? 0 : cap) == bestCap)
                            continue;
                        c.splitSweeps = split != 0;
                        c.vpl = vpl; c.warps = warps; c.perSMCap = cap == perSM ? 0 : cap;
                        if ((rc = size_class(b, c))) break;
                        float ms;
                        if ((rc = time_graph_frames(b, frames, &ms))) break;
                        if (ms < best) {
                            best = ms; bestV = vpl; bestW = warps; bestCap = c.perSMCap; bestSplit = split != 0;
                        }
                    }
                    if (rc) break;
                }
                if (rc) break;
            }
        }
        // Fewer resident strand blocks leave room on each SM for the concurrent SDF construct's
        // blocks: two lower caps for the best shape.
        const int perSM = fused_blocks_per_sm(c.n, bestV, bestW);
        const int from = (bestCap > 0 ? bestCap : perSM - 1) - 1;   // the loop above tried perSM and perSM - 1
        for (int cap = from; rc == TFX_OK && cap >= std::max(1, from - 1); --cap) {
            c.splitSweeps = bestSplit; c.vpl = bestV; c.warps = bestW; c.perSMCap = cap;
            if ((rc = size_class(b, c))) break;
            float ms;
            if ((rc = time_graph_frames(b, frames, &ms))) break;
            if (ms < best) { best = ms; bestCap = cap; }
        }
        c.vpl = bestV; c.warps = bestW; c.perSMCap = bestCap; c.splitSweeps = bestSplit;
        // the follow/collide form: one vertex at a time, both lookup stages queued, or the gradient stage
        int bestMode = c.followMode;
        for (int mode = 0; rc == TFX_OK && mode < 3; ++mode) {
            if (mode == bestMode) continue;
            c.followMode = mode;
            if ((rc = size_class(b, c))) break;
            float ms;
            if ((rc = time_graph_frames(b, frames, &ms))) break;
            if (ms < 0.99f * best) { best = ms; bestMode = mode; }   // a measured default yields to a clear gain only
        }
        c.followMode = bestMode;
        if (rc == TFX_OK) rc = size_class(b, c);
    }
    int rr = snapshot_restore(sn, s);
    return rc ? rc : rr;
}

// Which SDFs keep a corner-expanded copy: none, all, or (mode 2) those whose objects make at least
// four lookups per grid cell each frame (every vertex with j >= 2 is looked up at least once), where
// one 32-byte record per lookup beats eight scattered words by more than the copy costs.
static int apply_expand_mode(tfx_batch b) {
    const int nsdf = (int)b->sdfs.size(), nobj = (int)b->hairs.size();
    std::vector<double> lookups(nsdf, 0.0);
    for (int o = 0; o < nobj; ++o)
        if (b->hairSdf[o] >= 0) {
            tfx_hair h = b->hairs[o];
            lookups[b->hairSdf[o]] += (double)h->G * (h->F + 1) * (h->n - 2);
        }
    std::vector<BatchSdf> sdfs(nsdf);
    std::vector<BatchObject> objs(nobj);
    if (nsdf) TFX_CUDA(cudaMemcpy(sdfs.data(), b->sdfTable, sizeof(BatchSdf) * nsdf, cudaMemcpyDeviceToHost), "tfx_batch: SDFs");
    TFX_CUDA(cudaMemcpy(objs.data(), b->objTable, sizeof(BatchObject) * nobj, cudaMemcpyDeviceToHost), "tfx_batch: objects");
    std::vector<int> expSdf;
    std::vector<long long> expFirst(1, 0);
    for (int i = 0; i < nsdf; ++i) {
        const double cells = (double)b->sdfDims[3 * i] * b->sdfDims[3 * i + 1] * b->sdfDims[3 * i + 2];
        const bool on = b->expandMode == 1 || (b->expandMode == 2 && lookups[i] >= 4.0 * cells);
        sdfs[i].expanded = on ? b->sdfExpanded[i] : nullptr;
        if (on) {
            expSdf.push_back(i);
            expFirst.push_back(expFirst.back() + sdfs[i].numCells);
        }
    }
    if (!b->expTable && nsdf > 0)
        TFX_CUDA(cudaMalloc(&b->expTable, align256(sizeof(long long) * (size_t)(nsdf + 1)) + sizeof(int) * (size_t)nsdf),
                 "tfx_batch: expansion table");
    long long* devFirst = reinterpret_cast<long long*>(b->expTable);
    int* devSdf = reinterpret_cast<int*>(reinterpret_cast<char*>(b->expTable) + align256(sizeof(long long) * (size_t)(nsdf + 1)));
    if (!expSdf.empty()) {
        TFX_CUDA(cudaMemcpy(devFirst, expFirst.data(), sizeof(long long) * expFirst.size(), cudaMemcpyHostToDevice),
                 "tfx_batch: expansion table");
        TFX_CUDA(cudaMemcpy(devSdf, expSdf.data(), sizeof(int) * expSdf.size(), cudaMemcpyHostToDevice),
                 "tfx_batch: expansion table");
    }
    for (int o = 0; o < nobj; ++o) {
        const int si = b->hairSdf[o];
        objs[o].sdf8 = si >= 0 ? sdfs[si].expanded : nullptr;
    }
    if (nsdf) TFX_CUDA(cudaMemcpy(b->sdfTable, sdfs.data(), sizeof(BatchSdf) * nsdf, cudaMemcpyHostToDevice), "tfx_batch: SDFs");
    TFX_CUDA(cudaMemcpy(b->objTable, objs.data(), sizeof(BatchObject) * nobj, cudaMemcpyHostToDevice), "tfx_batch: objects");
    b->sdfL.expand = expSdf.empty() ? 0 : 1;
    b->sdfL.expSdf = devSdf;
    b->sdfL.expFirst = devFirst;
    b->sdfL.nexp = (int)expSdf.size();
    b->sdfL.expCells = expFirst.back();
    return TFX_OK;
}

extern "C" int tfx_batch_build(tfx_batch b, int reserved) {
    if (!b) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_build: null batch");
    if (b->built) return batch_fail_built("tfx_batch_build");
    if (b->hairs.empty()) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_build: no hair objects");
    if (reserved != 0) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_build: reserved must be 0");
    TFX_CUDA(cudaSetDevice(b->ctx->device), "cudaSetDevice");

    // ---- frame block layout
    size_t off = 0;
    for (auto h : b->hairs) {
        b->objOff.push_back(off);
        b->objBones.push_back(h->maxBone + 1);
        off = align16(off + offsetof(DevSimConsts, bones) + 64 * (size_t)(h->maxBone + 1));
    }
    for (size_t i = 0; i < b->sdfs.size(); ++i) {
        b->sdfOff.push_back(off);
        off = align16(off + sizeof(SdfFrame));
    }
    for (size_t i = 0; i < b->sdfs.size(); ++i) {
        tfx_mesh m = b->sdfMesh[i];
        b->meshOff.push_back(off);
        b->meshBones.push_back(m ? m->maxBone + 1 : 0);
        if (m) off = align16(off + 64 * (size_t)(m->maxBone + 1));
    }
    b->blockBytes = std::max<size_t>(off, 16);
    b->staging.assign(b->blockBytes, 0);
    for (int i = 0; i < kFrameSlots; ++i) {
        TFX_CUDA(cudaMallocHost((void**)&b->pinned[i], b->blockBytes), "tfx_batch: pinned frame block");
        TFX_CUDA(cudaEventCreateWithFlags(&b->done[i], cudaEventDisableTiming), "cudaEventCreate");
    }
    TFX_CUDA(cudaMalloc((void**)&b->devBlock, b->blockBytes), "tfx_batch: device frame block");
    TFX_CUDA(cudaMemset(b->devBlock, 0, b->blockBytes), "tfx_batch: clear frame block");

    // ---- device tables
    const int nobj = (int)b->hairs.size(), nsdf = (int)b->sdfs.size();
    b->nmeshes = 0;
    b->totalMeshVerts = 0;
    for (auto m : b->sdfMesh)
        if (m) { ++b->nmeshes; b->totalMeshVerts += m->nverts; }
    const size_t sizes[3] = {sizeof(BatchObject) * nobj, sizeof(BatchMesh) * std::max(1, b->nmeshes),
                             sizeof(BatchSdf) * std::max(1, nsdf)};
    TFX_CUDA(cudaMalloc(&b->devArena, align256(sizes[0]) + align256(sizes[1]) + align256(sizes[2]) + 256), "tfx_batch: tables");
    char* p = (char*)b->devArena;
    b->objTable = (BatchObject*)p; p += align256(sizes[0]);
    b->meshTable = (BatchMesh*)p; p += align256(sizes[1]);
    b->sdfTable = (BatchSdf*)p; p += align256(sizes[2]);
    b->devErr = (int*)p;
    TFX_CUDA(cudaMemset(b->devErr, 0, sizeof(int)), "tfx_batch: clear error flag");
    TFX_CUDA(cudaMallocHost((void**)&b->pinnedErr, kFrameSlots * sizeof(int)), "tfx_batch: pinned error flag");
    TFX_CUDA(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking), "tfx_batch: side stream");
    for (int i = 0; i < 5; ++i) {
        TFX_CUDA(cudaStreamCreateWithFlags(&b->classStream[i], cudaStreamNonBlocking), "tfx_batch: class stream");
        TFX_CUDA(cudaEventCreateWithFlags(&b->evClassDone[i], cudaEventDisableTiming), "cudaEventCreate");
    }
    TFX_CUDA(cudaEventCreateWithFlags(&b->evClasses, cudaEventDisableTiming), "cudaEventCreate");
    TFX_CUDA(cudaEventCreateWithFlags(&b->evFork, cudaEventDisableTiming), "cudaEventCreate");
    TFX_CUDA(cudaEventCreateWithFlags(&b->evJoin, cudaEventDisableTiming), "cudaEventCreate");
    for (int i = 0; i < kFrameSlots; ++i) b->pinnedErr[i] = 0;

    // corner-expanded grids: 8 floats per cell, at the SDF's quad prefix
    std::vector<long long> sdfFirstQuad(nsdf, 0);
    long long quadsTotal = 0;
    for (int i = 0; i < nsdf; ++i) {
        sdfFirstQuad[i] = quadsTotal;
        quadsTotal += ((long long)b->sdfDims[3 * i] * b->sdfDims[3 * i + 1] * b->sdfDims[3 * i + 2] + 3) / 4;
    }
    if (nsdf > 0)
        TFX_CUDA(cudaMalloc(&b->expandedArena, (size_t)quadsTotal * 4 * 32), "tfx_batch: corner-expanded grids");
    b->sdfExpanded.assign(nsdf, nullptr);
    for (int i = 0; i < nsdf; ++i) b->sdfExpanded[i] = reinterpret_cast<float4*>(b->expandedArena) + 2 * 4 * sdfFirstQuad[i];

    std::vector<BatchObject> objs(nobj);
    for (int o = 0; o < nobj; ++o) {
        tfx_hair h = b->hairs[o];
        objs[o].hair = h->view;
        objs[o].consts = reinterpret_cast<const DevSimConsts*>(b->devBlock + b->objOff[o]);
        const int si = b->hairSdf[o];
        objs[o].sdf = si >= 0 ? reinterpret_cast<const float*>(b->sdfs[si]->grid) : nullptr;
        objs[o].sdfFrame = si >= 0 ? reinterpret_cast<const SdfFrame*>(b->devBlock + b->sdfOff[si]) : nullptr;
        objs[o].sdf8 = nullptr;   // set by apply_expand_mode
    }
    TFX_CUDA(cudaMemcpy(b->objTable, objs.data(), sizeof(BatchObject) * nobj, cudaMemcpyHostToDevice), "tfx_batch: objects");

    // collision levels: level k = every object's k-th further SDF (distinct objects, one launch each)
    size_t levels = 0;
    for (auto& m : b->hairMoreSdf) levels = std::max(levels, m.size());
    for (size_t k = 0; k < levels; ++k) {
        std::vector<BatchCollide> pairs;
        long long first = 0;
        for (int o = 0; o < nobj; ++o) {
            if (b->hairMoreSdf[o].size() <= k) continue;
            const HairView& v = b->hairs[o]->view;
            pairs.push_back(BatchCollide{o, b->hairMoreSdf[o][k], first});
            first += (long long)v.G * (v.F + 1) * v.n;
        }
        BatchCollide* d = nullptr;
        TFX_CUDA(cudaMalloc(&d, sizeof(BatchCollide) * pairs.size()), "tfx_batch: collision levels");
        b->levelPairs.push_back(d);
        TFX_CUDA(cudaMemcpy(d, pairs.data(), sizeof(BatchCollide) * pairs.size(), cudaMemcpyHostToDevice),
                 "tfx_batch: collision levels");
        b->levelCount.push_back((int)pairs.size());
        b->levelVertices.push_back(first);
    }

    std::vector<BatchMesh> meshes;
    int firstVertex = 0;
    for (int i = 0; i < nsdf; ++i) {
        tfx_mesh m = b->sdfMesh[i];
        if (!m) continue;
        BatchMesh d{};
        d.bind = m->bind; d.skinned = m->skinned; d.skin = m->skin;
        d.bones = reinterpret_cast<const float4*>(b->devBlock + b->meshOff[i]);
        d.firstVertex = firstVertex; d.numVertices = m->nverts;
        firstVertex += m->nverts;
        meshes.push_back(d);
    }
    if (!meshes.empty())
        TFX_CUDA(cudaMemcpy(b->meshTable, meshes.data(), sizeof(BatchMesh) * meshes.size(), cudaMemcpyHostToDevice),
                 "tfx_batch: meshes");

    std::vector<BatchSdf> sdfs(nsdf);
    long long firstQuad = 0, firstTile = 0;
    int firstTri = 0;
    bool tilesOk = true;
    for (int i = 0; i < nsdf; ++i) {
        tfx_sdf s = b->sdfs[i];
        tfx_mesh m = b->sdfMesh[i];
        BatchSdf& d = sdfs[i];
        d.mesh = m ? m->skinned : s->mesh;
        d.indices = m ? m->idx : s->idx;
        d.numTriangles = m ? m->ntri : s->ntri;
        d.words = s->grid;
        d.frame = reinterpret_cast<const SdfFrame*>(b->devBlock + b->sdfOff[i]);
        d.numCells = (long long)b->sdfDims[3 * i] * b->sdfDims[3 * i + 1] * b->sdfDims[3 * i + 2];
        d.firstQuad = firstQuad;
        d.expanded = nullptr;     // set by apply_expand_mode
        d.firstTriangle = firstTri;
        d.tilesX = (b->sdfDims[3 * i] + SDF_TILE_X - 1) / SDF_TILE_X;
        d.tilesY = (b->sdfDims[3 * i + 1] + SDF_TILE_Y - 1) / SDF_TILE_Y;
        d.tilesZ = (b->sdfDims[3 * i + 2] + SDF_TILE_Z - 1) / SDF_TILE_Z;
        d.firstTile = (int)firstTile;
        firstQuad += (d.numCells + 3) / 4;
        firstTri += d.numTriangles;
        firstTile += (long long)d.tilesX * d.tilesY * d.tilesZ;
        tilesOk = tilesOk && b->sdfDims[3 * i] <= SDF_TILE_MAX_DIM && b->sdfDims[3 * i + 1] <= SDF_TILE_MAX_DIM &&
                  b->sdfDims[3 * i + 2] <= SDF_TILE_MAX_DIM;
    }
    tilesOk = tilesOk && firstTile < (1LL << 30);
    if (nsdf > 0 && tilesOk) {
        // tile arena: [tileCount | bigCount | workCounter] (zeroed per frame), tileStart, blockSum, list,
        // bigList, records
        const long long T = firstTile, nb = (T + 1023) / 1024, tris = std::max(firstTri, 1);
        const long long cap = (long long)SDF_BIG_TILES * tris;
        const size_t zeroBytes = sizeof(int) * (size_t)(T + nsdf + 1);
        const size_t parts[6] = {zeroBytes, sizeof(int) * (size_t)T, sizeof(int) * (size_t)nb, sizeof(int) * (size_t)cap,
                                 sizeof(int) * (size_t)tris, sizeof(float) * SDF_TRI_RECORD * (size_t)tris};
        size_t total = 0;
        for (size_t q : parts) total += align256(q);
        TFX_CUDA(cudaMalloc(&b->tileArena, total), "tfx_batch: SDF tile tables");
        TFX_CUDA(cudaMemset(b->tileArena, 0, total), "tfx_batch: clear SDF tile tables");
        char* q = (char*)b->tileArena;
        SdfTileLaunch& L = b->sdfT;
        L.sdfs = b->sdfTable;
        L.nsdf = nsdf;
        L.totalTris = firstTri;
        L.totalTiles = (int)T;
        L.tileCount = (int*)q;
        L.bigCount = L.tileCount + T;
        L.workCounter = L.bigCount + nsdf;
        L.zeroBytes = zeroBytes;
        q += align256(parts[0]);
        L.tileStart = (int*)q; q += align256(parts[1]);
        L.blockSum = (int*)q; q += align256(parts[2]);
        L.list = (int*)q; q += align256(parts[3]);
        L.listCapacity = cap;
        L.bigList = (int*)q; q += align256(parts[4]);
        L.records = (float*)q;
        L.blocks = sdf_tile_blocks_per_sm() * b->ctx->numSMs;
        b->tilesAvailable = true;
        b->sdfForm = 0;   // measured faster on every workload here; the autotuner tries the tiles
    } else {
        b->tilesAvailable = false;
        b->sdfForm = 0;
    }
    if (nsdf > 0)
        TFX_CUDA(cudaMemcpy(b->sdfTable, sdfs.data(), sizeof(BatchSdf) * nsdf, cudaMemcpyHostToDevice), "tfx_batch: SDFs");
    b->sdfL = SdfBatchLaunch{b->sdfTable, nsdf, firstTri, firstQuad, 128, 0, nullptr, nullptr, 0, 0};
    b->expandMode = 2;
    if (int r = apply_expand_mode(b)) return r;

    // ---- strand classes (one fused launch per vertices-per-strand count present)
    for (int n : {4, 8, 16, 32, 64}) {
        bool any = false;
        for (auto h : b->hairs) any |= (h->n == n);
        if (!any) continue;
        BatchClass c;
        c.n = n;
        make_items(b, c);   // vpl / warps: the BatchClass defaults (what the autotuner picks on the head and fur workloads)
        if (int r = upload_items(c)) return r;
        if (int r = size_class(b, c)) return r;
        b->classes.push_back(std::move(c));
    }
    if (int r = capture_graphs(b)) return r;
    b->built = true;
    describe(b);
    return TFX_OK;
}

extern "C" int tfx_batch_autotune(tfx_batch b, int frames) {
    if (!b || !b->built || frames <= 0) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_autotune: batch not built or no frames");
    for (size_t i = 0; i < b->hairSet.size(); ++i)
        if (!b->hairSet[i]) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_autotune: constants of object %zu never set", i);
    for (size_t i = 0; i < b->sdfSet.size(); ++i)
        if (!b->sdfSet[i]) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_autotune: grid of SDF %zu never set", i);
    TFX_CUDA(cudaSetDevice(b->ctx->device), "cudaSetDevice");
    TFX_CUDA(cudaStreamSynchronize(b->ctx->stream), "cudaStreamSynchronize");
    if (int r = autotune(b, frames)) return r;
    if (int r = capture_graphs(b)) return r;
    describe(b);
    return TFX_OK;
}

// ---------------------------------------------------------------------------------------------
extern "C" int tfx_batch_set_hair_constants(tfx_batch b, int index, const tfx_sim_params* p, int num_bones,
                                            int cpu_local_iterations) {
    if (!b || !p || index < 0 || index >= (int)b->hairs.size())
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_hair_constants: bad argument");
    if (!b->built) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_hair_constants: build the batch first");
    tfx_hair h = b->hairs[index];
    if (p->counts[0] != TFX_THREAD_GROUP_SIZE / h->n || p->counts[1] != h->F || p->counts[2] != h->n)
        return fail(TFX_ERR_MISMATCH, "tfx_batch_set_hair_constants: counts (%d,%d,%d) but object has (%d,%d,%d)", p->counts[0],
                    p->counts[1], p->counts[2], TFX_THREAD_GROUP_SIZE / h->n, h->F, h->n);
    if (num_bones < 0 || num_bones > TFX_MAX_BONES || cpu_local_iterations < 0 || cpu_local_iterations > 1024)
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_hair_constants: %d bones, %d local iterations", num_bones,
                    cpu_local_iterations);
    DevSimConsts* c = reinterpret_cast<DevSimConsts*>(b->staging.data() + b->objOff[index]);
    fill_consts_header(c, p, cpu_local_iterations);
    const int nb = std::min(num_bones, b->objBones[index]);
    std::memcpy(reinterpret_cast<char*>(c) + offsetof(DevSimConsts, bones), p->bone_matrices, 64 * (size_t)nb);
    b->hairSet[index] = true;
    return TFX_OK;
}

extern "C" int tfx_batch_set_sdf_frame(tfx_batch b, int index, const tfx_sdf_grid* g, float margin_world) {
    if (!b || !g || index < 0 || index >= (int)b->sdfs.size())
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_sdf_frame: bad argument");
    if (!b->built) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_sdf_frame: build the batch first");
    if (g->num_cells_x != b->sdfDims[3 * index] || g->num_cells_y != b->sdfDims[3 * index + 1] ||
        g->num_cells_z != b->sdfDims[3 * index + 2] || !(g->cell_size > 0.0f))
        return fail(TFX_ERR_MISMATCH, "tfx_batch_set_sdf_frame: grid %dx%dx%d (cell %g) differs from the batch's %dx%dx%d",
                    g->num_cells_x, g->num_cells_y, g->num_cells_z, (double)g->cell_size, b->sdfDims[3 * index],
                    b->sdfDims[3 * index + 1], b->sdfDims[3 * index + 2]);
    SdfFrame* f = reinterpret_cast<SdfFrame*>(b->staging.data() + b->sdfOff[index]);
    f->grid = SdfGrid{g->origin[0], g->origin[1], g->origin[2], g->cell_size, g->num_cells_x, g->num_cells_y,
                      g->num_cells_z, 0};
    f->margin = margin_world;
    b->sdfSet[index] = true;
    return TFX_OK;
}

extern "C" int tfx_batch_set_mesh_bones(tfx_batch b, int index, const float* bones, int num_bones) {
    if (!b || index < 0 || index >= (int)b->sdfs.size() || num_bones < 0 || (num_bones > 0 && !bones))
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_mesh_bones: bad argument");
    if (!b->built) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_mesh_bones: build the batch first");
    if (!b->sdfMesh[index]) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_mesh_bones: SDF %d has no skinned mesh", index);
    const int nb = std::min(num_bones, b->meshBones[index]);
    std::memcpy(b->staging.data() + b->meshOff[index], bones, 64 * (size_t)nb);
    return TFX_OK;
}

static int check_runnable(tfx_batch b, const char* who) {
    if (!b || !b->built) return fail(TFX_ERR_INVALID_ARGUMENT, "%s: batch not built", who);
    for (size_t i = 0; i < b->hairSet.size(); ++i)
        if (!b->hairSet[i]) return fail(TFX_ERR_INVALID_ARGUMENT, "%s: constants of object %zu never set", who, i);
    for (size_t i = 0; i < b->sdfSet.size(); ++i)
        if (!b->sdfSet[i]) return fail(TFX_ERR_INVALID_ARGUMENT, "%s: grid of SDF %zu never set", who, i);
    return TFX_OK;
}

// Claims the next pinned block: waits until its previous upload has executed, then fills it.
static int claim_block(tfx_batch b, int* slotOut) {
    const int s = b->slot;
    b->slot = (s + 1) % kFrameSlots;
    if (b->used[s]) {
        TFX_CUDA(cudaEventSynchronize(b->done[s]), "cudaEventSynchronize");
        if (b->pinnedErr[s]) {
            b->slot = s;   // the block stays unclaimed: the next call takes it
            return report_timeout(b);
        }
    }
    std::memcpy(b->pinned[s], b->staging.data(), b->blockBytes);
    *slotOut = s;
    return TFX_OK;
}

extern "C" int tfx_batch_run(tfx_batch b) {
    if (int r = check_runnable(b, "tfx_batch_run")) return r;
    TFX_CUDA(cudaSetDevice(b->ctx->device), "cudaSetDevice");
    int s = 0;
    if (int r = claim_block(b, &s)) return r;
    TFX_CUDA(cudaGraphLaunch(b->graph[s], b->ctx->stream), "cudaGraphLaunch");
    TFX_CUDA(cudaEventRecord(b->done[s], b->ctx->stream), "cudaEventRecord");
    b->used[s] = true;
    return TFX_OK;
}

extern "C" int tfx_batch_synchronize(tfx_batch b) {
    if (!b || !b->built) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_synchronize: batch not built");
    TFX_CUDA(cudaSetDevice(b->ctx->device), "cudaSetDevice");
    TFX_CUDA(cudaStreamSynchronize(b->ctx->stream), "cudaStreamSynchronize");
    for (int s = 0; s < kFrameSlots; ++s)
        if (b->used[s] && b->pinnedErr[s]) return report_timeout(b);
    return TFX_OK;
}

static int readback_init(tfx_batch b) {
    if (b->copy) return TFX_OK;
    b->snapFirst.assign(b->hairs.size(), 0);
    long long v = 0;
    for (size_t i = 0; i < b->hairs.size(); ++i) {
        b->snapFirst[i] = v;
        v += b->hairs[i]->Vtot;
    }
    b->snapVerts = v;
    for (int i = 0; i < 2; ++i) {
        TFX_CUDA(cudaMalloc(&b->snap[i], std::max<size_t>((size_t)v * sizeof(float4), 256)), "tfx_batch_readback: snapshot buffer");
        TFX_CUDA(cudaEventCreateWithFlags(&b->snapDone[i], cudaEventDisableTiming), "cudaEventCreate");
        TFX_CUDA(cudaEventCreateWithFlags(&b->copyDone[i], cudaEventDisableTiming), "cudaEventCreate");
    }
    TFX_CUDA(cudaMalloc(&b->devFirst, sizeof(long long) * std::max<size_t>(b->hairs.size(), 1)), "tfx_batch_readback: table");
    TFX_CUDA(cudaMemcpy(b->devFirst, b->snapFirst.data(), sizeof(long long) * b->hairs.size(), cudaMemcpyHostToDevice),
             "tfx_batch_readback: table");
    TFX_CUDA(cudaStreamCreateWithFlags(&b->copy, cudaStreamNonBlocking), "tfx_batch_readback: copy stream");
    return TFX_OK;
}

extern "C" int tfx_batch_readback(tfx_batch b, void* const* host_dst, int count, int format, int64_t* ticket) {
    if (!b || !host_dst || !ticket) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_readback: null argument");
    if (!b->built) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_readback: batch not built");
    if (format != TFX_READBACK_XYZW && format != TFX_READBACK_XYZ)
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_readback: format %d", format);
    if (count != (int)b->hairs.size())
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_readback: %d destinations for %d hair objects", count,
                    (int)b->hairs.size());
    for (int i = 0; i < count; ++i)
        if (!host_dst[i]) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_readback: destination %d is null", i);
    TFX_CUDA(cudaSetDevice(b->ctx->device), "cudaSetDevice");
    if (int r = readback_init(b)) return r;
    const int64_t t = b->nextTicket;
    const int s = (int)(t & 1);
    const size_t per = format == TFX_READBACK_XYZ ? 3 * sizeof(float) : sizeof(float4);
    cudaStream_t main = b->ctx->stream;
    // the snapshot may not overwrite a buffer whose copy to the host is still running
    if (b->copyUsed[s]) TFX_CUDA(cudaStreamWaitEvent(main, b->copyDone[s], 0), "cudaStreamWaitEvent");
    cudaError_t e = launch_snapshot_positions(b->objTable, b->devFirst, count, b->snapVerts,
                                              reinterpret_cast<float*>(b->snap[s]), format == TFX_READBACK_XYZ, main);
    if (e != cudaSuccess) return cuda_fail(e, "tfx_batch_readback: snapshot");
    TFX_CUDA(cudaEventRecord(b->snapDone[s], main), "cudaEventRecord");
    TFX_CUDA(cudaStreamWaitEvent(b->copy, b->snapDone[s], 0), "cudaStreamWaitEvent");
    for (int i = 0; i < count; ++i) {
        tfx_hair h = b->hairs[i];
        TFX_CUDA(cudaMemcpyAsync(host_dst[i], b->snap[s] + (size_t)b->snapFirst[i] * per, (size_t)h->Vtot * per,
                                 cudaMemcpyDeviceToHost, b->copy), "tfx_batch_readback: copy to host");
    }
    TFX_CUDA(cudaEventRecord(b->copyDone[s], b->copy), "cudaEventRecord");
    b->copyUsed[s] = true;
    b->nextTicket = t + 1;
    *ticket = t;
    return TFX_OK;
}

extern "C" int tfx_batch_wait_readback(tfx_batch b, int64_t ticket) {
    if (!b || ticket < 0 || ticket >= b->nextTicket)
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_wait_readback: no readback %lld", (long long)ticket);
    TFX_CUDA(cudaSetDevice(b->ctx->device), "cudaSetDevice");
    // the copy stream runs in order: the slot's latest copy finishing implies this one finished
    TFX_CUDA(cudaEventSynchronize(b->copyDone[ticket & 1]), "tfx_batch_wait_readback");
    return TFX_OK;
}

extern "C" int tfx_batch_profile_frame(tfx_batch b, float* part_ms, int max_parts, int* num_parts) {
    if (!num_parts) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_profile_frame: null output");
    if (int r = check_runnable(b, "tfx_batch_profile_frame")) return r;
    TFX_CUDA(cudaSetDevice(b->ctx->device), "cudaSetDevice");
    cudaStream_t st = b->ctx->stream;
    int s = 0;
    if (int r = claim_block(b, &s)) return r;
    TFX_CUDA(cudaMemcpyAsync(b->devBlock, b->pinned[s], b->blockBytes, cudaMemcpyHostToDevice, st), "tfx_batch: upload");
    std::vector<float> part;
    if (int r = launch_frame_direct(b, st, &part)) return r;
    TFX_CUDA(cudaEventRecord(b->done[s], st), "cudaEventRecord");
    b->used[s] = true;
    const int k = std::min((int)part.size(), std::max(max_parts, 0));
    for (int i = 0; i < k; ++i)
        if (part_ms) part_ms[i] = part[i];
    *num_parts = (int)part.size();
    return TFX_OK;
}

extern "C" int tfx_batch_set_option(tfx_batch b, int option, int value) {
    if (!b || !b->built) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_option: batch not built");
    switch (option) {
        case TFX_BATCH_EXPANDED_GRIDS:
            if (value < 0 || value > 2) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_option: expanded grids %d", value);
            TFX_CUDA(cudaStreamSynchronize(b->ctx->stream), "cudaStreamSynchronize");
            b->expandMode = value;
            if (int r = apply_expand_mode(b)) return r;
            break;
        case TFX_BATCH_OVERLAP_SDF:
            if (value != 0 && value != 1) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_option: overlap %d", value);
            b->overlap = value != 0;
            break;
        case TFX_BATCH_SDF_BLOCK:
            if (value != 64 && value != 128 && value != 256)
                return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_option: SDF block %d (64, 128 or 256)", value);
            b->sdfL.constructThreads = value;
            break;
        case TFX_BATCH_SPLIT_SWEEPS:
            if (value != 0 && value != 1) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_option: split %d", value);
            for (auto& c : b->classes) c.splitSweeps = value != 0;
            break;
        case TFX_BATCH_FOLLOW_FORM:
            if (value < 0 || value > 2) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_option: follow form %d", value);
            for (auto& c : b->classes) {
                c.followMode = value;
                if (int r = size_class(b, c)) return r;
            }
            break;
        case TFX_BATCH_WAIT_POLLS:
            if (value < 0) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_option: wait polls %d", value);
            b->waitPolls = value;
            break;
        case TFX_BATCH_SDF_FORM:
            if (value != 0 && value != 1) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_option: SDF form %d", value);
            if (value == 1 && !b->tilesAvailable)
                return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_option: tiled SDF build needs grids of at most %d cells "
                            "per axis", SDF_TILE_MAX_DIM);
            b->sdfForm = value;
            break;
        default: return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_set_option: unknown option %d", option);
    }
    TFX_CUDA(cudaSetDevice(b->ctx->device), "cudaSetDevice");
    TFX_CUDA(cudaStreamSynchronize(b->ctx->stream), "cudaStreamSynchronize");
    if (int r = capture_graphs(b)) return r;
    describe(b);
    return TFX_OK;
}

extern "C" int tfx_batch_get_option(tfx_batch b, int option, int* value) {
    if (!b || !value) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_get_option: null argument");
    switch (option) {
        case TFX_BATCH_EXPANDED_GRIDS: *value = b->expandMode; break;
        case TFX_BATCH_OVERLAP_SDF: *value = b->overlap ? 1 : 0; break;
        case TFX_BATCH_SDF_BLOCK: *value = b->sdfL.constructThreads; break;
        case TFX_BATCH_SPLIT_SWEEPS: *value = (!b->classes.empty() && b->classes[0].splitSweeps) ? 1 : 0; break;
        case TFX_BATCH_FOLLOW_FORM: *value = b->classes.empty() ? 0 : b->classes[0].followMode; break;
        case TFX_BATCH_WAIT_POLLS: *value = b->waitPolls; break;
        case TFX_BATCH_SDF_FORM: *value = b->sdfForm; break;
        default: return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_get_option: unknown option %d", option);
    }
    return TFX_OK;
}

extern "C" int tfx_batch_describe(tfx_batch b, char* buf, size_t len, int32_t* launches_per_frame) {
    if (!b) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_batch_describe: null batch");
    if (buf && len) {
        std::strncpy(buf, b->description.c_str(), len - 1);
        buf[len - 1] = 0;
    }
    if (launches_per_frame) *launches_per_frame = b->launchesPerFrame;
    return TFX_OK;
}
