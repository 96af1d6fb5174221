// C ABI of the learned collision proxy (tfx_nsdf_*): training data from the method's own grid SDFs,
// training, evaluation against the grids, queries, and collision with the exact-grid fallback.
#include <algorithm>
#include <climits>
#include <cstring>
#include <new>
#include <vector>

#include "tfx_handles.h"
#include "tfx_neural.cuh"

using namespace tfx;

struct tfx_nsdf_t {
    tfx_context ctx = nullptr;
    nsdf::Frame fr{};
    float band = 3.0f;
    float sphereC[3] = {0.f, 0.f, 0.f};
    float sphereR = 0.f;
    float slack = 1.0f;
    uint32_t seed = 1;
    void* arena = nullptr;          // params, grads, Adam m / v, bf16 weights, biases, loss
    float* params = nullptr;
    float* grads = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    __nv_bfloat16* wbf = nullptr;
    float* bias = nullptr;
    float* lossSum = nullptr;
    uint8_t* wtc = nullptr;         // packed weights of the tcgen05 forward pass
    int* err = nullptr;             // a bounded wait of the tcgen05 forward pass gave up
    int inference = 1;              // tfx_nsdf_set_inference: 1 tcgen05, 0 mma.sync
    nsdf::Sample* pool[2] = {nullptr, nullptr};
    int64_t poolCap[2] = {0, 0};
    int64_t poolSize[2] = {0, 0};
    __nv_bfloat16* acts = nullptr;
    int actsBatch = 0;
    int step = 0;
    uint32_t* marks = nullptr;
    int64_t marksCap = 0;           // words
    int* band_ = nullptr;           // [0] = count, then the list
    float poseLo[3] = {1e30f, 1e30f, 1e30f};   // range of the training poses (pool 0)
    float poseHi[3] = {-1e30f, -1e30f, -1e30f};
    int64_t bandCap = 0;
};

static int nsdf_grow(void** p, int64_t* cap, int64_t need, size_t elem, const char* what) {
    if (need <= *cap) return TFX_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    TFX_CUDA(cudaMalloc(p, (size_t)need * elem), what);
    *cap = need;
    return TFX_OK;
}

extern "C" int tfx_nsdf_create(tfx_context ctx, const tfx_nsdf_desc* d, tfx_nsdf* out) {
    if (!out) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_create: out is null");
    *out = nullptr;
    if (!ctx || !d) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_create: null argument");
    if (!(d->cell_size > 0.f) || !(d->band_cells > 0.f) || d->max_samples <= 0 || d->max_eval_samples < 0)
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_create: cell %g band %g samples %lld", (double)d->cell_size,
                    (double)d->band_cells, (long long)d->max_samples);
    for (int k = 0; k < 3; ++k)
        if (!(d->box_max[k] > d->box_min[k])) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_create: empty box");
    TFX_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    auto* h = new (std::nothrow) tfx_nsdf_t();
    if (!h) return fail(TFX_ERR_OUT_OF_MEMORY, "tfx_nsdf_create: host allocation");
    h->ctx = ctx;
    h->fr.cx = 0.5f * (d->box_min[0] + d->box_max[0]);
    h->fr.cy = 0.5f * (d->box_min[1] + d->box_max[1]);
    h->fr.cz = 0.5f * (d->box_min[2] + d->box_max[2]);
    h->fr.ihx = 2.0f / (d->box_max[0] - d->box_min[0]);
    h->fr.ihy = 2.0f / (d->box_max[1] - d->box_min[1]);
    h->fr.ihz = 2.0f / (d->box_max[2] - d->box_min[2]);
    h->fr.poseScale = d->pose_scale;
    h->fr.cell = d->cell_size;
    h->band = d->band_cells;
    std::memcpy(h->sphereC, d->sphere_center, sizeof(h->sphereC));
    h->sphereR = d->sphere_radius;
    h->slack = d->contact_slack_cells > 0.f ? d->contact_slack_cells : 1.0f;
    h->seed = d->seed ? d->seed : 1;
    const size_t pbytes = align256(sizeof(float) * nsdf::NPARAM);
    const size_t total = 4 * pbytes + align256(sizeof(__nv_bfloat16) * nsdf::WBF_ALL) + align256(sizeof(float) * nsdf::NBIAS) +
                         256 + align256(nsdf::TC_WBYTES) + 256;
    cudaError_t e = cudaMalloc(&h->arena, total);
    if (e != cudaSuccess) { delete h; return cuda_fail(e, "tfx_nsdf_create: cudaMalloc"); }
    char* p = (char*)h->arena;
    h->params = (float*)p; p += pbytes;
    h->grads = (float*)p; p += pbytes;
    h->m = (float*)p; p += pbytes;
    h->v = (float*)p; p += pbytes;
    h->wbf = (__nv_bfloat16*)p; p += align256(sizeof(__nv_bfloat16) * nsdf::WBF_ALL);
    h->bias = (float*)p; p += align256(sizeof(float) * nsdf::NBIAS);
    h->lossSum = (float*)p; p += 256;
    h->wtc = (uint8_t*)p; p += align256(nsdf::TC_WBYTES);
    h->err = (int*)p;
    int r = TFX_OK;
    if ((e = cudaMemsetAsync(h->arena, 0, total, ctx->stream)) != cudaSuccess) r = cuda_fail(e, "tfx_nsdf_create: clear");
    if (!r && (e = nsdf::launch_init_params(h->params, h->seed, h->wbf, h->bias, ctx->stream)) != cudaSuccess)
        r = cuda_fail(e, "tfx_nsdf_create: init");
    if (!r && (e = nsdf::launch_pack_tc(h->params, h->wtc, ctx->stream)) != cudaSuccess)
        r = cuda_fail(e, "tfx_nsdf_create: pack");
    if (!r) r = nsdf_grow((void**)&h->pool[0], &h->poolCap[0], d->max_samples, sizeof(nsdf::Sample), "tfx_nsdf_create: pool");
    if (!r && d->max_eval_samples > 0)
        r = nsdf_grow((void**)&h->pool[1], &h->poolCap[1], d->max_eval_samples, sizeof(nsdf::Sample), "tfx_nsdf_create: pool");
    if (r) {
        cudaFree(h->arena);
        if (h->pool[0]) cudaFree(h->pool[0]);
        if (h->pool[1]) cudaFree(h->pool[1]);
        delete h;
        return r;
    }
    context_retain(ctx);
    *out = h;
    return TFX_OK;
}

extern "C" int tfx_nsdf_destroy(tfx_nsdf h) {
    if (!h) return TFX_OK;
    cudaSetDevice(h->ctx->device);
    cudaStreamSynchronize(h->ctx->stream);
    cudaFree(h->arena);
    for (int k = 0; k < 2; ++k)
        if (h->pool[k]) cudaFree(h->pool[k]);
    if (h->acts) cudaFree(h->acts);
    if (h->marks) cudaFree(h->marks);
    if (h->band_) cudaFree(h->band_);
    context_release(h->ctx);
    delete h;
    return TFX_OK;
}

static nsdf::Pose pose_of(const float* p) { return nsdf::Pose{p ? p[0] : 0.f, p ? p[1] : 0.f, p ? p[2] : 0.f}; }

// Reports (once) that a bounded wait of the tcgen05 forward pass gave up since the last check; the
// caller has synchronized the stream.
static int check_err(tfx_nsdf h) {
    int flag = 0;
    TFX_CUDA(cudaMemcpy(&flag, h->err, sizeof(int), cudaMemcpyDeviceToHost), "tfx_nsdf: error flag");
    if (!flag) return TFX_OK;
    TFX_CUDA(cudaMemset(h->err, 0, sizeof(int)), "tfx_nsdf: error flag");
    return fail(TFX_ERR_TIMEOUT, "tfx_nsdf: a tensor-core wait gave up");
}

extern "C" int tfx_nsdf_add_samples(tfx_nsdf h, int pool, tfx_mesh mesh, tfx_sdf sdf, const tfx_sdf_grid* grid,
                                    const float* bones, int num_bones, const float pose[3], const float sphere[4],
                                    int count, float sigma_cells) {
    if (!h || !mesh || !sdf || !grid || (pool != 0 && pool != 1) || count <= 0 || !(sigma_cells > 0.f))
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_add_samples: bad argument");
    if (mesh->ctx != h->ctx || sdf->ctx != h->ctx) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_add_samples: other context");
    if (h->poolSize[pool] + count > h->poolCap[pool])
        return fail(TFX_ERR_SIZE, "tfx_nsdf_add_samples: pool %d holds %lld of %lld samples, %d more do not fit", pool,
                    (long long)h->poolSize[pool], (long long)h->poolCap[pool], count);
    if (int r = tfx_mesh_skin(mesh, bones, num_bones)) return r;
    if (int r = tfx_sdf_set_mesh(sdf, mesh->skinned, mesh->nverts, mesh->idx, mesh->ntri)) return r;
    if (int r = tfx_sdf_update(sdf, grid)) return r;
    TFX_CUDA(cudaSetDevice(h->ctx->device), "cudaSetDevice");
    const SdfGrid g{grid->origin[0], grid->origin[1], grid->origin[2], grid->cell_size, grid->num_cells_x,
                    grid->num_cells_y, grid->num_cells_z, 0};
    const uint32_t seed = h->seed * 0x9E3779B9u + (uint32_t)(h->poolSize[0] + 3 * h->poolSize[1]) * 7919u + (uint32_t)pool;
    cudaError_t e = nsdf::launch_sample(mesh->skinned, mesh->nverts, reinterpret_cast<const float*>(sdf->grid), g, h->band,
                                        sigma_cells * grid->cell_size,
                                        sphere ? make_float3(sphere[0], sphere[1], sphere[2])
                                               : make_float3(h->sphereC[0], h->sphereC[1], h->sphereC[2]),
                                        sphere ? sphere[3] : h->sphereR, pose_of(pose), count, seed,
                                        h->pool[pool] + h->poolSize[pool],
                                        h->ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "tfx_nsdf_add_samples: sample launch");
    h->poolSize[pool] += count;
    if (pool == 0 && pose)
        for (int k = 0; k < 3; ++k) {
            h->poseLo[k] = std::min(h->poseLo[k], pose[k]);
            h->poseHi[k] = std::max(h->poseHi[k], pose[k]);
        }
    return TFX_OK;
}

extern "C" int tfx_nsdf_train(tfx_nsdf h, int steps, int batch, float lr, float* mean_loss) {
    if (!h || steps < 0 || batch <= 0 || batch % 512 != 0 || !(lr > 0.f))
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_train: steps %d batch %d (a multiple of 512) lr %g", steps, batch, (double)lr);
    if (h->poolSize[0] == 0) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_train: no training samples");
    TFX_CUDA(cudaSetDevice(h->ctx->device), "cudaSetDevice");
    cudaStream_t s = h->ctx->stream;
    if (h->actsBatch < batch) {
        if (h->acts) cudaFree(h->acts);
        h->acts = nullptr;
        h->actsBatch = 0;
        TFX_CUDA(cudaMalloc(&h->acts, sizeof(__nv_bfloat16) * nsdf::acts_elements(batch)), "tfx_nsdf_train: activations");
        h->actsBatch = batch;
    }
    TFX_CUDA(cudaMemsetAsync(h->lossSum, 0, sizeof(float), s), "tfx_nsdf_train: loss");
    const int tail = std::max(1, steps / 10);   // the mean loss is taken over the last tenth of the steps
    for (int k = 0; k < steps; ++k) {
        if (k == steps - tail) TFX_CUDA(cudaMemsetAsync(h->lossSum, 0, sizeof(float), s), "tfx_nsdf_train: loss");
        ++h->step;
        cudaError_t e = nsdf::launch_train_step(h->wbf, h->bias, h->fr, h->pool[0], h->poolSize[0], batch,
                                                h->seed * 2654435761u + (uint32_t)h->step * 40503u, h->acts, h->grads,
                                                h->lossSum, s);
        // cosine decay of the learning rate over this call's steps, to a tenth of it
        const float lrk = lr * (0.1f + 0.45f * (1.0f + cosf(3.14159265f * (float)k / (float)steps)));
        if (e == cudaSuccess) e = nsdf::launch_adam(h->params, h->grads, h->m, h->v, h->step, lrk, 1.0f, h->wbf, h->bias, s);
        if (e != cudaSuccess) return cuda_fail(e, "tfx_nsdf_train: step launch");
    }
    if (cudaError_t e = nsdf::launch_pack_tc(h->params, h->wtc, s)) return cuda_fail(e, "tfx_nsdf_train: pack");
    if (mean_loss) {
        float l = 0.f;
        TFX_CUDA(cudaMemcpyAsync(&l, h->lossSum, sizeof(float), cudaMemcpyDeviceToHost, s), "tfx_nsdf_train: loss");
        TFX_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        *mean_loss = steps > 0 ? l / ((float)batch * (float)std::min(tail, steps)) : 0.f;
    }
    return TFX_OK;
}

extern "C" int tfx_nsdf_evaluate(tfx_nsdf h, int pool, float* pred_cells, float* target_cells, float* weight,
                                 int64_t max_count, int64_t* count) {
    if (!h || (pool != 0 && pool != 1) || !count) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_evaluate: bad argument");
    const int64_t n = std::min<int64_t>(h->poolSize[pool], std::max<int64_t>(max_count, 0));
    *count = n;
    if (n == 0) return TFX_OK;
    TFX_CUDA(cudaSetDevice(h->ctx->device), "cudaSetDevice");
    cudaStream_t s = h->ctx->stream;
    float* dev = nullptr;
    TFX_CUDA(cudaMalloc(&dev, sizeof(float) * n), "tfx_nsdf_evaluate: output");
    cudaError_t e;
    if (h->inference) {
        nsdf::TcArgs t{};
        t.wtc = h->wtc; t.fr = h->fr; t.samples = h->pool[pool]; t.count = (int)n; t.out = dev; t.err = h->err;
        e = nsdf::launch_query_samples_tc(t, s);
    } else {
        e = nsdf::launch_query_samples(h->wbf, h->bias, h->fr, h->pool[pool], (int)n, dev, s);
    }
    std::vector<nsdf::Sample> host;
    if (e == cudaSuccess && pred_cells) e = cudaMemcpyAsync(pred_cells, dev, sizeof(float) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && (target_cells || weight)) {
        host.resize(n);
        e = cudaMemcpyAsync(host.data(), h->pool[pool], sizeof(nsdf::Sample) * n, cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(dev);
    if (e != cudaSuccess) return cuda_fail(e, "tfx_nsdf_evaluate");
    if (int r = check_err(h)) return r;
    for (int64_t k = 0; k < (int64_t)host.size(); ++k) {
        if (target_cells) target_cells[k] = host[k].target;
        if (weight) weight[k] = host[k].weight;
    }
    return TFX_OK;
}

extern "C" int tfx_nsdf_query(tfx_nsdf h, const void* points, int count, const float pose[3], float* out) {
    if (!h || count < 0 || (count > 0 && (!points || !out))) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_query: bad argument");
    if (((uintptr_t)points & 15) != 0) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_query: points not 16-byte aligned");
    TFX_CUDA(cudaSetDevice(h->ctx->device), "cudaSetDevice");
    cudaError_t e;
    if (h->inference) {
        nsdf::TcArgs t{};
        t.wtc = h->wtc; t.fr = h->fr; t.pose = pose_of(pose); t.pts = static_cast<const float4*>(points);
        t.count = count; t.out = out; t.err = h->err;
        e = nsdf::launch_query_tc(t, h->ctx->stream);
    } else {
        e = nsdf::launch_query(h->wbf, h->bias, h->fr, static_cast<const float4*>(points), count, pose_of(pose), out,
                               h->ctx->stream);
    }
    return e == cudaSuccess ? TFX_OK : cuda_fail(e, "tfx_nsdf_query launch");
}

extern "C" int tfx_nsdf_collide(tfx_nsdf h, tfx_hair hair, tfx_sdf sdf, const tfx_sdf_grid* grid, float margin_world,
                                const float pose[3], int32_t* band_count) {
    if (!h || !hair || !sdf || !grid) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_collide: null argument");
    if (hair->ctx != h->ctx || sdf->ctx != h->ctx) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_collide: other context");
    const int64_t cells = (int64_t)grid->num_cells_x * grid->num_cells_y * grid->num_cells_z;
    if (grid->num_cells_x <= 0 || grid->num_cells_y <= 0 || grid->num_cells_z <= 0 || cells > sdf->alloc)
        return fail(TFX_ERR_SIZE, "tfx_nsdf_collide: grid of %lld cells (allocation %lld)", (long long)cells, (long long)sdf->alloc);
    if (sdf->ntri > 0 && !sdf->mesh) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_collide: no collision mesh bound");
    TFX_CUDA(cudaSetDevice(h->ctx->device), "cudaSetDevice");
    // a pose outside the range the network was trained on: the grid path for every vertex
    bool inRange = pose != nullptr;
    for (int k = 0; k < 3 && inRange; ++k) inRange = pose[k] >= h->poseLo[k] && pose[k] <= h->poseHi[k];
    if (!inRange) {
        if (int r = tfx_sdf_update(sdf, grid)) return r;
        if (int r = tfx_sdf_collide(sdf, hair, grid, margin_world)) return r;
        if (band_count) {
            *band_count = (int32_t)std::min<int64_t>(hair->Vtot, INT32_MAX);
            TFX_CUDA(cudaStreamSynchronize(h->ctx->stream), "cudaStreamSynchronize");
        }
        return TFX_OK;
    }
    // per-cell marks, then one bit per 4x4x4-cell block
    const long long coarseBits = (long long)((grid->num_cells_x + 3) / 4) * ((grid->num_cells_y + 3) / 4) *
                                 ((grid->num_cells_z + 3) / 4);
    if (int r = nsdf_grow((void**)&h->marks, &h->marksCap, (cells + 31) / 32 + (coarseBits + 31) / 32, sizeof(uint32_t),
                          "tfx_nsdf_collide: marks"))
        return r;
    if (int r = nsdf_grow((void**)&h->band_, &h->bandCap, hair->Vtot + 1, sizeof(int), "tfx_nsdf_collide: band")) return r;
    nsdf::CollideArgs a{};
    a.wbf = h->wbf; a.bias = h->bias; a.fr = h->fr; a.pose = pose_of(pose);
    a.pos = hair->view.pos; a.prev = hair->view.prev; a.n = hair->n; a.vtot = hair->Vtot;
    a.grid = SdfGrid{grid->origin[0], grid->origin[1], grid->origin[2], grid->cell_size, grid->num_cells_x,
                     grid->num_cells_y, grid->num_cells_z, 0};
    a.margin = margin_world;
    a.slackCells = h->slack;
    a.words = sdf->grid;
    a.marks = h->marks;
    a.bandCount = h->band_;
    a.bandList = h->band_ + 1;
    a.mesh = sdf->mesh; a.indices = sdf->idx; a.ntri = sdf->ntri;
    a.wtc = h->inference ? h->wtc : nullptr;
    a.err = h->err;
    cudaError_t e = nsdf::launch_collide(a, h->ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "tfx_nsdf_collide launch");
    if (band_count) {
        TFX_CUDA(cudaMemcpyAsync(band_count, h->band_, sizeof(int32_t), cudaMemcpyDeviceToHost, h->ctx->stream), "tfx_nsdf_collide");
        TFX_CUDA(cudaStreamSynchronize(h->ctx->stream), "cudaStreamSynchronize");
        if (int r = check_err(h)) return r;
    }
    return TFX_OK;
}

extern "C" int tfx_nsdf_get_params(tfx_nsdf h, float* host, size_t count) {
    if (!h || !host || count != (size_t)nsdf::NPARAM)
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_get_params: need %d floats", nsdf::NPARAM);
    TFX_CUDA(cudaSetDevice(h->ctx->device), "cudaSetDevice");
    TFX_CUDA(cudaMemcpyAsync(host, h->params, sizeof(float) * count, cudaMemcpyDeviceToHost, h->ctx->stream), "tfx_nsdf_get_params");
    TFX_CUDA(cudaStreamSynchronize(h->ctx->stream), "cudaStreamSynchronize");
    return TFX_OK;
}

extern "C" int tfx_nsdf_set_params(tfx_nsdf h, const float* host, size_t count) {
    if (!h || !host || count != (size_t)nsdf::NPARAM)
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_set_params: need %d floats", nsdf::NPARAM);
    TFX_CUDA(cudaSetDevice(h->ctx->device), "cudaSetDevice");
    cudaStream_t s = h->ctx->stream;
    TFX_CUDA(cudaMemcpyAsync(h->params, host, sizeof(float) * count, cudaMemcpyHostToDevice, s), "tfx_nsdf_set_params");
    TFX_CUDA(cudaMemsetAsync(h->m, 0, sizeof(float) * count, s), "tfx_nsdf_set_params");
    TFX_CUDA(cudaMemsetAsync(h->v, 0, sizeof(float) * count, s), "tfx_nsdf_set_params");
    TFX_CUDA(cudaMemsetAsync(h->wbf, 0, sizeof(__nv_bfloat16) * nsdf::WBF_ALL, s), "tfx_nsdf_set_params");
    cudaError_t e = nsdf::launch_adam(h->params, nullptr, nullptr, nullptr, 0, 0.f, 0.f, h->wbf, h->bias, s);
    if (e == cudaSuccess) e = nsdf::launch_pack_tc(h->params, h->wtc, s);
    if (e != cudaSuccess) return cuda_fail(e, "tfx_nsdf_set_params");
    h->step = 0;
    TFX_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    return TFX_OK;
}

extern "C" int tfx_nsdf_get_info(tfx_nsdf h, int32_t* num_params, int64_t* train_samples, int64_t* eval_samples,
                                 int32_t* steps) {
    if (!h) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_get_info: null handle");
    if (num_params) *num_params = nsdf::NPARAM;
    if (train_samples) *train_samples = h->poolSize[0];
    if (eval_samples) *eval_samples = h->poolSize[1];
    if (steps) *steps = h->step;
    return TFX_OK;
}

extern "C" int tfx_nsdf_set_inference(tfx_nsdf h, int form) {
    if (!h || (form != 0 && form != 1)) return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_set_inference: form %d", form);
    h->inference = form;
    return TFX_OK;
}

extern "C" int tfx_nsdf_set_samples(tfx_nsdf h, int pool, const float* samples, int64_t count) {
    if (!h || (pool != 0 && pool != 1) || count < 0 || (count > 0 && !samples))
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_set_samples: bad argument");
    if (count > h->poolCap[pool])
        return fail(TFX_ERR_SIZE, "tfx_nsdf_set_samples: %lld samples, pool %d holds %lld", (long long)count, pool,
                    (long long)h->poolCap[pool]);
    TFX_CUDA(cudaSetDevice(h->ctx->device), "cudaSetDevice");
    if (count > 0)
        TFX_CUDA(cudaMemcpyAsync(h->pool[pool], samples, sizeof(nsdf::Sample) * (size_t)count, cudaMemcpyHostToDevice,
                                 h->ctx->stream), "tfx_nsdf_set_samples");
    TFX_CUDA(cudaStreamSynchronize(h->ctx->stream), "cudaStreamSynchronize");
    h->poolSize[pool] = count;
    if (pool == 0) {   // the pose range the collision trusts the network on
        for (int k = 0; k < 3; ++k) { h->poseLo[k] = 1e30f; h->poseHi[k] = -1e30f; }
        for (int64_t i = 0; i < count; ++i)
            for (int k = 0; k < 3; ++k) {
                const float a = samples[8 * i + 4 + k];
                h->poseLo[k] = std::min(h->poseLo[k], a);
                h->poseHi[k] = std::max(h->poseHi[k], a);
            }
    }
    return TFX_OK;
}

extern "C" int tfx_nsdf_get_gradients(tfx_nsdf h, float* host, size_t count) {
    if (!h || !host || count != (size_t)nsdf::NPARAM)
        return fail(TFX_ERR_INVALID_ARGUMENT, "tfx_nsdf_get_gradients: need %d floats", nsdf::NPARAM);
    TFX_CUDA(cudaSetDevice(h->ctx->device), "cudaSetDevice");
    TFX_CUDA(cudaMemcpyAsync(host, h->grads, sizeof(float) * count, cudaMemcpyDeviceToHost, h->ctx->stream),
             "tfx_nsdf_get_gradients");
    TFX_CUDA(cudaStreamSynchronize(h->ctx->stream), "cudaStreamSynchronize");
    return TFX_OK;
}
