// Dispatch emulator for the reference's compute shaders compiled as C++ (test infrastructure).
//
// The translation units produced by translate.py (the reference's own shader source) are included
// below, one namespace per shader file.  A Dispatch(numGroups) runs every 64-thread group in turn:
// each thread of the group is a fiber (ucontext); GroupMemoryBarrierWithGroupSync() switches back
// to the scheduler, and a group advances to its next barrier phase only after all 64 threads have
// reached the barrier (or returned).  Within a phase the threads run in SV_GroupIndex order, so a
// thread reads shared memory before any higher-numbered thread of the same phase writes it, which
// is the lockstep wave64 behaviour the wind step relies on.  Resource accesses follow D3D
// out-of-bounds rules (reads return zero, writes are dropped), and the host-side dispatch sizes are
// the reference's own (TressFXSimulation.cpp:51-75, TressFXSDFCollision.cpp:122-208,
// TressFXBoneSkinning.cpp:490-497).
#include <ucontext.h>

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <vector>

#include "hlsl_shim.h"

#define AMD_TRESSFX_MAX_NUM_BONES 512
#define AMD_TRESSFX_MAX_HAIR_GROUP_RENDER 16
#define TRESSFX_MAX_NUM_COLLISION_CAPSULES 8

#include "ref_sim.inc"
#include "ref_sdf.inc"
#include "ref_skin.inc"
#include "ref_strands.inc"
#include "ref_mc.inc"
// the reference's own marching-cubes tables, from its source tree (include path set by the recipe)
#include "MarchingCubesTables.h"

// ------------------------------------------------------------------------------------ fibers
namespace {
constexpr int kGroup = 64;
constexpr size_t kStack = 256 * 1024;

typedef void (*KernelFn)(uint, uint3, uint3);

struct Fiber {
    ucontext_t ctx;
    bool done;
};

ucontext_t g_sched;
Fiber g_fiber[kGroup];
std::vector<char> g_stacks;
int g_cur = 0;
KernelFn g_kernel = nullptr;
uint g_groupId = 0;

void fiber_main() {
    const int t = g_cur;
    g_kernel((uint)t, uint3(g_groupId, 0, 0), uint3(g_groupId * kGroup + (uint)t, 0, 0));
    g_fiber[t].done = true;
    swapcontext(&g_fiber[t].ctx, &g_sched);
}

void run_group_with_barriers(KernelFn k, uint group) {
    if (g_stacks.empty()) g_stacks.resize(kStack * kGroup);
    g_kernel = k;
    g_groupId = group;
    for (int t = 0; t < kGroup; ++t) {
        getcontext(&g_fiber[t].ctx);
        g_fiber[t].ctx.uc_stack.ss_sp = g_stacks.data() + kStack * t;
        g_fiber[t].ctx.uc_stack.ss_size = kStack;
        g_fiber[t].ctx.uc_link = nullptr;
        makecontext(&g_fiber[t].ctx, fiber_main, 0);
        g_fiber[t].done = false;
    }
    bool any = true;
    while (any) {
        any = false;
        for (int t = 0; t < kGroup; ++t) {
            if (g_fiber[t].done) continue;
            g_cur = t;
            swapcontext(&g_sched, &g_fiber[t].ctx);
            any = true;
        }
    }
}

void dispatch(KernelFn k, int numGroups, bool barriers) {
    for (int g = 0; g < numGroups; ++g) {
        if (barriers) {
            run_group_with_barriers(k, (uint)g);
        } else {
            for (int t = 0; t < kGroup; ++t) k((uint)t, uint3((uint)g, 0, 0), uint3((uint)(g * kGroup + t), 0, 0));
        }
    }
}
}  // namespace

void GroupMemoryBarrierWithGroupSync() { swapcontext(&g_fiber[g_cur].ctx, &g_sched); }

// ------------------------------------------------------------------------------------ C interface
struct SimParamsF {
    float wind[4], wind1[4], wind2[4], wind3[4];
    float shape[4];
    float gravTimeTip[4];
    int32_t simInts[4];
    int32_t counts[4];
    float vsp[4];
    float resetPositions, clampPositionDelta, pad1, pad2;
    float bones[512][16];
};

struct HairF {
    int32_t G, n, F, pad;
    float* pos; float* prev; float* prevprev; float* tan; float* sld;
    float* init; float* rest; float* followOffset; float* skin;
};

struct SdfParamsF {
    float origin[4];
    float cellSize;
    int32_t nx, ny, nz;
};

static float4 f4(const float* p) { return float4(p[0], p[1], p[2], p[3]); }

static void load_bones(HArray<float4x4, 512>& dst, const float (*bones)[16]) {
    for (int b = 0; b < 512; ++b)
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) dst.a[b].m[r][c] = bones[b][4 * r + c];
}

static void bind_sim(const HairF* h, const SimParamsF* cb) {
    using namespace ref_sim;
    const int64_t S = (int64_t)h->G * (h->F + 1), V = S * h->n;
    g_HairVertexPositions.bind(h->pos, V);
    g_HairVertexPositionsPrev.bind(h->prev, V);
    g_HairVertexPositionsPrevPrev.bind(h->prevprev, V);
    g_HairVertexTangents.bind(h->tan, V);
    g_StrandLevelData.bind(h->sld, S);
    g_InitialHairPositions.bind(h->init, V);
    g_HairRestLengthSRV.bind(h->rest, V);
    g_FollowHairRootOffset.bind(h->followOffset, S);
    g_BoneSkinningData.bind(h->skin, S);
    g_Wind = f4(cb->wind); g_Wind1 = f4(cb->wind1); g_Wind2 = f4(cb->wind2); g_Wind3 = f4(cb->wind3);
    g_Shape = f4(cb->shape);
    g_GravTimeTip = f4(cb->gravTimeTip);
    for (int i = 0; i < 4; ++i) { g_SimInts[i] = cb->simInts[i]; g_Counts[i] = cb->counts[i]; }
    g_VSP = f4(cb->vsp);
    g_ResetPositions = cb->resetPositions;
    g_ClampPositionDelta = cb->clampPositionDelta;
    load_bones(g_BoneSkinningMatrix, cb->bones);
}

enum { K_INTEGRATE = 1, K_STRAND_LEVEL = 2, K_VSP = 3, K_LOCAL_SHAPE = 4, K_LENGTH_WIND = 5, K_FOLLOW = 6 };

// One EI Dispatch of a simulation kernel with the reference's group count.
extern "C" int tfxr_sim_dispatch(int kernel, const HairF* h, const SimParamsF* cb) {
    bind_sim(h, cb);
    const int64_t S = (int64_t)h->G * (h->F + 1), V = S * h->n;
    const int vGroups = (int)((float)V / (float)kGroup);
    const int sGroups = (int)((float)S / (float)kGroup);
    switch (kernel) {
        case K_INTEGRATE: dispatch(ref_sim::IntegrationAndGlobalShapeConstraints, vGroups, true); break;
        case K_STRAND_LEVEL: dispatch(ref_sim::CalculateStrandLevelData, sGroups, false); break;
        case K_VSP: dispatch(ref_sim::VelocityShockPropagation, vGroups, false); break;
        case K_LOCAL_SHAPE: dispatch(ref_sim::LocalShapeConstraints, sGroups, false); break;
        case K_LENGTH_WIND: dispatch(ref_sim::LengthConstriantsWindAndCollision, vGroups, true); break;
        case K_FOLLOW: dispatch(ref_sim::UpdateFollowHairVertices, vGroups, true); break;
        default: return 1;
    }
    return 0;
}

static void bind_sdf(const SdfParamsF* g, uint32_t* sdf, int64_t allocCells) {
    using namespace ref_sdf;
    g_Origin = float4(g->origin[0], g->origin[1], g->origin[2], 0.0f);
    g_CellSize = g->cellSize;
    g_NumCellsX = g->nx; g_NumCellsY = g->ny; g_NumCellsZ = g->nz;
    g_SignedDistanceField.bind(sdf, allocCells);
}

// TressFXSDFCollision::Update: Initialize / Construct / Finalize with the reference's group counts
// (the 1.4x allocation drives the cell-level dispatch size).
extern "C" int tfxr_sdf_update(uint32_t* sdf, int64_t allocCells, const SdfParamsF* g, const float* mesh, int nverts,
                               const uint32_t* idx, int ntri) {
    using namespace ref_sdf;
    bind_sdf(g, sdf, allocCells);
    g_TrimeshVertexIndices.bind((void*)idx, 3 * (int64_t)ntri);
    collMeshVertexPositions.bind((void*)mesh, nverts);
    const int cellGroups = (int)std::ceil((float)allocCells / (float)kGroup);
    dispatch(InitializeSignedDistanceField, cellGroups, false);
    dispatch(ConstructSignedDistanceField, (int)std::ceil((float)ntri / (float)kGroup), false);
    dispatch(FinalizeSignedDistanceField, cellGroups, false);
    return 0;
}

// TressFXSDFCollision::CollideWithHair: CollideHairVerticesWithSdf_forward over every vertex.
extern "C" int tfxr_sdf_collide(uint32_t* sdf, int64_t allocCells, const SdfParamsF* g, float marginWorld,
                                const HairF* h) {
    using namespace ref_sdf;
    bind_sdf(g, sdf, allocCells);
    const int64_t V = (int64_t)h->G * (h->F + 1) * h->n;
    g_HairVertices.bind(h->pos, V);
    g_PrevHairVertices.bind(h->prev, V);
    g_CollisionMargin = marginWorld;
    g_NumTotalHairVertices = (int)V;
    g_NumHairVerticesPerStrand = h->n;
    dispatch(CollideHairVerticesWithSdf_forward, (int)std::ceil((float)V / (float)kGroup), false);
    return 0;
}

// CollideHairVerticesWithSdf (the mixed-difference variant) over every vertex.
extern "C" int tfxr_sdf_collide_mixed(uint32_t* sdf, int64_t allocCells, const SdfParamsF* g, float marginWorld,
                                      const HairF* h) {
    using namespace ref_sdf;
    bind_sdf(g, sdf, allocCells);
    const int64_t V = (int64_t)h->G * (h->F + 1) * h->n;
    g_HairVertices.bind(h->pos, V);
    g_PrevHairVertices.bind(h->prev, V);
    g_CollisionMargin = marginWorld;
    g_NumTotalHairVertices = (int)V;
    g_NumHairVerticesPerStrand = h->n;
    dispatch(CollideHairVerticesWithSdf, (int)std::ceil((float)V / (float)kGroup), false);
    return 0;
}

// TressFXBoneSkinning::Update: BoneSkinning over every mesh vertex.
extern "C" int tfxr_mesh_skin(float* out, const float* in, const float* skin, const float (*bones)[16], int nverts) {
    using namespace ref_skin;
    bs_collMeshVertexPositions.bind(out, nverts);
    bs_initialVertexPositions.bind((void*)in, nverts);
    bs_boneSkinningData.bind((void*)skin, nverts);
    g_NumMeshVertices[0] = nverts;
    load_bones(g_BoneSkinningMatrix, bones);
    dispatch(BoneSkinning, (int)std::ceil((float)nverts / (float)kGroup), false);
    return 0;
}

// GetExpandedTressFXVert / GetExpandedTressFXShadowVert (TressFXStrands.hlsl) for every vertex id
// [0, 2 * Vtot): out = {Position, Tangent, p0p1, StrandColor} per id (16 floats).  params = the
// TressFXStrandParameters members in declaration order (MatBaseColor[4], MatTipColor[4], TipPercentage,
// StrandUVTilingFactor, FiberRatio, FiberRadius as floats, then NumVerticesPerStrand, EnableThinTip
// as ints); viewProj row-major, applied as mul(M, v).
extern "C" int tfxr_expand_strands(const float* pos, const float* tan, int64_t vtot, const float* fparams,
                                   const int* iparams, const float* eye, const float* win, const float* viewProj,
                                   int shadow, float* out) {
    using namespace ref_strands;
    g_GuideHairVertexPositions.bind((void*)pos, vtot);
    g_GuideHairVertexTangents.bind((void*)tan, vtot);
    MatBaseColor = float4(fparams[0], fparams[1], fparams[2], fparams[3]);
    MatTipColor = float4(fparams[4], fparams[5], fparams[6], fparams[7]);
    TipPercentage = fparams[8];
    StrandUVTilingFactor = fparams[9];
    FiberRatio = fparams[10];
    FiberRadius = fparams[11];
    NumVerticesPerStrand = iparams[0];
    EnableThinTip = iparams[1];
    const int64_t strands = vtot / NumVerticesPerStrand;
    std::vector<float2> texcd((size_t)strands);
    g_HairStrandTexCd.bind(texcd.data(), strands);
    float4x4 vp;
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) vp.m[r][c] = viewProj[4 * r + c];
    const float3 e(eye[0], eye[1], eye[2]);
    const float2 w(win[0], win[1]);
    for (int64_t id = 0; id < 2 * vtot; ++id) {
        TressFXVertex o = shadow ? GetExpandedTressFXShadowVert((uint)id, e, w, vp) : GetExpandedTressFXVert((uint)id, e, w, vp);
        const float4 f[4] = {o.Position, o.Tangent, o.p0p1, o.StrandColor};
        for (int k = 0; k < 4; ++k)
            for (int c = 0; c < 4; ++c) out[16 * id + 4 * k + c] = f[k][c];
    }
    return 0;
}

// The reference's MARCHING_CUBES_EDGE_TABLE[256] and MARCHING_CUBES_TRIANGLE_TABLE[256*16].
extern "C" int tfxr_mc_tables(int32_t* edge, int32_t* tri) {
    for (int i = 0; i < 256; ++i) edge[i] = MARCHING_CUBES_EDGE_TABLE[i];
    for (int i = 0; i < 256 * 16; ++i) tri[i] = MARCHING_CUBES_TRIANGLE_TABLE[i];
    return 0;
}

// TressFXSDFMarchingCubes::Update (TressFXSDFMarchingCubes.cpp:168-232): InitializeMCVertices over
// ceil(max / 64) groups, then RunMarchingCubesOnSdf over ceil(X*Y*Z / 64) groups, with the caller's
// tables.  out = {position, normal}[maxVerts] (8 floats each); sdf = the finalized grid words.
extern "C" int tfxr_marching_cubes(const uint32_t* sdf, int64_t allocCells, const SdfParamsF* g, float iso,
                                   const int32_t* edge, const int32_t* tri, int maxVerts, float* out, int32_t* counter) {
    using namespace ref_mc;
    g_MarchingCubesSignedDistanceField.bind((void*)sdf, allocCells);
    g_MarchingCubesTriangleVertices.bind(out, maxVerts);
    g_NumMarchingCubesVertices.bind(counter, 1);
    g_MarchingCubesEdgeTable.bind((void*)edge, 256);
    g_MarchingCubesTriangleTable.bind((void*)tri, 256 * 16);
    g_Origin = float4(g->origin[0], g->origin[1], g->origin[2], 0.0f);
    g_CellSize = g->cellSize;
    g_NumCellsX = g->nx; g_NumCellsY = g->ny; g_NumCellsZ = g->nz;
    g_MaxMarchingCubesVertices = maxVerts;
    g_MarchingCubesIsolevel = iso;
    const int64_t cells = (int64_t)g->nx * g->ny * g->nz;
    dispatch(InitializeMCVertices, (int)std::ceil((float)maxVerts / (float)kGroup), false);
    dispatch(RunMarchingCubesOnSdf, (int)std::ceil((float)cells / (float)kGroup), false);
    return 0;
}
