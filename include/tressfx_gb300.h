/*
 * tressfx_gb300.h -- C ABI of the GB300 (sm_103a) TressFX strand-simulation + SDF-collision library.
 *
 * The reference drives its HLSL compute shaders through the Engine Interface (EI):
 * EI_Device::CreateBufferResource / CreateComputeShaderPSO / CreateBindSet and
 * EI_CommandContext::BindPSO / BindSets / Dispatch / UpdateBuffer / SubmitBarrier
 * (src/EngineInterface.h:23-31, src/DX12/DX12EngineInterfaceImpl.cpp:1000-1014, 1600, 1638-1650).
 * This header is the replacement for that compute path: plain pointers, sizes and opaque handles,
 * every call returns an int status (0 = TFX_OK), nothing throws across it, and all device work is
 * issued in order on the CUDA stream owned by a tfx_context (the EI_CommandContext).
 *
 * Layout conventions (identical to the reference buffers, TressFXHairObject.cpp:60-105):
 *   - vertex buffers are float4 (16 B), strand-major: vertex j of strand s sits at s*n + j;
 *   - follow strands follow their guide: guide g is strand g*(F+1), its follows g*(F+1)+1..+F;
 *   - position.w is the inverse mass, w <= 0 marks an immovable vertex;
 *   - bone matrices are 16 floats, row-major, row-vector convention (p' = [p 1] * M), as the
 *     shader's `row_major float4x4 g_BoneSkinningMatrix[]` reads them (TressFXSimulation.hlsl:70).
 */
#ifndef TRESSFX_GB300_H_
#define TRESSFX_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TFX_ABI_VERSION 1
#define TFX_MAX_BONES 512              /* AMD_TRESSFX_MAX_NUM_BONES, src/TressFX/AMD_TressFX.h:45-47 */
#define TFX_THREAD_GROUP_SIZE 64       /* TRESSFX_SIM_THREAD_GROUP_SIZE, src/TressFX/TressFXCommon.h:34 */

/* ---------------------------------------------------------------------------------- status */
typedef enum tfx_status {
    TFX_OK = 0,
    TFX_ERR_INVALID_ARGUMENT = 1,   /* null handle/pointer, negative count, unknown id          */
    TFX_ERR_VERTS_PER_STRAND = 2,   /* n not in {4, 8, 16, 32, 64} (TressFXAsset.cpp:115-118)    */
    TFX_ERR_BONE_INDEX = 3,         /* a skinning bone index outside [0, 512)                    */
    TFX_ERR_BONE_WEIGHTS = 4,       /* skinning weights whose shader-side sum is <= 0            */
    TFX_ERR_CUDA = 5,               /* a CUDA runtime call or kernel launch failed               */
    TFX_ERR_OUT_OF_MEMORY = 6,
    TFX_ERR_TIMEOUT = 7,            /* a bounded device-side wait gave up                        */
    TFX_ERR_SIZE = 8,               /* counts that overflow the 32-bit vertex index space        */
    TFX_ERR_MISMATCH = 9,           /* constants whose counts disagree with the object           */
    TFX_ERR_NO_DEVICE = 10          /* no CUDA device, or not an sm_103 device                   */
} tfx_status;

/* Human-readable name of a status code. */
const char* tfx_status_string(int status);
/* Message of the last failing call on this host thread ("" if none). */
const char* tfx_last_error(void);
/* TFX_ABI_VERSION of the loaded library. */
int tfx_abi_version(void);

/* ---------------------------------------------------------------------------------- handles */
typedef struct tfx_context_t* tfx_context;   /* EI_CommandContext: one CUDA stream            */
typedef struct tfx_hair_t* tfx_hair;         /* TressFXHairObject + TressFXDynamicState       */
typedef struct tfx_sdf_t* tfx_sdf;           /* TressFXSDFCollision's signed distance grid    */
typedef struct tfx_mesh_t* tfx_mesh;         /* TressFXBoneSkinning's skinned collision mesh  */

/* Kernel ids: one per reference compute entry point. */
typedef enum tfx_kernel {
    TFX_KERNEL_INTEGRATION_AND_GLOBAL_SHAPE = 1, /* IntegrationAndGlobalShapeConstraints, TressFXSimulation.hlsl:609-666 */
    TFX_KERNEL_STRAND_LEVEL_DATA = 2,            /* CalculateStrandLevelData,             TressFXSimulation.hlsl:677-728 */
    TFX_KERNEL_VELOCITY_SHOCK_PROPAGATION = 3,   /* VelocityShockPropagation,             TressFXSimulation.hlsl:739-762 */
    TFX_KERNEL_LOCAL_SHAPE_CONSTRAINTS = 4,      /* LocalShapeConstraints,                TressFXSimulation.hlsl:773-829 */
    TFX_KERNEL_LENGTH_WIND_COLLISION = 5,        /* LengthConstriantsWindAndCollision,    TressFXSimulation.hlsl:875-975 */
    TFX_KERNEL_UPDATE_FOLLOW_HAIR = 6,           /* UpdateFollowHairVertices,             TressFXSimulation.hlsl:978-1001 */
    TFX_KERNEL_SDF_INITIALIZE = 7,               /* InitializeSignedDistanceField,        TressFXSDFCollision.hlsl:301-312 */
    TFX_KERNEL_SDF_CONSTRUCT = 8,                /* ConstructSignedDistanceField,         TressFXSDFCollision.hlsl:329-397 */
    TFX_KERNEL_SDF_FINALIZE = 9,                 /* FinalizeSignedDistanceField,          TressFXSDFCollision.hlsl:400-412 */
    TFX_KERNEL_SDF_COLLIDE = 10,                 /* CollideHairVerticesWithSdf_forward,   TressFXSDFCollision.hlsl:531-595 */
    TFX_KERNEL_MESH_BONE_SKINNING = 11           /* BoneSkinning,                         TressFXBoneSkinning.hlsl:57-94 */
} tfx_kernel;

/* Buffer ids of a hair object (TressFXDynamicState + TressFXHairObject SRVs). */
typedef enum tfx_buffer {
    TFX_BUF_POSITIONS = 1,           /* float4[Vtot]  UAV  m_Positions                 */
    TFX_BUF_POSITIONS_PREV = 2,      /* float4[Vtot]  UAV  m_PositionsPrev             */
    TFX_BUF_POSITIONS_PREV_PREV = 3, /* float4[Vtot]  UAV  m_PositionsPrevPrev         */
    TFX_BUF_TANGENTS = 4,            /* float4[Vtot]  UAV  m_Tangents                  */
    TFX_BUF_STRAND_LEVEL_DATA = 5,   /* float4[3*Stot] UAV m_StrandLevelData           */
    TFX_BUF_INITIAL_POSITIONS = 6,   /* float4[Vtot]  SRV  m_InitialHairPositionsBuffer */
    TFX_BUF_REST_LENGTHS = 7,        /* float[Vtot]   SRV  m_HairRestLengthSRVBuffer    */
    TFX_BUF_FOLLOW_ROOT_OFFSETS = 8, /* float4[Stot]  SRV  m_FollowHairRootOffsetBuffer */
    TFX_BUF_BONE_SKINNING = 9        /* float4[2*Stot] SRV m_BoneSkinningDataBuffer     */
} tfx_buffer;

/* ---------------------------------------------------------------------------------- constants */
/* Byte-for-byte TressFXSimulationParams (src/TressFX/TressFXConstantBuffers.h:41-85,
 * capsules compiled out) = cbuffer tressfxSimParameters (TressFXSimulation.hlsl:49-79). */
typedef struct tfx_sim_params {
    float wind[4], wind1[4], wind2[4], wind3[4];
    float shape[4];          /* damping, local stiffness, global stiffness, global range */
    float grav_time_tip[4];  /* gravity magnitude, time step, tip separation            */
    int32_t sim_ints[4];     /* length iterations, local iterations, collision flag     */
    int32_t counts[4];       /* strands per thread group (64/n), follows per guide, n   */
    float vsp[4];            /* VSP coefficient, VSP acceleration threshold             */
    float reset_positions;
    float clamp_position_delta;
    float pad1, pad2;
    float bone_matrices[TFX_MAX_BONES][16];
} tfx_sim_params;

/* TressFXSimulationSettings (src/TressFX/TressFXSettings.h:35-87), the user-facing knobs. */
typedef struct tfx_sim_settings {
    float vsp_coeff;
    float vsp_accel_threshold;
    float local_constraint_stiffness;
    int32_t local_constraints_iterations;
    float global_constraint_stiffness;
    float global_constraints_range;
    int32_t length_constraints_iterations;
    float damping;
    float gravity_magnitude;
    float tip_separation;
    float wind_magnitude;
    float wind_direction[3];
    float wind_angle_radians;
    float clamp_position_delta;
} tfx_sim_settings;

/* Fill `settings` with the TressFXSimulationSettings defaults (TressFXSettings.h:38-56). */
int tfx_sim_settings_default(tfx_sim_settings* settings);

/* TressFXHairObject::UpdateSimulationParameters (TressFXHairObject.cpp:380-437) on a host-side
 * constant block: writes every field it writes (wind via SetWind, :191-235), leaves the bone
 * matrices alone, sets reset_positions = 1 when frame < 2, and returns the number of
 * local-shape re-dispatches (m_CPULocalShapeIterations) in *cpu_local_iterations.
 * Host-only: needs no device. */
int tfx_fill_sim_params(tfx_sim_params* params, const tfx_sim_settings* settings, float time_step,
                        int verts_per_strand, int follow_hairs_per_guide, int simulation_frame,
                        int32_t* cpu_local_iterations);

/* ---------------------------------------------------------------------------------- context */
/* EI_Device + EI_CommandContext: selects `device` and creates a non-blocking stream. */
int tfx_context_create(int device, tfx_context* out);
int tfx_context_destroy(tfx_context ctx);
/* Blocks until all work issued on the context's stream has finished (WaitForCompute). */
int tfx_context_synchronize(tfx_context ctx);
/* The context's cudaStream_t, as void*. */
void* tfx_context_stream(tfx_context ctx);
/* GetTimeStamp(name) (src/EngineInterface.h / DX12EngineInterfaceImpl.cpp:1319-1322): records a
 * named CUDA event on the stream; tfx_context_timestamps returns up to `max` (name, ms since the
 * first stamp) pairs of the completed stamps and clears the list. */
int tfx_context_timestamp(tfx_context ctx, const char* name);
int tfx_context_timestamps(tfx_context ctx, char (*names)[64], float* ms, int max, int* count);

/* Page-locked host memory for overlapped uploads / read-backs (cudaHostAlloc, portable). */
int tfx_host_alloc(size_t bytes, void** out);
int tfx_host_free(void* ptr);

/* ---------------------------------------------------------------------------------- hair object */
typedef struct tfx_hair_desc {
    int32_t num_guide_strands;     /* G: guide strands (m_numGuideStrands)                 */
    int32_t verts_per_strand;      /* n in {4, 8, 16, 32, 64}                               */
    int32_t follow_hairs_per_guide;/* F >= 0; Stot = G*(F+1), Vtot = Stot*n                 */
    int32_t reserved;
} tfx_hair_desc;

/* TressFXHairObject ctor (TressFXHairObject.cpp:44-164) + TressFXDynamicState::CreateGPUResources
 * / UploadGPUData (:502-558).  Host arrays are copied:
 *   positions            float4[Vtot]   -> Pos, Prev, PrevPrev and InitialPositions
 *   tangents             float4[Vtot]   -> Tangents (NULL = zeros)
 *   rest_lengths         float[Vtot]    -> RestLength SRV
 *   follow_root_offsets  float4[Stot]   -> RootOffset SRV (NULL = zeros)
 *   bone_skinning        {float4 boneIndex, float4 boneWeight}[Stot] -> SkinningData SRV
 * Validates n, index-space size, bone indices and weights of every guide strand. */
int tfx_hair_create(tfx_context ctx, const tfx_hair_desc* desc, const float* positions,
                    const float* tangents, const float* rest_lengths, const float* follow_root_offsets,
                    const float* bone_skinning, tfx_hair* out);
int tfx_hair_destroy(tfx_hair hair);
/* The host-side checks of tfx_hair_create without a device: n, index-space size, and the bone
 * indices / weights of every guide strand exactly as ApplyVertexBoneSkinning reads them
 * (TressFXSimulation.hlsl:552-564). Returns the status tfx_hair_create would return for them. */
int tfx_hair_validate(const tfx_hair_desc* desc, const float* bone_skinning);
/* TressFXHairObject::UpdateConstantBuffer (TressFXHairObject.cpp:375-378): uploads the scalar
 * block and bone matrices [0, num_bones) of `params` for the next dispatches (stream ordered;
 * the host block may be reused as soon as the call returns). counts must equal (64/n, F, n). */
int tfx_hair_update_constants(tfx_hair hair, const tfx_sim_params* params, int num_bones);
/* One EI Dispatch of a simulation kernel over the whole object (TressFXSimulation.cpp:51-75),
 * repeated `repeat` times (the local-shape re-dispatch loop, :64-72). */
int tfx_hair_dispatch(tfx_hair hair, int kernel, int repeat);
/* TressFXSimulation::Simulate for one object (TressFXSimulation.cpp:77-112): the six stages in
 * order, local shape dispatched `cpu_local_iterations` times. */
int tfx_hair_simulate(tfx_hair hair, int cpu_local_iterations);
/* Stream-ordered, blocking copies between a buffer and host memory (snapshot / restore). */
int tfx_hair_read(tfx_hair hair, int buffer, void* host_dst, size_t bytes);
int tfx_hair_write(tfx_hair hair, int buffer, const void* host_src, size_t bytes);
/* Asynchronous variants: the caller keeps host memory alive (and pinned for overlap) until the
 * stream reaches the copy. */
int tfx_hair_read_async(tfx_hair hair, int buffer, void* host_dst, size_t bytes);
int tfx_hair_write_async(tfx_hair hair, int buffer, const void* host_src, size_t bytes);
/* Device address and byte size of a buffer (for a renderer or any interop). */
int tfx_hair_get_buffer(tfx_hair hair, int buffer, void** device_ptr, size_t* bytes);
/* out[0..3] = total vertices, total strands, vertices per strand, follow hairs per guide
 * (GetNumTotalHairVertices / Strands / VerticesPerStrand / FollowHairsPerGuideHair). */
int tfx_hair_get_counts(tfx_hair hair, int32_t out[4]);
/* Health check (report only): counts[0] / counts[1] = vertices of Pos / Prev with a NaN or infinite
 * component, after the work queued so far (synchronous).  The reference's only guard is the
 * velocity clamp (TressFXSimulation.hlsl:959-964), which a NaN passes through; the caller resets or
 * restores the object when a count is non-zero. */
int tfx_hair_count_nonfinite(tfx_hair hair, int64_t counts[2]);

/* ---------------------------------------------------------------------------------- strand quads */
/* TressFXStrandParams (TressFXConstantBuffers.h) = cbuffer TressFXStrandParameters
 * (TressFXRendering.hlsl:61-80). */
typedef struct tfx_strand_params {
    float mat_base_color[4];
    float mat_tip_color[4];
    float tip_percentage;
    float strand_uv_tiling_factor;
    float fiber_ratio;
    float fiber_radius;
    int32_t num_vertices_per_strand;
    int32_t enable_thin_tip;
    int32_t node_pool_size;
    int32_t render_params_index;
    int32_t enable_strand_uv;
    int32_t enable_strand_tangent;
    int32_t padding[2];
} tfx_strand_params;
/* GetExpandedTressFXVert (shadow = 0) or GetExpandedTressFXShadowVert (shadow = 1) of
 * TressFXStrands.hlsl for every vertex id [0, 2 * Vtot) of the hair object, headless: out_device
 * receives {Position, Tangent, p0p1, StrandColor} (4 float4) per id; the shadow form writes the
 * position and zeros.  view_proj: 16 floats, row-major, applied as mul(M, v).  The root colour is
 * mat_base_color (the albedo texture the shader samples is taken as white). */
int tfx_hair_expand_strands(tfx_hair hair, const tfx_strand_params* params, const float eye[3], const float win_size[2],
                            const float view_proj[16], int shadow, void* out_device);

/* ---------------------------------------------------------------------------------- SDF */
/* TressFXSDFCollisionParams (TressFXConstantBuffers.h:119-134), the grid part of it. */
typedef struct tfx_sdf_grid {
    float origin[4];
    float cell_size;
    int32_t num_cells_x, num_cells_y, num_cells_z;
} tfx_sdf_grid;

/* Grid sizing of the TressFXSDFCollision ctor (TressFXSDFCollision.cpp:38-86) from the mesh's
 * initial bounding box: cell = (max.x-min.x)/numCellsInX, padding = (int)(0.8*numCellsInX)
 * cells, dims = (int)((bbox + 2*padding)/cell), allocation = (int)(1.4*X*Y*Z) cells.
 * Host-only. */
int tfx_sdf_grid_from_bbox(const float bbox_min[3], const float bbox_max[3], int num_cells_in_x,
                           tfx_sdf_grid* grid, float* padding, int64_t* alloc_cells);
/* UpdateSDFGrid (TressFXSDFCollision.cpp:88-93): origin = current bbox min - padding. */
int tfx_sdf_grid_origin(const float bbox_min[3], float padding, tfx_sdf_grid* grid);

/* Allocates the grid buffer (uint32[alloc_cells], alloc_cells >= X*Y*Z of any grid used later). */
int tfx_sdf_create(tfx_context ctx, int64_t alloc_cells, tfx_sdf* out);
int tfx_sdf_destroy(tfx_sdf sdf);
/* Binds the collision mesh (TressFXSDFInputMeshInterface::GetMeshBuffer /
 * GetTrimeshVertexIndicesBuffer, TressFXSDFInputMeshInterface.h:38-48): borrowed DEVICE pointers
 * to {float4 position, float4 normal}[num_vertices] and uint32[3*num_triangles]. */
int tfx_sdf_set_mesh(tfx_sdf sdf, const void* mesh_vertices, int num_vertices, const uint32_t* indices,
                     int num_triangles);
/* TressFXSDFCollision::Update (TressFXSDFCollision.cpp:95-169): Initialize, Construct, Finalize
 * on `grid` (cells X*Y*Z <= allocation). */
int tfx_sdf_update(tfx_sdf sdf, const tfx_sdf_grid* grid);
/* One SDF kernel alone (SDF_INITIALIZE / SDF_CONSTRUCT / SDF_FINALIZE) on `grid`. */
int tfx_sdf_dispatch(tfx_sdf sdf, int kernel, const tfx_sdf_grid* grid);
/* TressFXSDFCollision::CollideWithHair (TressFXSDFCollision.cpp:171-221): margin_world =
 * collisionMargin * cellSize (:194), applied to every vertex of the object. */
int tfx_sdf_collide(tfx_sdf sdf, tfx_hair hair, const tfx_sdf_grid* grid, float margin_world);
/* CollideHairVerticesWithSdf (TressFXSDFCollision.hlsl:599-715), the shader's faster variant that the
 * reference's host code does not dispatch: every vertex (roots included), one 8-corner fetch, the
 * gradient by forward or backward differences inside the same cell. */
int tfx_sdf_collide_mixed(tfx_sdf sdf, tfx_hair hair, const tfx_sdf_grid* grid, float margin_world);
int tfx_sdf_read(tfx_sdf sdf, void* host_dst, size_t bytes);
int tfx_sdf_write(tfx_sdf sdf, const void* host_src, size_t bytes);
int tfx_sdf_get_buffer(tfx_sdf sdf, void** device_ptr, size_t* bytes);

/* Largest grid (X*Y*Z cells) that tfx_sdf_build_static accepts: 128^3, 8 MiB of scratch words. */
#define TFX_SDF_STATIC_MAX_CELLS 2097152
/* No counterpart in the reference.  Initialize + Construct + Finalize of `grid` from a DEVICE mesh
 * ({float4 position, float4 normal}[num_vertices], uint32[3*num_triangles]) into the DEVICE float
 * buffer sdf_out[X*Y*Z], the same grid tfx_sdf_update builds, without allocating anything: for
 * callers that may not allocate device memory once running (an engine with a fixed GPU memory
 * budget set at start-up, or a frame being recorded for replay).  The FloatFlip3 build words live
 * in one static device array per device (TFX_SDF_STATIC_MAX_CELLS words; larger grids return
 * TFX_ERR_SIZE).  Nothing has to be zeroed first.  The first call on a context looks the array's
 * address up and keeps it in the context (make that call before any stream capture).  Calls that
 * can overlap on one device (other contexts or streams) race on that array; calls on one context
 * are stream-ordered.  Triangle indices must be below num_vertices: they are not checked.  The
 * caller's current device is left as it was. */
int tfx_sdf_build_static(tfx_context ctx, const tfx_sdf_grid* grid, const void* mesh_vertices, int num_vertices,
                         const uint32_t* indices, int num_triangles, float* sdf_out);

/* ---------------------------------------------------------------------------------- SDF marching cubes */
/* TressFXSDFMarchingCubes (src/TressFX/TressFXSDFMarchingCubes.{h,cpp}): the iso-surface of a signed
 * distance grid as a triangle soup in a device buffer of {float4 position, float4 normal}
 * [max_vertices] (StandardVertex of TressFXMarchingCubes.hlsl:33-37), headless. */
typedef struct tfx_mc_t* tfx_mc;
/* Constructor + Initialize (TressFXSDFMarchingCubes.cpp:27-118): the vertex buffer (128*1024 vertices
 * in the reference), the counter, and scratch for grids of up to max_cells cells (< 2^31 - 256).  The
 * tables start as tfx_mc_default_tables'; the iso level starts at 0. */
int tfx_mc_create(tfx_context ctx, int max_vertices, int64_t max_cells, tfx_mc* out);
int tfx_mc_destroy(tfx_mc mc);
/* The library's own tables in the layout of MARCHING_CUBES_EDGE_TABLE[256] and
 * MARCHING_CUBES_TRIANGLE_TABLE[256*16] (src/MarchingCubesTables.h): a bit per crossing edge, and up
 * to five triangles of edge indices per configuration, -1 terminated.  Built from the cube's faces,
 * they separate the inside corners on every ambiguous face the same way in both cubes that share it,
 * so the surface is closed across cubes.  Host-only. */
int tfx_mc_default_tables(int32_t* edge_table, int32_t* tri_table);
/* Uploads the two tables the kernel reads (the reference's Initialize uploads its own,
 * TressFXSDFMarchingCubes.cpp:95-99); passing the reference's reproduces its triangles exactly.
 * Both null restores the defaults.  Triangle entries must be -1 or an edge 0..11. */
int tfx_mc_set_tables(tfx_mc mc, const int32_t* edge_table, const int32_t* tri_table);
/* SetSDFIsoLevel (TressFXSDFMarchingCubes.h:69), in cells: the surface is value = cell_size * iso. */
int tfx_mc_set_iso_level(tfx_mc mc, float iso_level);
/* Update (TressFXSDFMarchingCubes.cpp:168-232): InitializeMCVertices + RunMarchingCubesOnSdf over the
 * finalized grid of `sdf`.  The vertex order is cell-index order (the reference's atomic append
 * order is unspecified); a cube is written only if its vertices end below max_vertices, and the
 * counter holds the vertices every cube reserved, as the shader's counter does.  Vertices not
 * written are zero.  Stream-ordered; nothing synchronizes. */
int tfx_mc_update(tfx_mc mc, tfx_sdf sdf, const tfx_sdf_grid* grid);
/* The same over any DEVICE float grid [X*Y*Z] (a batch SDF, tfx_sdf_build_static's output). */
int tfx_mc_run(tfx_mc mc, const float* sdf_device, const tfx_sdf_grid* grid);
int tfx_mc_get_buffers(tfx_mc mc, void** vertices, int32_t** num_vertices);
/* Copies `bytes` of the vertex buffer and the counter to the host (synchronizes the stream). */
int tfx_mc_read(tfx_mc mc, void* host_vertices, size_t bytes, int32_t* num_vertices);

/* ---------------------------------------------------------------------------------- collision mesh */
/* TressFXBoneSkinning::Initialize (TressFXBoneSkinning.cpp:287-404): uploads the bind-pose mesh
 * {float4 position, float4 normal}[num_vertices], uint32[3*num_triangles] and per-vertex
 * {float4 boneIndex, float4 boneWeight}[num_vertices]. */
int tfx_mesh_create(tfx_context ctx, const float* vertices, int num_vertices, const uint32_t* indices,
                    int num_triangles, const float* bone_skinning, tfx_mesh* out);
int tfx_mesh_destroy(tfx_mesh mesh);
/* TressFXBoneSkinning::Update (TressFXBoneSkinning.cpp:460-504): uploads `num_bones` bone
 * matrices and runs the BoneSkinning kernel into the skinned vertex buffer. */
int tfx_mesh_skin(tfx_mesh mesh, const float* bone_matrices, int num_bones);
/* Device pointers of the skinned vertex buffer and the index buffer (to feed tfx_sdf_set_mesh). */
int tfx_mesh_get_buffers(tfx_mesh mesh, void** skinned_vertices, void** indices, int32_t* num_vertices,
                         int32_t* num_triangles);
int tfx_mesh_read_skinned(tfx_mesh mesh, float* host_dst, size_t bytes);

/* ---------------------------------------------------------------------------------- batched path */
/* The whole per-frame sequence of Simulation::StartSimulation (src/Simulation.cpp:50-94) for many
 * objects at once: skin every collision mesh, rebuild every SDF, run TressFXSimulation::Simulate
 * (TressFXSimulation.cpp:77-112) over every hair object and CollideWithHair
 * (TressFXSDFCollision.cpp:171-221) for each object with its SDF -- as one CUDA-graph launch of a
 * few persistent kernels instead of one dispatch per object per stage.  Results are bit-identical
 * to the per-object dispatches above.  Objects keep their own buffers (tfx_hair_read / _get_buffer
 * see the batched results); the mesh bound to an SDF must not change after tfx_batch_build. */
typedef struct tfx_batch_t* tfx_batch;

int tfx_batch_create(tfx_context ctx, tfx_batch* out);
int tfx_batch_destroy(tfx_batch batch);
/* Registers an SDF whose grid is nx*ny*nz cells every frame; `mesh` (or NULL for the mesh already
 * bound with tfx_sdf_set_mesh) is skinned by the batch before the SDF is rebuilt. */
int tfx_batch_add_sdf(tfx_batch batch, tfx_sdf sdf, tfx_mesh mesh, int nx, int ny, int nz, int* index);
/* Registers a hair object that collides with SDF `sdf_index` (-1: no collision). */
int tfx_batch_add_hair(tfx_batch batch, tfx_hair hair, int sdf_index, int* index);
/* Makes hair object `hair_index` also collide with SDF `sdf_index`, after the SDFs it already collides
 * with, in the order of these calls: Simulation::RunCollision applies every collision mesh to every
 * hair object in turn (src/Simulation.cpp:106-118).  The hair object must have been added with an
 * SDF, and collides with each SDF once. */
int tfx_batch_add_hair_collision(tfx_batch batch, int hair_index, int sdf_index);
/* Builds the object / work / tile tables and captures the frame graphs (reserved must be 0). */
int tfx_batch_build(tfx_batch batch, int reserved);
/* Times the candidate launch shapes over `frames` frames each on the current inputs, restores every
 * state buffer, and recaptures the graphs with the fastest shapes. */
int tfx_batch_autotune(tfx_batch batch, int frames);
/* Launch choices of a built batch (no counterpart in the reference; results are identical for every
 * value).  tfx_batch_autotune sets them too; setting one recaptures the frame graphs. */
typedef enum tfx_batch_option {
    TFX_BATCH_EXPANDED_GRIDS = 1,   /* collision lookups on a corner-expanded copy of an SDF (8 corners
                                       per cell): 0 never, 1 always, 2 (default) for the SDFs whose
                                       objects make at least 4 lookups per cell each frame          */
    TFX_BATCH_OVERLAP_SDF = 2,      /* 1 (default): the SDF build runs concurrently with the strand
                                       kernels, and each vertices-per-strand class (its strand and
                                       follow/collide kernels) is a concurrent branch of its own;
                                       0: one kernel after another                                   */
    TFX_BATCH_SDF_BLOCK = 3,        /* threads per block of the SDF construct: 64, 128 or 256         */
    TFX_BATCH_SPLIT_SWEEPS = 4,     /* 1: the local-shape sweeps run as their own launch (a thread per
                                       strand, up to four sweeps pipelined in registers) between two
                                       passes of the strand kernel; 0: inside the strand kernel      */
    TFX_BATCH_FOLLOW_FORM = 5,      /* the follow-hair + collision kernel of every class: 0 one vertex
                                       at a time per thread; 1 the vertices needing a lookup, then
                                       those within the margin, queued per warp and processed 32 at
                                       a time; 2 only the gradient stage queued.  Default per class:
                                       1 with follow hairs, else 2 at n >= 64, else 0 (get_option
                                       reports the first class's)                                   */
    TFX_BATCH_WAIT_POLLS = 6,       /* polls of the strand kernel's bounded wait for a group's bulk
                                       copies before its block gives up and the frame reports
                                       TFX_ERR_TIMEOUT (default 2^21; 0 gives up at once, for tests
                                       of that path).  Not a launch shape: the autotuner leaves it */
    TFX_BATCH_SDF_FORM = 7          /* the SDF construct: 0 (default) one warp per triangle, the
                                       reference's per-pair atomicMin; 1 triangles binned into
                                       8x8x4-cell tiles, one block per tile with the tile's words in
                                       shared memory, a warp per 4x4x2-cell brick walking its
                                       triangles nearest first, pairs skipped when an exact lower
                                       bound proves them farther than the cell's current value (grids
                                       of at most 1024 cells per axis).  Both give the same grid; the
                                       autotuner times both                                         */
} tfx_batch_option;
/* The positions of every hair object (in tfx_batch_add_hair order) as they stand after the frames
 * queued so far, copied into host memory: host_dst[i] receives num_vertices * 16 bytes (format
 * TFX_READBACK_XYZW: the float4 of the position buffer) or num_vertices * 12 bytes (TFX_READBACK_XYZ:
 * x, y, z packed; w is the inverse mass, which the simulation never changes).  Pinned memory copies
 * fastest.  The call queues a device snapshot on the context's stream and its copy to the host on a
 * separate copy stream, so the copy overlaps the next frames; it returns at once with a ticket.  The
 * destination must stay valid and untouched until tfx_batch_wait_readback(ticket) returns.  No
 * counterpart in the reference (its renderer reads the buffers on the GPU); this is how a host
 * consumer takes frames without stalling the simulation. */
#define TFX_READBACK_XYZW 0
#define TFX_READBACK_XYZ 1
int tfx_batch_readback(tfx_batch batch, void* const* host_dst, int count, int format, int64_t* ticket);
int tfx_batch_wait_readback(tfx_batch batch, int64_t ticket);
int tfx_batch_set_option(tfx_batch batch, int option, int value);
int tfx_batch_get_option(tfx_batch batch, int option, int* value);
/* Per-frame inputs (copied when tfx_batch_run is called): the constant block of hair object
 * `index` (TressFXSimulationParams, bone matrices [0, num_bones)), and its local-shape
 * re-dispatch count (m_CPULocalShapeIterations, TressFXHairObject.cpp:402-411). */
int tfx_batch_set_hair_constants(tfx_batch batch, int index, const tfx_sim_params* params, int num_bones,
                                 int cpu_local_iterations);
/* This frame's grid of SDF `index` (dimensions fixed at tfx_batch_add_sdf) and its collision margin
 * in world units (collisionMargin * cellSize). */
int tfx_batch_set_sdf_frame(tfx_batch batch, int index, const tfx_sdf_grid* grid, float margin_world);
/* This frame's bone matrices of the collision mesh of SDF `index`. */
int tfx_batch_set_mesh_bones(tfx_batch batch, int index, const float* bone_matrices, int num_bones);
/* Launches one frame on the context's stream (asynchronous).  Up to eight frames may be queued: the
 * call blocks only while the frame queued eight calls earlier is still running. */
int tfx_batch_run(tfx_batch batch);
/* Waits until every frame queued by tfx_batch_run has executed.  Returns TFX_ERR_TIMEOUT, once, if one
 * of them had a strand block give up its bounded wait (tfx_batch_run itself reports it when it next
 * reuses that frame's pinned block); that frame's state is then undefined and the caller restores it
 * (tfx_hair_write) or resets the objects.  No counterpart in the reference (D3D has no device-side
 * timeout); cudaStreamSynchronize on the context's stream plus the check. */
int tfx_batch_synchronize(tfx_batch batch);
/* The launch shapes in use, as text, and the number of kernels one frame launches. */
int tfx_batch_describe(tfx_batch batch, char* buf, size_t len, int32_t* launches_per_frame);
/* Runs one frame like tfx_batch_run but with direct launches and CUDA events between its parts;
 * waits for it and returns the milliseconds of each part: [0] = mesh skinning + SDF rebuild,
 * [1..] = the fused strand launch of each vertices-per-strand class present (ascending n), then the
 * follow/collide launch of each class, then (when some hair object collides with further SDFs,
 * tfx_batch_add_hair_collision) those collisions. */
int tfx_batch_profile_frame(tfx_batch batch, float* part_ms, int max_parts, int* num_parts);

/* ---------------------------------------------------------------------------------- learned collision proxy */
/* No counterpart in the reference.  A pose-conditioned neural SDF: an MLP (xyz with 16 Fourier
 * frequencies + 3 pose angles -> 4 x 64 SiLU -> 1, BF16 weights, FP32 accumulation, tensor cores) that
 * predicts the grid SDF's distance (in cells, truncated to +-band) and is trained on samples of grid
 * SDFs built by this library at sampled poses.  At collision time it replaces the grid for vertices
 * it places farther than margin + contact_slack_cells from the surface; the others (the contact band) are
 * collided exactly on the grid, built only on the cells their lookups read. */
typedef struct tfx_nsdf_t* tfx_nsdf;
typedef struct tfx_nsdf_desc {
    float box_min[3], box_max[3];   /* input normalisation box (world)                              */
    float cell_size;                /* distance unit: grid cell (world)                              */
    float band_cells;               /* targets truncated to +-band_cells                             */
    float pose_scale;               /* network input = pose angle (radians) * pose_scale             */
    float sphere_center[3];         /* sphere around the mesh: unset grid points outside it are far  */
    float sphere_radius;
    uint32_t seed;
    int64_t max_samples;            /* training pool capacity                                        */
    int64_t max_eval_samples;       /* evaluation pool capacity                                      */
    float contact_slack_cells;      /* band = network distance below margin + slack cells (0: 1)      */
} tfx_nsdf_desc;
int tfx_nsdf_create(tfx_context ctx, const tfx_nsdf_desc* desc, tfx_nsdf* out);
int tfx_nsdf_destroy(tfx_nsdf nsdf);
/* One pose of training (pool 0) or evaluation (pool 1) data: skins `mesh` with the bone matrices,
 * rebuilds `sdf` on `grid` from it, and appends `count` samples labelled by that grid (75% near the
 * surface with normal offsets of sigma_cells cells, 25% uniform in the grid box).  sphere = centre xyz
 * and radius of a sphere around the posed mesh (NULL: the descriptor's): grid points left unset that
 * lie outside it are labelled far (+band), those inside it are left out. */
int tfx_nsdf_add_samples(tfx_nsdf nsdf, int pool, tfx_mesh mesh, tfx_sdf sdf, const tfx_sdf_grid* grid,
                         const float* bone_matrices, int num_bones, const float pose[3], const float sphere[4],
                         int count, float sigma_cells);
/* `steps` Adam steps on minibatches of `batch` (a multiple of 512) samples of pool 0, the learning
 * rate decaying from learning_rate to a tenth of it along a cosine; *mean_loss = mean squared error
 * (cells^2) over the last tenth of the steps. */
int tfx_nsdf_train(tfx_nsdf nsdf, int steps, int batch, float learning_rate, float* mean_loss);
/* Network output (cells), target (cells) and weight of every sample of a pool, to host arrays. */
int tfx_nsdf_evaluate(tfx_nsdf nsdf, int pool, float* pred_cells, float* target_cells, float* weight,
                      int64_t max_count, int64_t* count);
/* Distances (world units) at `count` DEVICE points (float4, xyz used) under `pose`. */
int tfx_nsdf_query(tfx_nsdf nsdf, const void* points, int count, const float pose[3], float* out);
/* CollideHairVerticesWithSdf_forward for every vertex of `hair` with the proxy in front of the grid:
 * the band vertices are collided on `sdf` (mesh already bound and skinned for this frame), built on
 * `grid` at their cells only.  A pose outside the range of the training poses (pool 0) takes the
 * grid path for every vertex: the whole grid is built (tfx_sdf_update) and collided
 * (tfx_sdf_collide), and band_count reports every vertex.  band_count (optional, host) receives the
 * band size and synchronizes. */
int tfx_nsdf_collide(tfx_nsdf nsdf, tfx_hair hair, tfx_sdf sdf, const tfx_sdf_grid* grid, float margin_world,
                     const float pose[3], int32_t* band_count);
/* Master FP32 parameters (tfx_nsdf_get_info's num_params floats), e.g. to save or load a network. */
int tfx_nsdf_get_params(tfx_nsdf nsdf, float* params, size_t count);
int tfx_nsdf_set_params(tfx_nsdf nsdf, const float* params, size_t count);
/* The network's forward pass for queries, evaluation and collision (no reference counterpart):
 * 1 (default) on the fifth-generation tensor cores (tcgen05.mma, accumulators in tensor memory,
 * 128 points per tile); 0 with mma.sync (the form the training kernels use).  Both compute the same
 * network in bf16 with fp32 accumulation; their outputs differ in the last bits (accumulation order,
 * bias precision).  A bounded tensor-core wait that gives up is reported as TFX_ERR_TIMEOUT by the next
 * tfx_nsdf_evaluate, or tfx_nsdf_collide with band_count. */
int tfx_nsdf_set_inference(tfx_nsdf nsdf, int form);
/* Replaces pool `pool`'s samples with the caller's: count records of 8 floats (world x, y, z, target
 * distance in cells, the 3 pose angles, weight), e.g. distances from an offline SDF.  Pool 0 also
 * resets the pose range the collision trusts the network on to the samples' poses.  No counterpart
 * in the reference. */
int tfx_nsdf_set_samples(tfx_nsdf nsdf, int pool, const float* samples, int64_t count);
/* The gradient of the loss with respect to the master parameters from the last training step
 * (tfx_nsdf_get_info's num_params floats, parameter layout).  No counterpart in the reference. */
int tfx_nsdf_get_gradients(tfx_nsdf nsdf, float* grads, size_t count);
int tfx_nsdf_get_info(tfx_nsdf nsdf, int32_t* num_params, int64_t* train_samples, int64_t* eval_samples,
                      int32_t* steps);

#ifdef __cplusplus
}
#endif

#endif /* TRESSFX_GB300_H_ */
