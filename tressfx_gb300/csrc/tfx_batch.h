// Structures of the batched path shared by its kernels (tfx_batch_kernels.cu) and its host side
// (tfx_batch_capi.cu).
#pragma once
#include <algorithm>

#include "tfx_internal.h"

namespace tfx {

// Per-frame grid of one SDF (origin moves with the follow bone) and the collision margin in world
// units (collisionMargin * cellSize, TressFXSDFCollision.cpp:194).
struct SdfFrame {
    SdfGrid grid;
    float margin;
    float pad[3];
};

struct BatchObject {
    HairView hair;                 // state buffers and counts of the hair object
    const DevSimConsts* consts;    // this frame's constants (inside the device frame block)
    const float* sdf;              // decoded SDF grid of the object's collision mesh, or null
    const float4* sdf8;            // its corner-expanded copy (8 corners per cell), or null
    const SdfFrame* sdfFrame;      // this frame's grid + margin (inside the device frame block)
};

// One (hair object, SDF) pair of a collision level: level k holds every object's k-th SDF after its
// first (tfx_batch_add_hair_collision), so a level's pairs touch distinct objects and run in one launch.
struct BatchCollide {
    int obj;                  // index into the object table
    int sdf;                  // index into the SDF table
    long long firstVertex;    // prefix over the level's pairs of their objects' vertices
};

// A group of guide strands of one object (at most fused_group_size(n)): one block of the fused
// kernel at a time.
struct WorkItem {
    int obj;         // index into the object table
    int firstGuide;  // first guide strand of the group
    int count;       // guide strands in the group
    int pad;
};

struct BatchMesh {
    const float4* bind;     // {position, normal}[V]
    float4* skinned;        // {position, normal}[V]
    const float4* skin;     // {boneIndex, boneWeight}[V]
    const float4* bones;    // this frame's bone matrices (inside the device frame block)
    int firstVertex;        // prefix over meshes
    int numVertices;
    int pad[2];
};

struct BatchSdf {
    const float4* mesh;       // skinned {position, normal}[V]
    const uint32_t* indices;  // uint32[3T]
    uint32_t* words;          // the grid: FloatFlip3 words while built, floats after
    float4* expanded;         // corner-expanded copy, 2 float4 per cell, or null when not kept
    const SdfFrame* frame;    // grid of this frame
    long long firstQuad;      // prefix over SDFs of ceil(cells / 4)
    long long numCells;       // X*Y*Z
    int firstTriangle;        // prefix over SDFs
    int numTriangles;
    int firstTile;            // prefix over SDFs of the 8x8x4-cell tiles (tiled construct)
    int tilesX, tilesY, tilesZ;
};

// Polls of k_fused_strands' bounded wait for a group's bulk copies before the block gives up.
constexpr int kFusedWaitPollsDefault = 1 << 21;

struct FusedLaunch {
    int n, vpl, warpsPerBlock, blocks;
    const BatchObject* objs;
    const WorkItem* items;
    int numItems;
    int* err;        // set to 1 when a block gives up waiting for its bulk copies
    int mode;        // 0 the whole frame, 1 up to the local-shape sweeps, 2 after them
    int waitPolls;   // limit of the first wait (kFusedWaitPollsDefault; 0 in tests of the timeout path)
};

struct FollowLaunch {
    int n, blocks;
    const BatchObject* objs;
    const WorkItem* items;
    int numItems;
    int chunks;      // chunks per work item (1 .. follow_max_chunks_per_item(n))
    int queued;      // 0 k_follow_collide; 1 k_follow_collide_queued (both stages queued); 2 (gradient stage queued)
    int noFollow;    // every object of the class has no follow hairs: the kernels specialised for F = 0
};

struct SdfBatchLaunch {
    const BatchSdf* sdfs;
    int nsdf;
    int totalTris;
    long long totalQuads;
    int constructThreads;
    int expand;      // some SDF keeps a corner-expanded copy: run the expansion
    // the SDFs that keep one, so that the expansion runs over their cells only: their indices into
    // `sdfs`, the prefix of their cell counts (nexp + 1 entries), and the sum
    const int* expSdf;
    const long long* expFirst;
    int nexp;
    long long expCells;
};

// The tiled SDF build (tfx_sdf_tiles.cu): triangles binned into 8x8x4-cell tiles, one block per tile
// with the tile's words in shared memory, pairs culled by an exact lower bound.  A triangle whose cell
// box spans more than SDF_BIG_TILES tiles goes to its SDF's big list, which every tile of the SDF scans,
// so a tile list never holds more than SDF_BIG_TILES entries per triangle.
constexpr int SDF_BIG_TILES = 16;
constexpr int SDF_TILE_X = 8, SDF_TILE_Y = 8, SDF_TILE_Z = 4;
constexpr int SDF_TRI_RECORD = 20;       // floats of a triangle's record (vertices, bound terms, cell box)
constexpr int SDF_TILE_MAX_DIM = 1024;   // grid dimensions the packed cell boxes can hold

struct SdfTileLaunch {
    const BatchSdf* sdfs;
    int nsdf, totalTris, totalTiles, blocks;
    int* tileCount;      // [totalTiles], then bigCount [nsdf] and workCounter [1]: zeroed by one memset
    int* bigCount;
    int* workCounter;
    size_t zeroBytes;
    int* tileStart;      // [totalTiles]: exclusive prefix within its block of 1024 tiles
    int* blockSum;       // [ceil(totalTiles / 1024)]: exclusive prefix of the block totals
    int* list;           // [listCapacity]: triangle indices, tile by tile
    long long listCapacity;
    int* bigList;        // [totalTris]: SDF i's big triangles from its firstTriangle on
    float* records;      // [totalTris * SDF_TRI_RECORD]: each triangle's record, written by the binning
};
cudaError_t launch_sdf_tiles(const SdfTileLaunch& L, cudaStream_t s);
int sdf_tile_blocks_per_sm();
// k_batch_sdf_expand alone (after the tiled build)
cudaError_t launch_batch_sdf_expand(const SdfBatchLaunch& L, cudaStream_t s);

cudaError_t launch_fused_strands(const FusedLaunch& fl, cudaStream_t s);
// k_local_sweep over the groups of fl (mode 1 has run on them, mode 2 runs after)
cudaError_t launch_local_sweep(const FusedLaunch& fl, cudaStream_t s);
cudaError_t launch_follow_collide(const FollowLaunch& fl, cudaStream_t s);
// CollideHairVerticesWithSdf_forward of one collision level's pairs
cudaError_t launch_collide_level(const BatchObject* objs, const BatchSdf* sdfs, const BatchCollide* pairs, int npairs,
                                 long long totalVertices, cudaStream_t s);
cudaError_t launch_batch_mesh_skin(const BatchMesh* meshes, int nmeshes, int totalVerts, cudaStream_t s);
cudaError_t launch_batch_sdf(const SdfBatchLaunch& l, cudaStream_t s);
// Every object's positions, consecutively (first[i] = object i's first vertex), into `out` as float4 or packed xyz.
cudaError_t launch_snapshot_positions(const BatchObject* objs, const long long* first, int nobj, long long total,
                                      float* out, int xyzOnly, cudaStream_t s);
bool fused_config_valid(int n, int vpl);
int fused_smem_bytes(int n, int vpl, int warps);
int fused_blocks_per_sm(int n, int vpl, int warps);
int fused_group_size(int n);
int follow_max_chunks_per_item(int n);   // 256-vertex chunks a work item can be cut into
int follow_blocks_per_sm(int n, int mode, bool noFollow);   // mode: FollowLaunch::queued

}  // namespace tfx
