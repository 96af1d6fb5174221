// TressFXBoneSkinning (src/TressFX/TressFXBoneSkinning.h:50-125): a collision mesh loaded from a
// .tfxmesh file and skinned on the device every frame, presented to the SDF through
// TressFXSDFInputMeshInterface.  Rendering of the mesh (DrawMesh) is not part of this library.
#pragma once

#include <string>
#include <vector>

#include "EngineInterface.h"
#include "TressFXAsset.h"
#include "TressFXSDFInputMeshInterface.h"

class TressFXBoneSkinning : public TressFXSDFInputMeshInterface {
public:
    TressFXBoneSkinning() = default;
    ~TressFXBoneSkinning() override;

    // Parses a .tfxmesh text file (TressFXBoneSkinning.cpp:100-285): bone names, then per vertex
    // "index px py pz nx ny nz b0 b1 b2 b3 w0 w1 w2 w3", then per triangle "index i0 i1 i2"; lines
    // starting with '#' are comments.  Bone names map to engine ids through the scene.
    bool LoadTressFXCollisionMeshData(EI_Scene* scene, const char* filePath, int skinNumber, const char* followBone);
    // The same data given directly (bind-pose {float4 position, float4 normal}[numVertices], uint32
    // indices, {float4 boneIndex, float4 weight}[numVertices]).
    void SetMeshData(const float* vertices, int numVertices, const uint32_t* indices, int numTriangles,
                     const float* boneSkinning, int followBone);

    // Uploads the mesh (TressFXBoneSkinning.cpp:287-404) and computes the bounding box: centre =
    // mean vertex, radius = largest distance from it.
    void Initialize(EI_Device* pDevice, EI_CommandContext& commandContext, const char* name);

    // Skins the mesh with the given bone matrices (row-major, row-vector convention); the follow
    // bone's matrix also moves the bounding box.
    void Update(EI_CommandContext& commandContext, const AMD::float4x4* boneMatrices, int numBones);

    // TressFXSDFInputMeshInterface
    EI_Resource& GetMeshBuffer() override { return m_skinned; }
    EI_Resource& GetTrimeshVertexIndicesBuffer() override { return m_indices; }
    int GetNumMeshVertices() override { return m_NumVertices; }
    int GetNumMeshTriangle() override { return m_NumTriangles; }
    size_t GetSizeOfMeshElement() override { return 4 * sizeof(float) + 4 * sizeof(float); }
    void GetBoundingBox(Vector3& min, Vector3& max) override;
    void GetInitialBoundingBox(Vector3& min, Vector3& max) override { min = m_bbMin; max = m_bbMax; }

    tfx_mesh GetHandle() const { return m_mesh; }
    int GetFollowBone() const { return m_followBone; }
    // The mesh as loaded (host copies): {pos.xyz, 0, normal.xyz, 0} per vertex, uint32 triangle
    // indices, and {boneIndex[4], weight[4]} per vertex with bones as engine ids.
    const std::vector<float>& GetBindPose() const { return m_vertices; }
    const std::vector<uint32_t>& GetIndices() const { return m_tempIndices; }
    const std::vector<float>& GetSkinning() const { return m_skinning; }

private:
    std::vector<float> m_vertices;     // {pos.xyz, 0, normal.xyz, 0} per vertex
    std::vector<uint32_t> m_tempIndices;
    std::vector<float> m_skinning;     // {boneIndex[4], weight[4]} per vertex
    int m_NumVertices = 0, m_NumTriangles = 0;
    int m_followBone = 0;
    Vector3 m_bbMin, m_bbMax;
    AMD::float4x4 m_followMatrix{{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1}};
    tfx_mesh m_mesh = nullptr;
    EI_Resource m_skinned, m_indices;
};
