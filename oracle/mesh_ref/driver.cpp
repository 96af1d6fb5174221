// Test infrastructure: the reference's own .tfxmesh parser (SuStringTokenizer and
// TressFXBoneSkinning::LoadTressFXCollisionMeshData, cut unchanged out of
// src/TressFX/TressFXBoneSkinning.cpp into bone_skinning_load.inc by build.py) compiled in a stand-in
// class with the members it fills, and what it loads dumped in tests/cpp/mesh_dump.cpp's layout.
//
//   tfx_mesh_ref <in.tfxmesh> <followBone> <out.bin>
//
// Bone names map to engine ids as in the asset drivers: "b<k>" -> k, any other name -> 0.
#include <cassert>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "EngineInterface.h"
#include "TressFXAsset.h"

class TressFXBoneSkinning {
public:
    bool LoadTressFXCollisionMeshData(EI_Scene* scene, const char* filePath, int skinNumber, const char* followBone);

    EI_Scene* m_pScene = nullptr;
    std::vector<AMD::float3> m_pTempVertices;
    std::vector<AMD::float3> m_pTempNormals;
    std::vector<int> m_pTempIndices;
    std::vector<TressFXBoneSkinningData> boneSkinningData;
    AMD::uint32 m_NumVertices = 0;
    AMD::uint32 m_NumTriangles = 0;
    int m_skinNumber = 0;
    int m_followBone = 0;
};

#include "bone_skinning_load.inc"

namespace {
struct IdentityScene : EI_Scene {
    int GetBoneIdByName(int, const char* name) override { return (name && name[0] == 'b') ? std::atoi(name + 1) : 0; }
};
template <class T> void put(FILE* f, const std::vector<T>& v) {
    const unsigned long long n = v.size() * sizeof(T);
    std::fwrite(&n, sizeof(n), 1, f);
    if (n) std::fwrite(v.data(), 1, n, f);
}
}  // namespace

int main(int argc, char** argv) {
    if (argc != 4) { std::fprintf(stderr, "usage: %s mesh.tfxmesh followBone out\n", argv[0]); return 2; }
    IdentityScene scene;
    TressFXBoneSkinning m;
    if (!m.LoadTressFXCollisionMeshData(&scene, argv[1], 0, argv[2])) { std::fprintf(stderr, "load failed\n"); return 3; }
    // {pos.xyz, 0, normal.xyz, 0} and {boneIndex[4], weight[4]} per vertex, uint32 indices
    std::vector<float> verts((size_t)m.m_NumVertices * 8, 0.0f), skin((size_t)m.m_NumVertices * 8, 0.0f);
    for (size_t v = 0; v < m.m_NumVertices; ++v) {
        verts[8 * v + 0] = m.m_pTempVertices[v].x; verts[8 * v + 1] = m.m_pTempVertices[v].y;
        verts[8 * v + 2] = m.m_pTempVertices[v].z;
        verts[8 * v + 4] = m.m_pTempNormals[v].x; verts[8 * v + 5] = m.m_pTempNormals[v].y;
        verts[8 * v + 6] = m.m_pTempNormals[v].z;
        for (int k = 0; k < 4; ++k) {
            skin[8 * v + k] = m.boneSkinningData[v].boneIndex[k];
            skin[8 * v + 4 + k] = m.boneSkinningData[v].weight[k];
        }
    }
    std::vector<unsigned> idx(m.m_pTempIndices.begin(), m.m_pTempIndices.end());
    FILE* o = std::fopen(argv[3], "wb");
    if (!o) return 5;
    const int counts[3] = {(int)m.m_NumVertices, (int)m.m_NumTriangles, m.m_followBone};
    std::fwrite(counts, sizeof(counts), 1, o);
    put(o, verts); put(o, idx); put(o, skin);
    std::fclose(o);
    return 0;
}
