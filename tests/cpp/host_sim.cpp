// Runs frames of hair simulation with SDF collision through the C++ host classes of
// libtressfx_host (TressFXAsset, TressFXHairObject, TressFXSimulation, TressFXBoneSkinning,
// TressFXSDFCollision) and dumps the asset, the per-frame inputs and the final state.
//
//   host_sim <in.tfx> <in.tfxbone> <in.tfxmesh> <followHairs> <frames> <out.bin>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "tressfx/TressFXBoneSkinning.h"
#include "tressfx/TressFXSDFCollision.h"
#include "tressfx/TressFXSDFMarchingCubes.h"
#include "tressfx/TressFXSimulation.h"

namespace {
struct IdentityScene : EI_Scene {
    int GetBoneIdByName(int, const char* name) override { return (name && name[0] == 'b') ? std::atoi(name + 1) : 0; }
};
FILE* g_out = nullptr;
void put(const char* name, const void* data, size_t bytes) {
    const uint32_t nl = (uint32_t)std::strlen(name);
    const unsigned long long nb = bytes;
    std::fwrite(&nl, 4, 1, g_out);
    std::fwrite(name, 1, nl, g_out);
    std::fwrite(&nb, 8, 1, g_out);
    if (bytes) std::fwrite(data, 1, bytes, g_out);
}
template <class T> void put(const char* name, const std::vector<T>& v) { put(name, v.data(), v.size() * sizeof(T)); }

// Row-vector rotation about y (bone 1) / x (bone 2) around the origin.
AMD::float4x4 rot(int axis, float a) {
    AMD::float4x4 m{{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1}};
    const float c = std::cos(a), s = std::sin(a);
    if (axis == 1) { m.m[0] = c; m.m[2] = -s; m.m[8] = s; m.m[10] = c; }
    else { m.m[5] = c; m.m[6] = s; m.m[9] = -s; m.m[10] = c; }
    return m;
}
}  // namespace

int main(int argc, char** argv) {
    if (argc != 7) { std::fprintf(stderr, "usage: %s tfx tfxbone tfxmesh F frames out\n", argv[0]); return 2; }
    try {
        IdentityScene scene;
        TressFXAsset asset;
        asset.SetRandomSeed(7);
        FILE* f = std::fopen(argv[1], "rb");
        if (!f || !asset.LoadHairData(f)) return 3;
        std::fclose(f);
        asset.GenerateFollowHairs(std::atoi(argv[4]), 0.5f, 0.002f);
        asset.ProcessAsset();
        FILE* b = std::fopen(argv[2], "rb");
        if (!b || !asset.LoadBoneData(b, 0, &scene)) return 4;
        std::fclose(b);

        EI_Device device(0);
        EI_CommandContext cc(device);
        TressFXSimulation sim;
        sim.Initialize(&device);
        TressFXSDFCollisionSystem sdfSystem;
        sdfSystem.Initialize(&device);
        TressFXHairObject hair(&asset, &device, cc, "hair", 0);
        TressFXBoneSkinning mesh;
        if (!mesh.LoadTressFXCollisionMeshData(&scene, argv[3], 0, "b0")) return 5;
        mesh.Initialize(&device, cc, "mesh");
        TressFXSDFCollision sdf(&device, &mesh, "mesh", 40, 1.5f);

        TressFXSimulationSettings s;
        s.m_gravityMagnitude = 9.8f;
        s.m_damping = 0.035f;
        s.m_globalConstraintStiffness = 0.2f;
        s.m_globalConstraintsRange = 0.3f;
        s.m_localConstraintStiffness = 0.8f;
        s.m_localConstraintsIterations = 3;
        s.m_lengthConstraintsIterations = 3;
        s.m_tipSeparation = 0.5f;
        s.m_windMagnitude = 2.0f;

        g_out = std::fopen(argv[6], "wb");
        if (!g_out) return 6;
        put("positions", asset.m_positions);
        put("tangents", asset.m_tangents);
        put("rest_lengths", asset.m_restLengths);
        put("follow_root_offsets", asset.m_followRootOffsets);
        put("bone_skinning", asset.m_boneSkinningData);
        const int counts[3] = {asset.m_numGuideStrands, asset.m_numVerticesPerStrand, asset.m_numFollowStrandsPerGuide};
        put("counts", counts, sizeof(counts));
        const int nsdf[4] = {0, 0, 0, sdf.GetGridNumTotalCells()};
        put("sdf_alloc", nsdf, sizeof(nsdf));

        std::vector<TressFXHairObject*> objects{&hair};
        const int frames = std::atoi(argv[5]);
        std::vector<float> bonesAll, grids, lsIters;
        for (int fr = 0; fr < frames; ++fr) {
            const AMD::float4x4 bones[3] = {rot(1, 0.0f), rot(1, 0.6f * std::sin(0.3f * fr)), rot(2, 0.4f * std::sin(0.2f * fr))};
            for (auto& m : bones) bonesAll.insert(bonesAll.end(), m.m, m.m + 16);
            hair.UpdateBoneMatrices(bones, 3);
            hair.UpdateSimulationParameters(&s, 1.0f / 60.0f);
            lsIters.push_back((float)hair.GetCPULocalShapeIterations());
            mesh.Update(cc, bones, 3);
            sdf.Update(cc, sdfSystem);
            sim.Simulate(cc, objects);
            sdf.CollideWithHair(cc, sdfSystem, hair);
            const tfx_sdf_grid g = sdf.GetGrid();
            grids.insert(grids.end(), {g.origin[0], g.origin[1], g.origin[2], g.cell_size, (float)g.num_cells_x,
                                       (float)g.num_cells_y, (float)g.num_cells_z, sdf.GetSDFCollisionMargin()});
        }
        device.WaitForCompute();
        put("bones", bonesAll);
        put("grids", grids);
        put("ls_iters", lsIters);
        const int bufs[5] = {TFX_BUF_POSITIONS, TFX_BUF_POSITIONS_PREV, TFX_BUF_POSITIONS_PREV_PREV, TFX_BUF_TANGENTS,
                             TFX_BUF_STRAND_LEVEL_DATA};
        const char* names[5] = {"out_pos", "out_prev", "out_prevprev", "out_tan", "out_sld"};
        for (int k = 0; k < 5; ++k) {
            void* p = nullptr;
            size_t bytes = 0;
            if (tfx_hair_get_buffer(hair.GetHandle(), bufs[k], &p, &bytes) != TFX_OK) return 7;
            std::vector<char> host(bytes);
            if (tfx_hair_read(hair.GetHandle(), bufs[k], host.data(), bytes) != TFX_OK) return 8;
            put(names[k], host.data(), bytes);
        }
        std::vector<char> grid((size_t)sdf.GetGridNumTotalCells() * 4);
        if (tfx_sdf_read(sdf.GetHandle(), grid.data(), grid.size()) != TFX_OK) return 9;
        put("out_sdf", grid.data(), grid.size());
        // the iso-surface of the last frame's grid at the collision margin (src/SDF.cpp:63)
        TressFXSDFMarchingCubes mc(1 << 17);
        mc.Initialize("mesh", &device);
        mc.SetSDF(&sdf);
        mc.SetSDFIsoLevel(sdf.GetSDFCollisionMargin());
        mc.Update(cc);
        std::vector<float> mcv;
        const int mcCount = mc.ReadVertices(mcv);
        put("mc_count", &mcCount, sizeof(int));
        put("mc_vertices", mcv.data(), mcv.size() * sizeof(float));
        const auto stamps = device.GetTimeStamps();
        std::string names_joined;
        for (auto& st : stamps) names_joined += st.first + "\n";
        put("stamps", names_joined.data(), names_joined.size());
        std::fclose(g_out);
    } catch (const TressFXError& e) {
        std::fprintf(stderr, "TressFXError %d: %s\n", e.status(), e.what());
        return 10;
    }
    return 0;
}
