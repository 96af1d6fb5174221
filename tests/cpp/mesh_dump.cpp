// Drives libtressfx_host's TressFXBoneSkinning::LoadTressFXCollisionMeshData over a .tfxmesh file and
// dumps what it loaded, in the layout of oracle/mesh_ref/driver.cpp (the reference's own parser), so
// the two dumps can be compared.
//
//   mesh_dump <in.tfxmesh> <followBone> <out.bin>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "tressfx/TressFXBoneSkinning.h"

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
    FILE* o = std::fopen(argv[3], "wb");
    if (!o) return 5;
    const int counts[3] = {m.GetNumMeshVertices(), m.GetNumMeshTriangle(), m.GetFollowBone()};
    std::fwrite(counts, sizeof(counts), 1, o);
    put(o, m.GetBindPose()); put(o, m.GetIndices()); put(o, m.GetSkinning());
    std::fclose(o);
    return 0;
}
