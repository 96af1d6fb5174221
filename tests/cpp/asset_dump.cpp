// Drives libtressfx_host's TressFXAsset over a .tfx / .tfxbone pair and dumps every array it
// produces, in the layout of oracle/asset_ref/asset_ref_driver.cpp (the reference's own
// TressFXAsset), so the two dumps can be compared.
//
//   asset_dump <in.tfx> <in.tfxbone|-> <followHairs> <tipSeparation> <radius> <seed> <out.bin>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "tressfx/TressFXAsset.h"

namespace {
struct IdentityScene : EI_Scene {
    int GetBoneIdByName(int, const char* name) override { return (name && name[0] == 'b') ? std::atoi(name + 1) : 0; }
};
float rand01(void*) { return float(std::rand()) / float(RAND_MAX); }
template <class T> void put(FILE* f, const std::vector<T>& v) {
    const unsigned long long n = v.size() * sizeof(T);
    std::fwrite(&n, sizeof(n), 1, f);
    if (n) std::fwrite(v.data(), 1, n, f);
}
}  // namespace

int main(int argc, char** argv) {
    if (argc != 8) { std::fprintf(stderr, "usage: %s tfx tfxbone|- F tip radius seed out\n", argv[0]); return 2; }
    TressFXAsset a;
    a.SetRandomSource(rand01, nullptr);
    FILE* f = std::fopen(argv[1], "rb");
    if (!f || !a.LoadHairData(f)) { std::fprintf(stderr, "LoadHairData failed\n"); return 3; }
    std::fclose(f);
    std::srand((unsigned)std::atoi(argv[6]));
    a.GenerateFollowHairs(std::atoi(argv[3]), (float)std::atof(argv[4]), (float)std::atof(argv[5]));
    a.ProcessAsset();
    if (std::strcmp(argv[2], "-") != 0) {
        IdentityScene scene;
        FILE* b = std::fopen(argv[2], "rb");
        if (!b || !a.LoadBoneData(b, 0, &scene)) { std::fprintf(stderr, "LoadBoneData failed\n"); return 4; }
        std::fclose(b);
    }
    FILE* o = std::fopen(argv[7], "wb");
    if (!o) return 5;
    const int counts[6] = {a.m_numTotalStrands, a.m_numTotalVertices, a.m_numVerticesPerStrand, a.m_numGuideStrands,
                           a.m_numGuideVertices, a.m_numFollowStrandsPerGuide};
    std::fwrite(counts, sizeof(counts), 1, o);
    put(o, a.m_positions); put(o, a.m_strandUV); put(o, a.m_tangents); put(o, a.m_followRootOffsets);
    put(o, a.m_strandTypes); put(o, a.m_thicknessCoeffs); put(o, a.m_restLengths); put(o, a.m_triangleIndices);
    put(o, a.m_boneSkinningData);
    std::fclose(o);
    return 0;
}
