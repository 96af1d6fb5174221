// TressFXAsset (src/TressFX/TressFXAsset.h:48-107): hair data from a .tfx file, optional procedural
// follow hairs, the derived simulation data, and bone skinning from a .tfxbone file.  Same members
// and the same loading / processing rules (including the padding of the guide-strand count to the
// next multiple of 64 above the file's count, TressFXAsset.cpp:111).
#pragma once

#include <cstdio>
#include <vector>

#include "EngineInterface.h"
#include "TressFXCommon.h"

struct TressFXBoneSkinningData {
    float boneIndex[TRESSFX_MAX_INFLUENTIAL_BONE_COUNT];
    float weight[TRESSFX_MAX_INFLUENTIAL_BONE_COUNT];
};

// .tfx header (src/TressFX/TressFXFileFormat.h:35-54): offsets are bytes from the file start.
struct TressFXTFXFileHeader {
    float version;
    unsigned int numHairStrands;
    unsigned int numVerticesPerStrand;
    unsigned int offsetVertexPosition;   // float4[numHairStrands * numVerticesPerStrand]
    unsigned int offsetStrandUV;         // float2[numHairStrands]
    unsigned int offsetVertexUV;
    unsigned int offsetStrandThickness;
    unsigned int offsetVertexColor;
    unsigned int reserved[32];
};

class TressFXAsset {
public:
    TressFXAsset();
    ~TressFXAsset();

    // hair data from *.tfx
    std::vector<Vector3> m_positions;
    std::vector<AMD::float2> m_strandUV;
    std::vector<AMD::float4> m_tangents;
    std::vector<Vector3> m_followRootOffsets;
    std::vector<AMD::int32> m_strandTypes;
    std::vector<AMD::real32> m_thicknessCoeffs;
    std::vector<AMD::real32> m_restLengths;
    std::vector<AMD::int32> m_triangleIndices;

    // bone skinning data from *.tfxbone
    std::vector<TressFXBoneSkinningData> m_boneSkinningData;

    AMD::int32 m_numTotalStrands;
    AMD::int32 m_numTotalVertices;
    AMD::int32 m_numVerticesPerStrand;
    AMD::int32 m_numGuideStrands;
    AMD::int32 m_numGuideVertices;
    AMD::int32 m_numFollowStrandsPerGuide;

    // Loads *.tfx hair data (TressFXAsset.cpp:94-169).  Returns false on a version older than 4, an
    // unsupported vertices-per-strand count or a short read.
    bool LoadHairData(FILE* ioObject);

    // Generates follow hairs around each guide (TressFXAsset.cpp:173-245): random root offsets
    // within maxRadiusAroundGuideHair in the plane normal to the guide's first segment.
    bool GenerateFollowHairs(int numFollowHairsPerGuideHair = 0, float tipSeparationFactor = 0,
                             float maxRadiusAroundGuideHair = 0);

    // Tangents, thickness coefficients, rest lengths, triangle indices, strand types
    // (TressFXAsset.cpp:247-399).
    bool ProcessAsset();

    // Loads *.tfxbone data (TressFXAsset.cpp:401-480); bone names are mapped through the scene.
    bool LoadBoneData(FILE* ioObject, int skinNumber, EI_Scene* scene);

    AMD::uint32 GetNumHairSegments() { return m_numTotalStrands * (m_numVerticesPerStrand - 1); }
    AMD::uint32 GetNumHairTriangleIndices() { return 6 * GetNumHairSegments(); }
    AMD::uint32 GetNumHairLineIndices() { return 2 * GetNumHairSegments(); }

    // Source of the uniform [0, 1] numbers GenerateFollowHairs draws (the reference calls
    // rand() / RAND_MAX).  The default is a seeded xorshift64* generator.
    typedef float (*RandomSource)(void* user);
    void SetRandomSource(RandomSource fn, void* user) { m_random = fn; m_randomUser = user; }
    void SetRandomSeed(uint64_t seed) { m_seed = seed ? seed : 0x9E3779B97F4A7C15ull; }

private:
    void ComputeThicknessCoeffs();
    void ComputeStrandTangent();
    void ComputeRestLengths();
    void FillTriangleIndexArray();
    float GetRandom(float mn, float mx);

    RandomSource m_random = nullptr;
    void* m_randomUser = nullptr;
    uint64_t m_seed = 0x9E3779B97F4A7C15ull;
};
