// TressFXAsset: .tfx / .tfxbone loading, procedural follow hairs and the derived simulation data,
// following src/TressFX/TressFXAsset.cpp step for step (same arithmetic on the same types).
#include <algorithm>
#include <cstring>
#include <string>

#include "tressfx/TressFXAsset.h"

namespace {

// GetTangentVectors (TressFXAsset.cpp:35-62): two unit vectors orthogonal to the unit vector n.
void tangent_vectors(const Vector3& n, Vector3& t0, Vector3& t1) {
    if (fabsf(n[2]) > 0.707f) {
        const float a = n[1] * n[1] + n[2] * n[2];
        const float k = 1.0f / sqrtf(a);
        t0[0] = 0;
        t0[1] = -n[2] * k;
        t0[2] = n[1] * k;
        t1[0] = a * k;
        t1[1] = -n[0] * t0[2];
        t1[2] = n[0] * t0[1];
    } else {
        const float a = n[0] * n[0] + n[1] * n[1];
        const float k = 1.0f / sqrtf(a);
        t0[0] = -n[1] * k;
        t0[1] = n[0] * k;
        t0[2] = 0;
        t1[0] = -n[2] * t0[1];
        t1[1] = n[2] * t0[0];
        t1[2] = a * k;
    }
}

bool read_exact(void* dst, size_t bytes, FILE* f) { return EI_Read(dst, bytes, f) == bytes; }

}  // namespace

TressFXAsset::TressFXAsset()
    : m_numTotalStrands(0), m_numTotalVertices(0), m_numVerticesPerStrand(0), m_numGuideStrands(0),
      m_numGuideVertices(0), m_numFollowStrandsPerGuide(0) {}

TressFXAsset::~TressFXAsset() {}

float TressFXAsset::GetRandom(float mn, float mx) {
    float u;
    if (m_random) {
        u = m_random(m_randomUser);
    } else {   // xorshift64* (Vigna 2016), top 24 bits scaled to [0, 1]
        m_seed ^= m_seed >> 12;
        m_seed ^= m_seed << 25;
        m_seed ^= m_seed >> 27;
        const uint64_t r = m_seed * 0x2545F4914F6CDD1Dull;
        u = float(uint32_t(r >> 40)) / float(0xFFFFFF);
    }
    return (u * (mx - mn)) + mn;
}

bool TressFXAsset::LoadHairData(FILE* ioObject) {
    if (!ioObject) return false;
    TressFXTFXFileHeader header;
    std::memset(&header, 0, sizeof(header));
    EI_Seek(ioObject, 0);
    if (!read_exact(&header, sizeof(header), ioObject)) return false;
    if (header.version < AMD_TRESSFX_VERSION_MAJOR) return false;

    const unsigned int numStrandsInFile = header.numHairStrands;
    const int n = (int)header.numVerticesPerStrand;
    if (numStrandsInFile == 0 || !(n > 2 && n <= TRESSFX_SIM_THREAD_GROUP_SIZE && TRESSFX_SIM_THREAD_GROUP_SIZE % n == 0))
        return false;
    // the strand count is raised to a multiple of the thread-group size, always by at least one
    // strand (TressFXAsset.cpp:111)
    m_numGuideStrands = (int)((numStrandsInFile - numStrandsInFile % TRESSFX_SIM_THREAD_GROUP_SIZE) +
                              TRESSFX_SIM_THREAD_GROUP_SIZE);
    m_numVerticesPerStrand = n;
    m_numFollowStrandsPerGuide = 0;
    m_numTotalStrands = m_numGuideStrands;
    m_numGuideVertices = m_numGuideStrands * m_numVerticesPerStrand;
    m_numTotalVertices = m_numGuideVertices;

    m_positions.assign(m_numTotalVertices, Vector3());
    EI_Seek(ioObject, (long)header.offsetVertexPosition);
    if (!read_exact(m_positions.data(), (size_t)numStrandsInFile * n * sizeof(AMD::float4), ioObject)) return false;
    // made-up strands repeat the file's last strand
    const int padStrands = m_numGuideStrands - (int)numStrandsInFile;
    for (int i = 0; i < padStrands; ++i)
        for (int j = 0; j < n; ++j)
            m_positions[(numStrandsInFile + i) * n + j] = m_positions[(numStrandsInFile - 1) * n + j];

    m_strandUV.assign(m_numTotalStrands, AMD::float2{0.0f, 0.0f});
    EI_Seek(ioObject, (long)header.offsetStrandUV);
    if (!read_exact(m_strandUV.data(), (size_t)numStrandsInFile * sizeof(AMD::float2), ioObject)) return false;
    for (int i = 0; i < padStrands; ++i) m_strandUV[numStrandsInFile + i] = m_strandUV[numStrandsInFile - 1];

    m_followRootOffsets.assign(m_numTotalStrands, Vector3());
    return true;
}

bool TressFXAsset::GenerateFollowHairs(int numFollowHairsPerGuideHair, float tipSeparationFactor,
                                       float maxRadiusAroundGuideHair) {
    if (numFollowHairsPerGuideHair < 0) return false;
    m_numFollowStrandsPerGuide = numFollowHairsPerGuideHair;
    if (numFollowHairsPerGuideHair == 0) return false;

    const int n = m_numVerticesPerStrand;
    const int group = numFollowHairsPerGuideHair + 1;      // a guide and its follow strands, in that order
    m_numTotalStrands = m_numGuideStrands * group;
    m_numTotalVertices = m_numTotalStrands * n;

    std::vector<Vector3> guides;
    std::vector<AMD::float2> guideUV;
    guides.swap(m_positions);
    guideUV.swap(m_strandUV);
    m_positions.assign(m_numTotalVertices, Vector3());
    m_strandUV.assign(m_numTotalStrands, AMD::float2{0.0f, 0.0f});
    m_followRootOffsets.assign(m_numTotalStrands, Vector3());

    // a follow strand's offset from its guide grows linearly along the strand, from 1x at the root
    std::vector<float> spread(n);
    for (int k = 0; k < n; ++k) spread[k] = tipSeparationFactor * ((float)k / ((float)n)) + 1.0f;

    for (int g = 0; g < m_numGuideStrands; ++g) {
        const int lead = g * group;                         // the guide's strand index in the output
        const Vector3* src = &guides[(size_t)g * n];
        Vector3* guide = &m_positions[(size_t)lead * n];
        std::copy(src, src + n, guide);
        m_strandUV[lead] = guideUV[g];
        m_followRootOffsets[lead] = Vector3(0.0f, 0.0f, 0.0f, (float)lead);

        // the plane of root offsets: normal to the guide's first segment
        Vector3 axis = guide[1] - guide[0];
        axis.Normalize();
        Vector3 u, v;
        tangent_vectors(axis, u, v);

        for (int f = 1; f < group; ++f) {
            const int s = lead + f;
            m_strandUV[s] = m_strandUV[lead];
            // The reference forms the offset from two draws in one expression, which leaves their order
            // to the compiler; g++ draws the coefficient of the second direction first, and so does this.
            const float cv = GetRandom(-maxRadiusAroundGuideHair, maxRadiusAroundGuideHair);
            const float cu = GetRandom(-maxRadiusAroundGuideHair, maxRadiusAroundGuideHair);
            const Vector3 offset = cu * u + cv * v;
            m_followRootOffsets[s] = offset;
            m_followRootOffsets[s].w = (float)lead;
            Vector3* follow = &m_positions[(size_t)s * n];
            for (int k = 0; k < n; ++k) {
                follow[k] = guide[k] + offset * spread[k];
                follow[k].w = guide[k].w;                   // the inverse mass is the guide's
            }
        }
    }
    return true;
}

bool TressFXAsset::ProcessAsset() {
    if (m_numTotalStrands <= 0 || m_numVerticesPerStrand <= 1) return false;
    m_strandTypes.assign(m_numTotalStrands, 0);
    m_tangents.assign(m_numTotalVertices, AMD::float4{0.0f, 0.0f, 0.0f, 0.0f});
    m_restLengths.assign(m_numTotalVertices, 0.0f);
    m_thicknessCoeffs.assign(m_numTotalVertices, 0.0f);
    m_triangleIndices.assign(GetNumHairTriangleIndices(), 0);
    ComputeStrandTangent();
    ComputeThicknessCoeffs();
    ComputeRestLengths();
    FillTriangleIndexArray();
    return true;
}

// Two triangles per segment over the expanded vertex pairs (vertex v of the strands expands to 2v and
// 2v + 1, TressFXAsset.cpp:392-399).
void TressFXAsset::FillTriangleIndexArray() {
    const int n = m_numVerticesPerStrand;
    AMD::int32* out = m_triangleIndices.data();
    for (int s = 0; s < m_numTotalStrands; ++s)
        for (int j = 0; j + 1 < n; ++j) {
            const AMD::int32 a = 2 * (s * n + j);
            const AMD::int32 quad[6] = {a, a + 1, a + 2, a + 2, a + 1, a + 3};
            out = std::copy(quad, quad + 6, out);
        }
}

// Tangents (TressFXAsset.cpp:294-332): the root along its segment, an inner vertex along the sum of the
// unit directions of its two segments, the tip left at zero.
void TressFXAsset::ComputeStrandTangent() {
    const int n = m_numVerticesPerStrand;
    auto dir = [](const Vector3& from, const Vector3& to) {
        Vector3 d = to - from;
        d.Normalize();
        return d;
    };
    for (int s = 0; s < m_numTotalStrands; ++s) {
        const Vector3* p = &m_positions[(size_t)s * n];
        AMD::float4* t = &m_tangents[(size_t)s * n];
        const Vector3 root = dir(p[0], p[1]);
        t[0] = AMD::float4{root.x, root.y, root.z, root.w};
        for (int i = 1; i + 1 < n; ++i) {
            Vector3 sum = dir(p[i - 1], p[i]) + dir(p[i], p[i + 1]);
            sum.Normalize();
            t[i] = AMD::float4{sum.x, sum.y, sum.z, sum.w};
        }
    }
}

// Thickness coefficients (TressFXAsset.cpp:334-364).  The reference divides a running value, first the
// strand length L, by L once per vertex, so vertex k gets sqrt(1 - r^2) with r = L^-k (in float); kept as
// it is, since renderers read these values.
void TressFXAsset::ComputeThicknessCoeffs() {
    const int n = m_numVerticesPerStrand;
    for (int s = 0; s < m_numTotalStrands; ++s) {
        const Vector3* p = &m_positions[(size_t)s * n];
        float length = 0;
        for (int i = 1; i < n; ++i) length += (p[i] - p[i - 1]).Length();
        float ratio = length;
        float* out = &m_thicknessCoeffs[(size_t)s * n];
        for (int i = 0; i < n; ++i) {
            ratio /= length;
            out[i] = sqrtf(1.f - ratio * ratio);
        }
    }
}

// Rest lengths (TressFXAsset.cpp:366-390): the length of the segment after each vertex, 0 at the tip.
void TressFXAsset::ComputeRestLengths() {
    const int n = m_numVerticesPerStrand;
    for (int s = 0; s < m_numTotalStrands; ++s) {
        const Vector3* p = &m_positions[(size_t)s * n];
        float* out = &m_restLengths[(size_t)s * n];
        for (int j = 0; j + 1 < n; ++j) out[j] = (p[j] - p[j + 1]).Length();
        out[n - 1] = 0;
    }
}

bool TressFXAsset::LoadBoneData(FILE* ioObject, int skinNumber, EI_Scene* scene) {
    m_boneSkinningData.clear();
    if (!ioObject || !scene) return false;
    AMD::int32 boneCount = 0;
    EI_Seek(ioObject, 0);
    if (!read_exact(&boneCount, sizeof(boneCount), ioObject) || boneCount < 0) return false;

    std::vector<int> engineId(boneCount);
    for (int i = 0; i < boneCount; i++) {
        AMD::int32 boneIndex = 0, charLen = 0;
        if (!read_exact(&boneIndex, sizeof(boneIndex), ioObject)) return false;
        if (!read_exact(&charLen, sizeof(charLen), ioObject) || charLen < 0 || charLen > 128) return false;
        char boneName[129] = {};
        if (!read_exact(boneName, (size_t)charLen, ioObject)) return false;
        engineId[i] = scene->GetBoneIdByName(skinNumber, boneName);
    }

    AMD::int32 recordCount = 0;
    if (!read_exact(&recordCount, sizeof(recordCount), ioObject)) return false;
    if (m_numGuideStrands < recordCount || recordCount <= 0) return false;

    m_boneSkinningData.assign(m_numTotalStrands, TressFXBoneSkinningData{{0, 0, 0, 0}, {0, 0, 0, 0}});
    TressFXBoneSkinningData record{{0, 0, 0, 0}, {0, 0, 0, 0}};
    for (int i = 0; i < recordCount; ++i) {
        AMD::int32 index = 0;
        if (!read_exact(&index, sizeof(index), ioObject)) return false;
        for (int j = 0; j < TRESSFX_MAX_INFLUENTIAL_BONE_COUNT; ++j) {
            AMD::int32 boneIndex = 0;
            if (!read_exact(&boneIndex, sizeof(boneIndex), ioObject)) return false;
            if (boneIndex < 0 || boneIndex >= boneCount) return false;
            record.boneIndex[j] = (float)engineId[boneIndex];
            if (!read_exact(&record.weight[j], sizeof(float), ioObject)) return false;
        }
        // an index of -1 (no bone) becomes 0; its weight is zero
        for (int j = 0; j < TRESSFX_MAX_INFLUENTIAL_BONE_COUNT; ++j)
            record.boneIndex[j] = record.boneIndex[j] == -1.f ? 0 : record.boneIndex[j];
        m_boneSkinningData[(size_t)i * (m_numFollowStrandsPerGuide + 1)] = record;
    }
    // made-up guide strands take the last strand's skinning
    for (int i = recordCount; i < m_numGuideStrands; ++i)
        m_boneSkinningData[(size_t)i * (m_numFollowStrandsPerGuide + 1)] = record;
    return true;
}
