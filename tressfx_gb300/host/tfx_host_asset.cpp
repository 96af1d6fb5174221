// TressFXAsset: .tfx / .tfxbone loading, procedural follow hairs and the derived simulation data,
// following src/TressFX/TressFXAsset.cpp step for step (same arithmetic on the same types).
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
    const int numStrandsToMakeUp = m_numGuideStrands - (int)numStrandsInFile;
    for (int i = 0; i < numStrandsToMakeUp; ++i)
        for (int j = 0; j < n; ++j)
            m_positions[(numStrandsInFile + i) * n + j] = m_positions[(numStrandsInFile - 1) * n + j];

    m_strandUV.assign(m_numTotalStrands, AMD::float2{0.0f, 0.0f});
    EI_Seek(ioObject, (long)header.offsetStrandUV);
    if (!read_exact(m_strandUV.data(), (size_t)numStrandsInFile * sizeof(AMD::float2), ioObject)) return false;
    for (int i = 0; i < numStrandsToMakeUp; ++i) m_strandUV[numStrandsInFile + i] = m_strandUV[numStrandsInFile - 1];

    m_followRootOffsets.assign(m_numTotalStrands, Vector3());
    return true;
}

bool TressFXAsset::GenerateFollowHairs(int numFollowHairsPerGuideHair, float tipSeparationFactor,
                                       float maxRadiusAroundGuideHair) {
    if (numFollowHairsPerGuideHair < 0) return false;
    m_numFollowStrandsPerGuide = numFollowHairsPerGuideHair;
    if (numFollowHairsPerGuideHair == 0) return false;

    const int n = m_numVerticesPerStrand;
    m_numTotalStrands = m_numGuideStrands * (m_numFollowStrandsPerGuide + 1);
    m_numTotalVertices = m_numTotalStrands * n;

    const std::vector<Vector3> positionsGuide = m_positions;
    const std::vector<AMD::float2> strandUVGuide = m_strandUV;
    m_positions.assign(m_numTotalVertices, Vector3());
    m_strandUV.assign(m_numTotalStrands, AMD::float2{0.0f, 0.0f});
    m_followRootOffsets.assign(m_numTotalStrands, Vector3());

    Vector3* pos = m_positions.data();
    Vector3* followOffset = m_followRootOffsets.data();
    for (int i = 0; i < m_numGuideStrands; i++) {
        const int indexGuideStrand = i * (m_numFollowStrandsPerGuide + 1);
        const int indexRootVertMaster = indexGuideStrand * n;
        std::memcpy(&pos[indexRootVertMaster], &positionsGuide[(size_t)i * n], sizeof(Vector3) * n);
        m_strandUV[indexGuideStrand] = strandUVGuide[i];

        followOffset[indexGuideStrand].Set(0, 0, 0);
        followOffset[indexGuideStrand].w = (float)indexGuideStrand;
        Vector3 v01 = pos[indexRootVertMaster + 1] - pos[indexRootVertMaster];
        v01.Normalize();
        Vector3 t0, t1;
        tangent_vectors(v01, t0, t1);

        for (int j = 0; j < m_numFollowStrandsPerGuide; j++) {
            const int indexStrandFollow = indexGuideStrand + j + 1;
            const int indexRootVertFollow = indexStrandFollow * n;
            m_strandUV[indexStrandFollow] = m_strandUV[indexGuideStrand];
            // offset = r0 * t0 + r1 * t1.  The reference writes both draws in one expression, which
            // leaves their order to the compiler; g++ draws the t1 coefficient first, and so does this.
            const float r1 = GetRandom(-maxRadiusAroundGuideHair, maxRadiusAroundGuideHair);
            const float r0 = GetRandom(-maxRadiusAroundGuideHair, maxRadiusAroundGuideHair);
            const Vector3 offset = r0 * t0 + r1 * t1;
            followOffset[indexStrandFollow] = offset;
            followOffset[indexStrandFollow].w = (float)indexGuideStrand;
            for (int k = 0; k < n; k++) {
                const Vector3& guideVert = pos[indexRootVertMaster + k];
                Vector3& followVert = pos[indexRootVertFollow + k];
                const float factor = tipSeparationFactor * ((float)k / ((float)n)) + 1.0f;
                followVert = guideVert + offset * factor;
                followVert.w = guideVert.w;
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

void TressFXAsset::FillTriangleIndexArray() {
    AMD::int32 id = 0;
    int iCount = 0;
    for (int i = 0; i < m_numTotalStrands; i++) {
        for (int j = 0; j < m_numVerticesPerStrand - 1; j++) {
            m_triangleIndices[iCount++] = 2 * id;
            m_triangleIndices[iCount++] = 2 * id + 1;
            m_triangleIndices[iCount++] = 2 * id + 2;
            m_triangleIndices[iCount++] = 2 * id + 2;
            m_triangleIndices[iCount++] = 2 * id + 1;
            m_triangleIndices[iCount++] = 2 * id + 3;
            id++;
        }
        id++;
    }
}

// ComputeStrandTangent (TressFXAsset.cpp:294-332): vertex 0 along the first segment, inner vertices
// along the sum of the two unit segment directions, the last vertex left at zero.
void TressFXAsset::ComputeStrandTangent() {
    const int n = m_numVerticesPerStrand;
    auto store = [&](int idx, const Vector3& t) { m_tangents[idx] = AMD::float4{t.x, t.y, t.z, t.w}; };
    for (int iStrand = 0; iStrand < m_numTotalStrands; ++iStrand) {
        const int root = iStrand * n;
        {
            Vector3 tangent = m_positions[root + 1] - m_positions[root];
            tangent.Normalize();
            store(root, tangent);
        }
        for (int i = 1; i < n - 1; i++) {
            Vector3 pre = m_positions[root + i] - m_positions[root + i - 1];
            pre.Normalize();
            Vector3 next = m_positions[root + i + 1] - m_positions[root + i];
            next.Normalize();
            Vector3 tangent = pre + next;
            tangent = tangent.Normalize();
            store(root + i, tangent);
        }
    }
}

// ComputeThicknessCoeffs (TressFXAsset.cpp:334-364), including its running division of the strand
// length.
void TressFXAsset::ComputeThicknessCoeffs() {
    const int n = m_numVerticesPerStrand;
    int index = 0;
    for (int iStrand = 0; iStrand < m_numTotalStrands; ++iStrand) {
        const int root = iStrand * n;
        float strandLength = 0;
        float tVal = 0;
        for (int i = 1; i < n; ++i) {
            const Vector3 vec = m_positions[root + i] - m_positions[root + i - 1];
            const float disSeg = vec.Length();
            tVal += disSeg;
            strandLength += disSeg;
        }
        for (int i = 0; i < n; ++i) {
            tVal /= strandLength;
            m_thicknessCoeffs[index++] = sqrtf(1.f - tVal * tVal);
        }
    }
}

// ComputeRestLengths (TressFXAsset.cpp:366-390): |p_j - p_{j+1}|, 0 for the last vertex.
void TressFXAsset::ComputeRestLengths() {
    const int n = m_numVerticesPerStrand;
    int index = 0;
    for (int i = 0; i < m_numTotalStrands; i++) {
        const int root = i * n;
        for (int j = 0; j < n - 1; j++) m_restLengths[index++] = (m_positions[root + j] - m_positions[root + j + 1]).Length();
        m_restLengths[index++] = 0;
    }
}

bool TressFXAsset::LoadBoneData(FILE* ioObject, int skinNumber, EI_Scene* scene) {
    m_boneSkinningData.clear();
    if (!ioObject || !scene) return false;
    AMD::int32 numOfBones = 0;
    EI_Seek(ioObject, 0);
    if (!read_exact(&numOfBones, sizeof(numOfBones), ioObject) || numOfBones < 0) return false;

    std::vector<int> boneEngineIds(numOfBones);
    for (int i = 0; i < numOfBones; i++) {
        AMD::int32 boneIndex = 0, charLen = 0;
        if (!read_exact(&boneIndex, sizeof(boneIndex), ioObject)) return false;
        if (!read_exact(&charLen, sizeof(charLen), ioObject) || charLen < 0 || charLen > 128) return false;
        char boneName[129] = {};
        if (!read_exact(boneName, (size_t)charLen, ioObject)) return false;
        boneEngineIds[i] = scene->GetBoneIdByName(skinNumber, boneName);
    }

    AMD::int32 numOfStrandsInStream = 0;
    if (!read_exact(&numOfStrandsInStream, sizeof(numOfStrandsInStream), ioObject)) return false;
    if (m_numGuideStrands < numOfStrandsInStream || numOfStrandsInStream <= 0) return false;

    m_boneSkinningData.assign(m_numTotalStrands, TressFXBoneSkinningData{{0, 0, 0, 0}, {0, 0, 0, 0}});
    TressFXBoneSkinningData skinData{{0, 0, 0, 0}, {0, 0, 0, 0}};
    for (int i = 0; i < numOfStrandsInStream; ++i) {
        AMD::int32 index = 0;
        if (!read_exact(&index, sizeof(index), ioObject)) return false;
        for (int j = 0; j < TRESSFX_MAX_INFLUENTIAL_BONE_COUNT; ++j) {
            AMD::int32 boneIndex = 0;
            if (!read_exact(&boneIndex, sizeof(boneIndex), ioObject)) return false;
            if (boneIndex < 0 || boneIndex >= numOfBones) return false;
            skinData.boneIndex[j] = (float)boneEngineIds[boneIndex];
            if (!read_exact(&skinData.weight[j], sizeof(float), ioObject)) return false;
        }
        // an index of -1 (no bone) becomes 0; its weight is zero
        for (int j = 0; j < TRESSFX_MAX_INFLUENTIAL_BONE_COUNT; ++j)
            skinData.boneIndex[j] = skinData.boneIndex[j] == -1.f ? 0 : skinData.boneIndex[j];
        m_boneSkinningData[(size_t)i * (m_numFollowStrandsPerGuide + 1)] = skinData;
    }
    // made-up guide strands take the last strand's skinning
    for (int i = numOfStrandsInStream; i < m_numGuideStrands; ++i)
        m_boneSkinningData[(size_t)i * (m_numFollowStrandsPerGuide + 1)] = skinData;
    return true;
}
