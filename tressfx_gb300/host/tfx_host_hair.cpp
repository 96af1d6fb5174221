// TressFXHairObject and TressFXSimulation over the C ABI (src/TressFX/TressFXHairObject.cpp:44-437,
// src/TressFX/TressFXSimulation.cpp:51-112).
#include <algorithm>
#include <cstring>

#include "tfx_host_check.h"
#include "tressfx/TressFXSimulation.h"

using tfxhost::check;

TressFXHairObject::TressFXHairObject(TressFXAsset* asset, EI_Device* pDevice, EI_CommandContext& /*commandContext*/,
                                     const char* /*name*/, int RenderIndex)
    : m_RenderIndex(RenderIndex) {
    if (!asset || !pDevice) throw TressFXError(TFX_ERR_INVALID_ARGUMENT, "TressFXHairObject: null asset or device");
    m_NumTotalVertices = asset->m_numTotalVertices;
    m_NumTotalStrands = asset->m_numTotalStrands;
    m_NumVerticesPerStrand = asset->m_numVerticesPerStrand;
    m_NumFollowHairsPerGuideHair = asset->m_numFollowStrandsPerGuide;
    const size_t V = (size_t)m_NumTotalVertices, S = (size_t)m_NumTotalStrands;
    if (asset->m_positions.size() < V || asset->m_tangents.size() < V || asset->m_restLengths.size() < V ||
        asset->m_followRootOffsets.size() < S || asset->m_boneSkinningData.size() < S)
        throw TressFXError(TFX_ERR_INVALID_ARGUMENT,
                           "TressFXHairObject: asset arrays shorter than its counts (call ProcessAsset and LoadBoneData)");

    tfx_hair_desc d;
    std::memset(&d, 0, sizeof(d));
    d.num_guide_strands = asset->m_numGuideStrands;
    d.verts_per_strand = m_NumVerticesPerStrand;
    d.follow_hairs_per_guide = m_NumFollowHairsPerGuideHair;
    check(tfx_hair_create(pDevice->GetContext(), &d, reinterpret_cast<const float*>(asset->m_positions.data()),
                          reinterpret_cast<const float*>(asset->m_tangents.data()), asset->m_restLengths.data(),
                          reinterpret_cast<const float*>(asset->m_followRootOffsets.data()),
                          reinterpret_cast<const float*>(asset->m_boneSkinningData.data()), &m_hair),
          "TressFXHairObject");

    m_SimCBStorage.reset(new tfx_sim_params[2]);
    std::memset(m_SimCBStorage.get(), 0, 2 * sizeof(tfx_sim_params));
    m_SimCB = m_SimCBStorage.get();

    auto bind = [&](int buf, EI_Resource& r) {
        void* p = nullptr;
        size_t bytes = 0;
        check(tfx_hair_get_buffer(m_hair, buf, &p, &bytes), "TressFXHairObject: buffer");
        r = EI_Resource(p, bytes);
    };
    bind(TFX_BUF_POSITIONS, m_DynamicState.m_Positions);
    bind(TFX_BUF_TANGENTS, m_DynamicState.m_Tangents);
    bind(TFX_BUF_POSITIONS_PREV, m_DynamicState.m_PositionsPrev);
    bind(TFX_BUF_POSITIONS_PREV_PREV, m_DynamicState.m_PositionsPrevPrev);
    bind(TFX_BUF_STRAND_LEVEL_DATA, m_DynamicState.m_StrandLevelData);
    ResetPositions();
}

TressFXHairObject::~TressFXHairObject() {
    if (m_hair) tfx_hair_destroy(m_hair);
}

void TressFXHairObject::UpdateBoneMatrices(const AMD::float4x4* pBoneMatricesInWS, int numBoneMatrices) {
    const int numMatrices = std::min(numBoneMatrices, AMD_TRESSFX_MAX_NUM_BONES);
    for (int i = 0; i < numMatrices; ++i)
        std::memcpy(m_SimCB[m_SimulationFrame % 2].bone_matrices[i], pBoneMatricesInWS[i].m, sizeof(float) * 16);
    m_numBones = std::max(m_numBones, numMatrices);
}

void TressFXHairObject::UpdateConstantBuffer(EI_CommandContext& /*commandContext*/) {
    check(tfx_hair_update_constants(m_hair, &m_SimCB[m_SimulationFrame % 2], m_numBones), "UpdateConstantBuffer");
}

void TressFXHairObject::UpdateSimulationParameters(const TressFXSimulationSettings* settings, float timeStep) {
    if (!settings) throw TressFXError(TFX_ERR_INVALID_ARGUMENT, "UpdateSimulationParameters: null settings");
    const tfx_sim_settings s = settings->ToC();
    int32_t it = 0;
    check(tfx_fill_sim_params(&m_SimCB[m_SimulationFrame % 2], &s, timeStep, m_NumVerticesPerStrand,
                              m_NumFollowHairsPerGuideHair, m_SimulationFrame, &it),
          "UpdateSimulationParameters");
    m_CPULocalShapeIterations = it;
}

// ---------------------------------------------------------------------------------------------
void TressFXSimulation::Initialize(EI_Device* pDevice) { m_device = pDevice; }

void TressFXSimulation::Simulate(EI_CommandContext& commandContext, std::vector<TressFXHairObject*>& hairObjects) {
    struct Stage {
        int kernel;
        const char* stamp;
        bool iterate;
    };
    static const Stage stages[] = {
        {TFX_KERNEL_INTEGRATION_AND_GLOBAL_SHAPE, "IntegrationAndGlobalShapeContraints", false},
        {TFX_KERNEL_STRAND_LEVEL_DATA, "CalculateStrandLevelData", false},
        {TFX_KERNEL_VELOCITY_SHOCK_PROPAGATION, "VelocityShockPropagation", false},
        {TFX_KERNEL_LOCAL_SHAPE_CONSTRAINTS, "LocalShapeConstraints", true},
        {TFX_KERNEL_LENGTH_WIND_COLLISION, "LengthConstriantsWindAndCollision", false},
        {TFX_KERNEL_UPDATE_FOLLOW_HAIR, "UpdateFollowHairVertices", false},
    };
    EI_Device& device = m_device ? *m_device : commandContext.GetDevice();
    for (auto* o : hairObjects) o->UpdateConstantBuffer(commandContext);
    for (const Stage& st : stages) {
        for (auto* o : hairObjects)
            check(tfx_hair_dispatch(o->GetHandle(), st.kernel, st.iterate ? o->GetCPULocalShapeIterations() : 1), st.stamp);
        device.GetTimeStamp(st.stamp);
    }
    for (auto* o : hairObjects) o->IncreaseSimulationFrame();
}
