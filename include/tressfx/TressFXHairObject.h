// TressFXHairObject / TressFXDynamicState (src/TressFX/TressFXHairObject.h:43-191): the simulation
// side of a hair object.  Same constructor and members a simulation caller uses; the GPU buffers
// live in a tfx_hair handle of the C ABI, the two constant blocks m_SimCB[frame % 2] on the host.
#pragma once

#include <memory>
#include <vector>

#include "EngineInterface.h"
#include "TressFXAsset.h"
#include "TressFXSettings.h"

struct TressFXStrandLevelData {
    AMD::float4 skinningQuat;
    AMD::float4 vspQuat;
    AMD::float4 vspTranslation;
};

// The dynamic buffers shared by simulation, SDF collision and rendering.
class TressFXDynamicState {
public:
    EI_Resource& GetPositions() { return m_Positions; }
    EI_Resource& GetTangents() { return m_Tangents; }
    EI_Resource& GetPositionsPrev() { return m_PositionsPrev; }
    EI_Resource& GetPositionsPrevPrev() { return m_PositionsPrevPrev; }
    EI_Resource& GetStrandLevelData() { return m_StrandLevelData; }
    // Buffers are device memory in stream order: nothing to transition.
    void UAVBarrier(EI_CommandContext&) {}
    void TransitionSimToRendering(EI_CommandContext&) {}
    void TransitionRenderingToSim(EI_CommandContext&) {}

private:
    friend class TressFXHairObject;
    EI_Resource m_Positions, m_Tangents, m_PositionsPrev, m_PositionsPrevPrev, m_StrandLevelData;
};

class TressFXHairObject : private TressFXNonCopyable {
public:
    TressFXHairObject(TressFXAsset* asset, EI_Device* pDevice, EI_CommandContext& commandContext, const char* name,
                      int RenderIndex);
    ~TressFXHairObject();

    // Bone matrices (row-major, row-vector convention) into this frame's constant block.
    void UpdateBoneMatrices(const AMD::float4x4* pBoneMatricesInWS, int numBoneMatrices);
    // Uploads this frame's constant block.
    void UpdateConstantBuffer(EI_CommandContext& commandContext);
    void UpdateSimulationParameters(const TressFXSimulationSettings* parameters, float timeStep);

    void ResetPositions() { m_SimCB[m_SimulationFrame % 2].reset_positions = 1.0f; }
    void IncreaseSimulationFrame() {
        m_SimCB[m_SimulationFrame % 2].reset_positions = 0.0f;
        m_SimulationFrame++;
    }

    TressFXDynamicState& GetDynamicState() { return m_DynamicState; }

    int GetNumTotalHairVertices() const { return m_NumTotalVertices; }
    int GetNumTotalHairStrands() const { return m_NumTotalStrands; }
    int GetNumVerticesPerStrand() const { return m_NumVerticesPerStrand; }
    int GetCPULocalShapeIterations() const { return m_CPULocalShapeIterations; }
    int GetNumFollowHairsPerGuideHair() const { return m_NumFollowHairsPerGuideHair; }
    int GetSimulationFrame() const { return m_SimulationFrame; }

    // The C-ABI handle and this frame's constant block (for the batched path and for readback).
    tfx_hair GetHandle() const { return m_hair; }
    const tfx_sim_params& GetCurrentConstants() const { return m_SimCB[m_SimulationFrame % 2]; }
    int GetNumBones() const { return m_numBones; }

private:
    int m_NumTotalVertices = 0, m_NumTotalStrands = 0, m_NumVerticesPerStrand = 0;
    int m_NumFollowHairsPerGuideHair = 0;
    int m_CPULocalShapeIterations = 0;
    int m_SimulationFrame = 0;
    int m_RenderIndex = 0;
    int m_numBones = 0;
    tfx_hair m_hair = nullptr;
    std::unique_ptr<tfx_sim_params[]> m_SimCBStorage;
    tfx_sim_params* m_SimCB = nullptr;   // [2]
    TressFXDynamicState m_DynamicState;
};
