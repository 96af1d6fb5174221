// TressFXSDFMarchingCubes (src/TressFX/TressFXSDFMarchingCubes.h:46-118): the iso-surface of a
// TressFXSDFCollision's grid as a triangle soup, headless.  The reference's Draw / DrawGrid render the
// soup through the engine's graphics pipeline; here the vertex buffer ({float4 position, float4
// normal}[max vertices], StandardVertex of TressFXMarchingCubes.hlsl:33-37) is handed out instead.
#pragma once

#include <vector>

#include "EngineInterface.h"
#include "TressFXSDFCollision.h"

class TressFXSDFMarchingCubes : private TressFXNonCopyable {
public:
    TressFXSDFMarchingCubes();                      // 128 * 1024 vertices, as the reference
    explicit TressFXSDFMarchingCubes(int maxVertices);
    ~TressFXSDFMarchingCubes();

    // The reference creates its compute PSOs, buffers and draw pipeline here (name, scene and render
    // targets); the kernels are linked in, so this records the device.  The buffers are created at
    // the first Update, sized for the SDF's allocation.
    void Initialize(const char* name, EI_Device* pDevice);
    void SetSDF(TressFXSDFCollision* SDF) { m_pSDF = SDF; }
    // In cells: the surface is the SDF value cellSize * isoLevel.
    void SetSDFIsoLevel(float isoLevel) { m_SDFIsoLevel = isoLevel; }
    // InitializeMCVertices + RunMarchingCubesOnSdf over the SDF's current grid (stream ordered).
    void Update(EI_CommandContext& commandContext);

    int GetMaxVertices() const { return m_MaxMarchingCubesVertices; }
    // The device vertex buffer and counter (valid after the first Update).
    EI_Resource GetVerticesGPUBuffer() const;
    // Copies the vertex buffer to `out` (8 floats per vertex) and returns the counter (synchronizes).
    int ReadVertices(std::vector<float>& out) const;
    tfx_mc GetHandle() const { return m_mc; }

private:
    EI_Device* m_pDevice = nullptr;
    TressFXSDFCollision* m_pSDF = nullptr;
    float m_SDFIsoLevel = 0.0f;
    const int m_MaxMarchingCubesVertices;
    tfx_mc m_mc = nullptr;
};
