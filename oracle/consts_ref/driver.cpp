// Compiles the reference's own SetWindCorner / TressFXHairObject::SetWind /
// TressFXHairObject::UpdateSimulationParameters (cut unchanged out of
// src/TressFX/TressFXHairObject.cpp into hair_object_consts.inc by build.py) inside a minimal
// stand-in for TressFXHairObject: the two constant blocks m_SimCB[2], the frame counter, the strand
// counts and ResetPositions (TressFXHairObject.h:104).  Test infrastructure: a checker for the
// library's tfx_fill_sim_params and the oracle's restatement.
//
// The reference is a Windows program (src/CMakeLists.txt:63, build/GenerateSolutions.bat), and MSVC
// declares the float overloads of the math functions in the global namespace, so its unqualified
// sin(float), pow(float, float) and asin(float) are the float functions.  libstdc++'s <math.h> does
// the same; it is included first so that the cut code resolves those calls as the reference's own
// build does (with only <cmath>, g++ would call the double versions).
#include <math.h>

#include <cstdint>
#include <cstring>

#include "AMD_TressFX.h"
#include "AMD_Types.h"
#include "Math/Matrix44.h"
#include "Math/Quaternion.h"
#include "Math/Vector3D.h"
#include "TressFXCommon.h"
#include "TressFXConstantBuffers.h"
#include "TressFXSettings.h"

using namespace AMD;

#define TRESSFX_MIN_VERTS_PER_STRAND_FOR_GPU_ITERATION 64   // TressFXHairObject.cpp:40

// TressFXConstantBuffer<T> (the EI constant-buffer wrapper) reduced to what the cut code uses: ->.
template <class T> struct ConstantBufferStandIn {
    T data;
    T* operator->() { return &data; }
};

class TressFXHairObject {
public:
    void SetWind(const Vector3& windDir, float windMag, int frame);
    void UpdateSimulationParameters(const TressFXSimulationSettings* settings, float timeStep);
    void ResetPositions() { m_SimCB[m_SimulationFrame % 2]->g_ResetPositions = 1.0f; }
    void IncreaseSimulationFrame() { m_SimCB[m_SimulationFrame % 2]->g_ResetPositions = 0.0f; m_SimulationFrame++; }

    ConstantBufferStandIn<TressFXSimulationParams> m_SimCB[2];
    int m_SimulationFrame = 0;
    int m_NumVerticesPerStrand = 0;
    int m_NumFollowHairsPerGuideHair = 0;
    int m_CPULocalShapeIterations = 0;
};

#include "hair_object_consts.inc"

static_assert(sizeof(TressFXSimulationSettings) == 16 * 4, "TressFXSimulationSettings layout");
static_assert(offsetof(TressFXSimulationParams, m_BoneSkinningMatrix) == 160, "TressFXSimulationParams layout");

extern "C" void ref_settings_default(TressFXSimulationSettings* out) { *out = TressFXSimulationSettings(); }

// An object whose constant blocks start zeroed, advanced from frame 0 to `frame` by
// IncreaseSimulationFrame (as Simulate does once per frame), then UpdateSimulationParameters:
// the 160-byte header of m_SimCB[frame % 2] and m_CPULocalShapeIterations.
extern "C" int ref_update_simulation_parameters(const TressFXSimulationSettings* s, float timeStep, int n, int F, int frame,
                                                void* header160, int32_t* cpuIterations) {
    if (!s || !header160 || frame < 0 || n <= 0) return 1;
    static TressFXHairObject obj;   // 64 KB of constant blocks: kept off the stack
    std::memset(&obj.m_SimCB[0].data, 0, sizeof(TressFXSimulationParams));
    std::memset(&obj.m_SimCB[1].data, 0, sizeof(TressFXSimulationParams));
    obj.m_SimulationFrame = 0;
    obj.m_NumVerticesPerStrand = n;
    obj.m_NumFollowHairsPerGuideHair = F;
    obj.ResetPositions();   // the constructor's reset (TressFXHairObject.cpp:157)
    for (int f = 0; f < frame; ++f) obj.IncreaseSimulationFrame();
    obj.UpdateSimulationParameters(s, timeStep);
    std::memcpy(header160, &obj.m_SimCB[frame % 2].data, 160);
    if (cpuIterations) *cpuIterations = obj.m_CPULocalShapeIterations;
    return 0;
}
