// TressFXSimulation (src/TressFX/TressFXSimulation.h:31-48): runs the six simulation stages over a
// list of hair objects, stage-major and object-minor as TressFXSimulation::Simulate does
// (TressFXSimulation.cpp:77-112), with the same timestamps.
#pragma once

#include <vector>

#include "EngineInterface.h"
#include "TressFXHairObject.h"

class TressFXSimulation : private TressFXNonCopyable {
public:
    void Initialize(EI_Device* pDevice);
    void Simulate(EI_CommandContext& commandContext, std::vector<TressFXHairObject*>& hairObjects);
private:
    EI_Device* m_device = nullptr;
};
