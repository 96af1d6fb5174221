// EI_Device over a tfx_context.
#include <cstring>

#include "tfx_host_check.h"
#include "tressfx/EngineInterface.h"

EI_Device::EI_Device(int cudaDevice) { tfxhost::check(tfx_context_create(cudaDevice, &m_ctx), "EI_Device"); }

EI_Device::~EI_Device() {
    if (m_ctx) tfx_context_destroy(m_ctx);
}

void EI_Device::GetTimeStamp(const char* name) { tfxhost::check(tfx_context_timestamp(m_ctx, name), "GetTimeStamp"); }

std::vector<std::pair<std::string, float>> EI_Device::GetTimeStamps() {
    const int maxCount = 256;
    std::vector<char> names(64 * maxCount);
    std::vector<float> ms(maxCount);
    int n = 0;
    tfxhost::check(tfx_context_timestamps(m_ctx, reinterpret_cast<char(*)[64]>(names.data()), ms.data(), maxCount, &n),
                   "GetTimeStamps");
    std::vector<std::pair<std::string, float>> out;
    for (int i = 0; i < n; ++i) out.emplace_back(std::string(&names[64 * i], strnlen(&names[64 * i], 64)), ms[i]);
    return out;
}

void EI_Device::WaitForCompute() { tfxhost::check(tfx_context_synchronize(m_ctx), "WaitForCompute"); }
