// The compute subset of the reference's Engine Interface (src/EngineInterface.h:23-31, 90-100,
// 253-259) that the simulation and SDF host classes use, backed by CUDA through the C ABI:
// EI_Device owns a tfx_context (device + stream), EI_CommandContext records on that stream,
// EI_Resource is a device buffer, GetTimeStamp records a CUDA event.
#pragma once

#include <cstdio>
#include <vector>
#include <string>
#include <utility>

#include "TressFXCommon.h"

// A device buffer: pointer and size, owned by the object that created it.
class EI_Resource {
public:
    EI_Resource() = default;
    EI_Resource(void* ptr, size_t bytes) : m_ptr(ptr), m_bytes(bytes) {}
    void* GetDevicePointer() const { return m_ptr; }
    size_t GetSizeInBytes() const { return m_bytes; }
private:
    void* m_ptr = nullptr;
    size_t m_bytes = 0;
};

class EI_Device {
public:
    explicit EI_Device(int cudaDevice = 0);
    ~EI_Device();
    EI_Device(const EI_Device&) = delete;
    EI_Device& operator=(const EI_Device&) = delete;

    // EI_Device::GetTimeStamp: a named event on the compute stream.
    void GetTimeStamp(const char* name);
    // The recorded timestamps as (name, milliseconds since the previous one); clears them.
    std::vector<std::pair<std::string, float>> GetTimeStamps();
    // Blocks until all recorded work has run.
    void WaitForCompute();
    tfx_context GetContext() const { return m_ctx; }
private:
    tfx_context m_ctx = nullptr;
};

// EI_CommandContext: work is recorded, in order, on the device's stream.
class EI_CommandContext {
public:
    explicit EI_CommandContext(EI_Device& device) : m_device(&device) {}
    EI_Device& GetDevice() const { return *m_device; }
    tfx_context GetContext() const { return m_device->GetContext(); }
private:
    EI_Device* m_device;
};

// The scene side of bone lookups (EI_Scene::GetBoneIdByName, used by the asset and collision-mesh
// loaders to map the file's bone names to the engine's skeleton indices).
class EI_Scene {
public:
    virtual ~EI_Scene() = default;
    virtual int GetBoneIdByName(int skinNumber, const char* boneName) = 0;
};

// EI_Read / EI_Seek of the reference's file loaders (EngineInterface.h): plain stdio.
inline size_t EI_Read(void* ptr, size_t size, FILE* f) { return std::fread(ptr, 1, size, f); }
inline int EI_Seek(FILE* f, long offset) { return std::fseek(f, offset, SEEK_SET); }
