// Stands in for the reference's core/gpu/context.h when its detector is
// compiled as an oracle: the detector's headers only name gpu::Context (by
// pointer and reference) and hold a gpu::DeviceInfo, and the real header's
// defaulted Options argument does not compile with GCC 13. Test
// infrastructure for oracle/ref/detector_shim.cpp.
#pragma once
#include <cstdint>
#include <string>
#include <vulkan/vulkan.h>
#include "core/error.h"
VK_DEFINE_HANDLE(VmaAllocator)
namespace revenant::gpu {
struct DeviceInfo {
    std::uint32_t index = 0;
    std::string name;
};
class Context;
}  // namespace revenant::gpu
