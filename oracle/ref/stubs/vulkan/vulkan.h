// Declarations only, so that the reference's detector headers compile
// without a Vulkan SDK: the detector uses none of these at run time. Test
// infrastructure for oracle/ref/detector_shim.cpp.
#pragma once
#include <stdint.h>
#define VK_DEFINE_HANDLE(object) typedef struct object##_opaque* object;
#define VK_NULL_HANDLE nullptr
VK_DEFINE_HANDLE(VkInstance)
VK_DEFINE_HANDLE(VkPhysicalDevice)
VK_DEFINE_HANDLE(VkDevice)
VK_DEFINE_HANDLE(VkQueue)
VK_DEFINE_HANDLE(VkCommandBuffer)
VK_DEFINE_HANDLE(VkBuffer)
VK_DEFINE_HANDLE(VkCommandPool)
VK_DEFINE_HANDLE(VkDescriptorPool)
VK_DEFINE_HANDLE(VkDescriptorSetLayout)
VK_DEFINE_HANDLE(VkDescriptorSet)
VK_DEFINE_HANDLE(VkFence)
VK_DEFINE_HANDLE(VkPipeline)
VK_DEFINE_HANDLE(VkPipelineLayout)
VK_DEFINE_HANDLE(VkShaderModule)
VK_DEFINE_HANDLE(VkSemaphore)
VK_DEFINE_HANDLE(VkDeviceMemory)
VK_DEFINE_HANDLE(VkDebugUtilsMessengerEXT)
typedef uint64_t VkDeviceSize;
typedef uint32_t VkFlags;
typedef VkFlags VkBufferUsageFlags;
typedef enum VkResult { VK_SUCCESS = 0 } VkResult;
typedef enum VkPhysicalDeviceType { VK_PHYSICAL_DEVICE_TYPE_OTHER = 0 } VkPhysicalDeviceType;
typedef struct VkSubmitInfo { int unused; } VkSubmitInfo;
inline VkResult vkQueueSubmit(VkQueue, uint32_t, const VkSubmitInfo*, VkFence) { return VK_SUCCESS; }
