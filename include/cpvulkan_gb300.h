/*
 * cpvulkan_gb300.h — the C ABI of libcpvulkan_gb300.so, the GB300 (sm_103a)
 * Vulkan ICD for the draw hot path.
 *
 * The drop-in boundary is the Vulkan loader ↔ ICD interface: the Khronos
 * loader (or any application acting as one) reads a manifest
 * (cpvulkan_gb300/CPVulkan.json) whose library_path names this library,
 * negotiates the interface version and resolves every Vulkan entry point
 * through vk_icdGetInstanceProcAddr / vkGetDeviceProcAddr. These three
 * exports replace the reference ICD's exports one for one.
 *
 * Dispatchable handles (VkInstance, VkPhysicalDevice, VkDevice, VkQueue,
 * VkCommandBuffer) point at objects whose first word is ICD_LOADER_MAGIC,
 * which a loader overwrites with its dispatch table pointer. Errors are
 * returned as VkResult values; nothing aborts and no kernel traps.
 */
#ifndef CPVULKAN_GB300_H
#define CPVULKAN_GB300_H

#include <stdint.h>

#include "cpv/vk_subset.h"

#if defined(__GNUC__)
#define CPV_EXPORT __attribute__((visibility("default")))
#else
#define CPV_EXPORT
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Clamps *pVersion to the highest loader interface version supported (5).
 * Replaces vk_icdNegotiateLoaderICDInterfaceVersion of the reference
 * (CPVulkan/CPVulkan.cpp:94-104). */
CPV_EXPORT VkResult VKAPI_CALL vk_icdNegotiateLoaderICDInterfaceVersion(uint32_t* pVersion);

/* Name → entry point for global, instance and device functions
 * (vkCreateInstance, vkCreateGraphicsPipelines, vkCmdBindVertexBuffers,
 * vkCmdDraw, vkCmdDrawIndexed, vkQueueSubmit, ...). Replaces
 * vk_icdGetInstanceProcAddr of the reference (CPVulkan/CPVulkan.cpp:14-87,
 * table CPVulkan/Extensions.cpp:170-300). */
CPV_EXPORT PFN_vkVoidFunction VKAPI_CALL vk_icdGetInstanceProcAddr(VkInstance instance, const char* pName);

/* Physical-device-level extension functions: none (returns NULL), as the
 * reference (CPVulkan/CPVulkan.cpp:89-92). */
CPV_EXPORT PFN_vkVoidFunction VKAPI_CALL vk_icdGetPhysicalDeviceProcAddr(VkInstance instance, const char* pName);

/* ---- diagnostics (no counterpart in the reference) ---- */

/* Last error message recorded on the calling thread (pipeline rejections,
 * NVRTC logs, CUDA errors). Never NULL. */
CPV_EXPORT const char* cpv_last_error(void);

/* Number of kernels this library has launched since load. */
CPV_EXPORT uint64_t cpv_kernel_launches(void);

/* 1 when a CUDA device can be used (creates the context), else 0. */
CPV_EXPORT int cpv_device_available(void);

/* Device-side timing on a queue's stream: records event `slot` (0..15) on
 * the queue; cpv_queue_elapsed_ms returns the time between two recorded
 * slots after synchronising on the later one (negative on error). */
CPV_EXPORT int cpv_queue_record(VkQueue queue, uint32_t slot);
CPV_EXPORT double cpv_queue_elapsed_ms(VkQueue queue, uint32_t slot_begin, uint32_t slot_end);

#ifdef __cplusplus
}
#endif

#endif /* CPVULKAN_GB300_H */
