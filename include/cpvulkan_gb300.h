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

/* The calling thread's last batch tuning (a render pass of many draws timed
 * under each tile size / warps-per-tile / batch / schedule candidate on its
 * first submission): each candidate's time and the choice, e.g. "tile 16
 * warps 8 schedule 2 batch 256: 65.4 ms; ...; chosen tile 16 warps 8
 * schedule 2 batch 256". Empty when no tuning ran. No reference
 * counterpart. */
CPV_EXPORT const char* cpv_batch_tuning(void);

/* Statistics of the most recent batched render pass that had completed when
 * the next batched pass was submitted: out[0] primitives, out[1] vertex
 * slots shaded by the vertex stage, out[2] (primitive, screen tile) pairs
 * binned. No reference counterpart. */
CPV_EXPORT void cpv_batch_stats(uint64_t out[3]);

/* 1 when a CUDA device can be used (creates the context), else 0. */
CPV_EXPORT int cpv_device_available(void);

/* Device-side timing on a queue's stream: records event `slot` (0..15) on
 * the queue; cpv_queue_elapsed_ms returns the time between two recorded
 * slots after synchronising on the later one (negative on error). */
CPV_EXPORT int cpv_queue_record(VkQueue queue, uint32_t slot);
CPV_EXPORT double cpv_queue_elapsed_ms(VkQueue queue, uint32_t slot_begin, uint32_t slot_end);

/* How many times the queue's grow-only binning scratch has been allocated
 * or regrown (cudaMalloc) since the queue was created; 0 for a queue that
 * only ever ran cpv_queue_submit_no_alloc. */
CPV_EXPORT uint64_t cpv_queue_scratch_generation(VkQueue queue);

/* Per-kernel device timing: while enabled, every kernel of the draw paths is
 * bracketed by CUDA events on its stream (batched render passes then run
 * without their CUDA graph). cpv_profile_get returns the launches and the
 * summed milliseconds recorded under `kernel` (e.g. "cpv_raster",
 * "cpv_batch_raster"); cpv_profile_reset clears the totals. */
CPV_EXPORT void cpv_profile_enable(int on);
CPV_EXPORT int cpv_profile_get(const char* kernel, uint64_t* launches, double* total_ms);
CPV_EXPORT void cpv_profile_reset(void);

/* ---- submission without allocation (no counterpart in the reference) ----
 *
 * Same signature and results as vkQueueSubmit, for callers that cannot
 * allocate device memory while submitting: a renderer working inside a fixed
 * device-memory budget that must not grow, or a submit thread that must not
 * stall, as cudaMalloc / cudaFree may synchronise the device. vkQueueSubmit
 * grows each queue's binning scratch with cudaMalloc the first time a draw
 * needs more of it; this variant bins every draw through one file-scope
 * 32 MiB device array instead, and allocates no device or pinned memory and
 * creates no CUDA objects (host-side bookkeeping of the submission is as in
 * vkQueueSubmit).
 *
 * - The first call on a device resolves the array's address
 *   (cudaGetSymbolAddress) with that device current; make that first call
 *   outside any stream capture, before relying on it.
 * - A draw needs 8 bytes per primitive for its tile rectangles plus its bins;
 *   a submission holding a draw that does not fit is rejected before any of
 *   its work is enqueued: VK_ERROR_OUT_OF_DEVICE_MEMORY, reason in
 *   cpv_last_error(). Draws of up to about 4 million primitives fit.
 *   Indirect draws are checked through their records as they stand at the
 *   call (read from host-visible memory, or from device memory after the
 *   queue's earlier work); a record that a command of the same submission
 *   rewrites is checked again when its draw runs, and one that no longer
 *   fits then ends the submission with VK_ERROR_OUT_OF_DEVICE_MEMORY after
 *   the commands before it were enqueued.
 * - The bin counters must start at zero for every draw; the call zeroes
 *   them on the queue's stream itself. Nothing else needs an initial value.
 * - The array is shared by every queue of the process on a device: calls
 *   whose work overlaps on the GPU (two queues, or two devices' queues on
 *   one GPU) race on it. Serialise them, e.g. wait for the fence of one
 *   before submitting on another queue. Successive calls on one queue are
 *   ordered by its stream and do not race. */
CPV_EXPORT VkResult VKAPI_CALL cpv_queue_submit_no_alloc(VkQueue queue, uint32_t submitCount, const VkSubmitInfo* pSubmits, VkFence fence);

#ifdef __cplusplus
}
#endif

#endif /* CPVULKAN_GB300_H */
