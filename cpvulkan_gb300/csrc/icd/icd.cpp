// icd.cpp — Vulkan entry points of the cpvulkan_gb300 ICD and the loader
// interface (vk_icdNegotiateLoaderICDInterfaceVersion,
// vk_icdGetInstanceProcAddr, vk_icdGetPhysicalDeviceProcAddr).
//
// Reference counterparts: CPVulkan/CPVulkan.cpp:14-104 (loader interface),
// CPVulkan/Extensions.cpp:170-300 (name → function table), and the object
// methods of CPVulkan/Instance.cpp, PhysicalDevice.cpp, Device.cpp,
// Buffer.cpp, Image.cpp, ... The hot-path entry points are
// vkCreateGraphicsPipelines (pipeline.cpp), vkCmdBindVertexBuffers,
// vkCmdDraw, vkCmdDrawIndexed (recording here) and vkQueueSubmit (here,
// executing through command.cpp).
#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <new>
#include <thread>
#include <unordered_map>

#include "../../../include/cpvulkan_gb300.h"
#include "icd.h"

namespace cpv::icd {

uint32_t format_texel_size(VkFormat f) {
    switch (f) {
    case VK_FORMAT_R8_UNORM: case VK_FORMAT_R8_UINT: case VK_FORMAT_R8_SINT: case VK_FORMAT_S8_UINT: return 1;
    case VK_FORMAT_R8G8_UNORM: case VK_FORMAT_R8G8_UINT: case VK_FORMAT_R8G8_SINT: case VK_FORMAT_D16_UNORM: case VK_FORMAT_R16_UNORM:
    case VK_FORMAT_R16_UINT: case VK_FORMAT_R16_SINT: case VK_FORMAT_R16_SFLOAT: return 2;
    case VK_FORMAT_D16_UNORM_S8_UINT: return 3;
    case VK_FORMAT_R8G8B8A8_UNORM: case VK_FORMAT_R8G8B8A8_SNORM: case VK_FORMAT_R8G8B8A8_UINT: case VK_FORMAT_R8G8B8A8_SINT:
    case VK_FORMAT_R8G8B8A8_SRGB: case VK_FORMAT_B8G8R8A8_UNORM: case VK_FORMAT_B8G8R8A8_SRGB: case VK_FORMAT_R32_UINT:
    case VK_FORMAT_R32_SINT: case VK_FORMAT_R32_SFLOAT: case VK_FORMAT_D32_SFLOAT: case VK_FORMAT_X8_D24_UNORM_PACK32:
    case VK_FORMAT_D24_UNORM_S8_UINT: case VK_FORMAT_R16G16_UNORM: case VK_FORMAT_R16G16_SFLOAT: case VK_FORMAT_R16G16_UINT:
    case VK_FORMAT_R16G16_SINT:
        return 4;
    case VK_FORMAT_R32G32_UINT: case VK_FORMAT_R32G32_SINT: case VK_FORMAT_R32G32_SFLOAT: case VK_FORMAT_D32_SFLOAT_S8_UINT:
    case VK_FORMAT_R16G16B16A16_UNORM: case VK_FORMAT_R16G16B16A16_UINT: case VK_FORMAT_R16G16B16A16_SINT: case VK_FORMAT_R16G16B16A16_SFLOAT: return 8;
    case VK_FORMAT_R32G32B32_UINT: case VK_FORMAT_R32G32B32_SINT: case VK_FORMAT_R32G32B32_SFLOAT: return 12;
    case VK_FORMAT_R32G32B32A32_UINT: case VK_FORMAT_R32G32B32A32_SINT: case VK_FORMAT_R32G32B32A32_SFLOAT: return 16;
    default: return 0;
    }
}

bool colour_layout(VkFormat f, ColourLayout& out) {
    switch (f) {
    case VK_FORMAT_R8G8B8A8_UNORM: out = {4, 4, 8, 0, false}; return true;
    case VK_FORMAT_B8G8R8A8_UNORM: out = {4, 4, 8, 0, true}; return true;
    case VK_FORMAT_R8_UNORM: out = {1, 1, 8, 0, false}; return true;
    case VK_FORMAT_R8G8_UNORM: out = {2, 2, 8, 0, false}; return true;
    case VK_FORMAT_R8G8B8A8_SNORM: out = {4, 4, 8, 1, false}; return true;
    case VK_FORMAT_R16_UNORM: out = {2, 1, 16, 0, false}; return true;
    case VK_FORMAT_R16G16_UNORM: out = {4, 2, 16, 0, false}; return true;
    case VK_FORMAT_R16G16_SFLOAT: out = {4, 2, 16, 2, false}; return true;
    case VK_FORMAT_R32_SFLOAT: out = {4, 1, 32, 2, false}; return true;
    // integer formats (kind 3 UINT, 4 SINT): the shader output's bits,
    // clamped to the channel's range (LLVMRuntime/ImageCompiler.cpp:1121-1175)
    case VK_FORMAT_R8_UINT: out = {1, 1, 8, 3, false}; return true;
    case VK_FORMAT_R8_SINT: out = {1, 1, 8, 4, false}; return true;
    case VK_FORMAT_R8G8_UINT: out = {2, 2, 8, 3, false}; return true;
    case VK_FORMAT_R8G8_SINT: out = {2, 2, 8, 4, false}; return true;
    case VK_FORMAT_R8G8B8A8_UINT: out = {4, 4, 8, 3, false}; return true;
    case VK_FORMAT_R8G8B8A8_SINT: out = {4, 4, 8, 4, false}; return true;
    case VK_FORMAT_R16_UINT: out = {2, 1, 16, 3, false}; return true;
    case VK_FORMAT_R16_SINT: out = {2, 1, 16, 4, false}; return true;
    case VK_FORMAT_R16G16_UINT: out = {4, 2, 16, 3, false}; return true;
    case VK_FORMAT_R16G16_SINT: out = {4, 2, 16, 4, false}; return true;
    case VK_FORMAT_R32_UINT: out = {4, 1, 32, 3, false}; return true;
    case VK_FORMAT_R32_SINT: out = {4, 1, 32, 4, false}; return true;
    // 8- and 16-byte texels: channel i in 32-bit word i * bits / 32
    case VK_FORMAT_R16G16B16A16_UNORM: out = {8, 4, 16, 0, false}; return true;
    case VK_FORMAT_R16G16B16A16_SFLOAT: out = {8, 4, 16, 2, false}; return true;
    case VK_FORMAT_R16G16B16A16_UINT: out = {8, 4, 16, 3, false}; return true;
    case VK_FORMAT_R16G16B16A16_SINT: out = {8, 4, 16, 4, false}; return true;
    case VK_FORMAT_R32G32_SFLOAT: out = {8, 2, 32, 2, false}; return true;
    case VK_FORMAT_R32G32_UINT: out = {8, 2, 32, 3, false}; return true;
    case VK_FORMAT_R32G32_SINT: out = {8, 2, 32, 4, false}; return true;
    case VK_FORMAT_R32G32B32A32_SFLOAT: out = {16, 4, 32, 2, false}; return true;
    case VK_FORMAT_R32G32B32A32_UINT: out = {16, 4, 32, 3, false}; return true;
    case VK_FORMAT_R32G32B32A32_SINT: out = {16, 4, 32, 4, false}; return true;
    default: return false;
    }
}

bool format_is_depth(VkFormat f) {
    return f == VK_FORMAT_D16_UNORM || f == VK_FORMAT_D32_SFLOAT || f == VK_FORMAT_D32_SFLOAT_S8_UINT || f == VK_FORMAT_S8_UINT ||
           f == VK_FORMAT_D16_UNORM_S8_UINT || f == VK_FORMAT_D24_UNORM_S8_UINT || f == VK_FORMAT_X8_D24_UNORM_PACK32;
}

bool format_has_stencil(VkFormat f) {
    return f == VK_FORMAT_D32_SFLOAT_S8_UINT || f == VK_FORMAT_S8_UINT || f == VK_FORMAT_D16_UNORM_S8_UINT || f == VK_FORMAT_D24_UNORM_S8_UINT;
}

// GetNormalImageSize (CPVulkanBase/Formats.cpp:453-484).
void image_layout(Image& img) {
    img.level.assign(img.levels, ImageLevel{});
    uint32_t w = img.extent.width, h = img.extent.height, d = img.extent.depth;
    uint64_t layer = 0;
    for (uint32_t i = 0; i < img.levels; i++) {
        ImageLevel& L = img.level[i];
        L.offset = layer;
        L.width = w;
        L.height = h;
        L.depth = d;
        L.stride = static_cast<uint64_t>(img.texel) * w;
        L.plane = L.stride * h;
        L.size = L.plane * d;
        layer += L.size;
        w = std::max(w / 2, 1u);
        h = std::max(h / 2, 1u);
        d = std::max(d / 2, 1u);
    }
    img.layer_size = layer;
    img.total_size = layer * img.layers;
}

namespace {

template <typename T>
T* from(uint64_t h) { return reinterpret_cast<T*>(static_cast<uintptr_t>(h)); }

template <typename H, typename T>
H to_handle(T* p) { return reinterpret_cast<H>(p); }

constexpr uint32_t kMemoryTypeHostVisible = 0;  // DEVICE_LOCAL | HOST_VISIBLE | HOST_COHERENT (the reference's only type)
constexpr uint32_t kMemoryTypeDeviceOnly = 1;   // DEVICE_LOCAL

std::mutex g_instance_mutex;

// Host objects live in the application's allocator when it passes one, as
// the reference's Allocate / Free do (CPVulkanBase/Base.h:256-294), else on
// the ICD's heap; a destroy call passes the allocator its create call did.
// (Pipelines, queues, command buffers and descriptor sets always use the
// ICD's heap: the latter three belong to their device or pool.)
template <typename T>
T* host_new(const VkAllocationCallbacks* alloc, int scope) {
    if (!alloc || !alloc->pfnAllocation) return new T();
    void* p = alloc->pfnAllocation(alloc->pUserData, sizeof(T), alignof(T) < 16 ? 16 : alignof(T), scope);
    return p ? new (p) T() : nullptr;
}
template <typename T>
void host_delete(T* t, const VkAllocationCallbacks* alloc) {
    if (!t) return;
    if (!alloc || !alloc->pfnFree) {
        delete t;
        return;
    }
    t->~T();
    alloc->pfnFree(alloc->pUserData, t);
}
constexpr int kScopeObject = 1, kScopeDevice = 3, kScopeInstance = 4;  // VkSystemAllocationScope

// ---------------------------------------------------------------- instance --

VKAPI_ATTR VkResult VKAPI_CALL CreateInstance(const VkInstanceCreateInfo* ci, const VkAllocationCallbacks* alloc, VkInstance* out) {
    if (!ci || !out) return VK_ERROR_INITIALIZATION_FAILED;
    for (uint32_t i = 0; i < ci->enabledExtensionCount; i++) return VK_ERROR_EXTENSION_NOT_PRESENT;
    auto* inst = host_new<Instance>(alloc, kScopeInstance);
    if (!inst) return VK_ERROR_OUT_OF_HOST_MEMORY;
    inst->physical = new PhysicalDevice();
    inst->physical->instance = inst;
    if (ci->pApplicationInfo && ci->pApplicationInfo->apiVersion) inst->api_version = ci->pApplicationInfo->apiVersion;
    *out = to_handle<VkInstance>(inst);
    return VK_SUCCESS;
}

VKAPI_ATTR void VKAPI_CALL DestroyInstance(VkInstance instance, const VkAllocationCallbacks* alloc) {
    auto* inst = reinterpret_cast<Instance*>(instance);
    if (!inst) return;
    delete inst->physical;
    host_delete(inst, alloc);
}

VKAPI_ATTR VkResult VKAPI_CALL EnumerateInstanceExtensionProperties(const char*, uint32_t* count, VkExtensionProperties*) {
    *count = 0;
    return VK_SUCCESS;
}

VKAPI_ATTR VkResult VKAPI_CALL EnumerateInstanceVersion(uint32_t* v) {
    *v = VK_API_VERSION_1_1 | 121;
    return VK_SUCCESS;
}

VKAPI_ATTR VkResult VKAPI_CALL EnumeratePhysicalDevices(VkInstance instance, uint32_t* count, VkPhysicalDevice* out) {
    auto* inst = reinterpret_cast<Instance*>(instance);
    if (!out) {
        *count = 1;
        return VK_SUCCESS;
    }
    if (*count < 1) return VK_INCOMPLETE;
    out[0] = to_handle<VkPhysicalDevice>(inst->physical);
    *count = 1;
    return VK_SUCCESS;
}

VKAPI_ATTR void VKAPI_CALL GetPhysicalDeviceProperties(VkPhysicalDevice, VkPhysicalDeviceProperties* p) {
    std::memset(p, 0, sizeof(*p));
    p->apiVersion = VK_API_VERSION_1_1 | 121;
    p->driverVersion = VK_MAKE_VERSION(0, 1, 0);
    p->vendorID = 0x10DE;
    p->deviceID = 0x0103;
    p->deviceType = VK_PHYSICAL_DEVICE_TYPE_DISCRETE_GPU;
    std::snprintf(p->deviceName, sizeof(p->deviceName), "cpvulkan_gb300 (sm_103a)");
    const char uuid[16] = {'c', 'p', 'v', 'g', 'b', '3', '0', '0', 'p', 'i', 'p', 'e', 'v', '1', 0, 0};
    std::memcpy(p->pipelineCacheUUID, uuid, 16);
    auto& l = p->limits;
    l.maxImageDimension1D = 16384;
    l.maxImageDimension2D = 16384;
    l.maxImageDimension3D = 2048;
    l.maxImageDimensionCube = 16384;
    l.maxImageArrayLayers = 2048;
    l.maxTexelBufferElements = 1u << 27;
    l.maxUniformBufferRange = 65536;
    l.maxStorageBufferRange = 1u << 30;
    l.maxPushConstantsSize = 128;
    l.maxMemoryAllocationCount = 1u << 20;
    l.maxSamplerAllocationCount = 1u << 20;
    l.bufferImageGranularity = 1;
    l.maxBoundDescriptorSets = 8;
    l.maxPerStageDescriptorSamplers = 4;
    l.maxPerStageDescriptorUniformBuffers = 8;
    l.maxPerStageDescriptorSampledImages = 4;
    l.maxPerStageResources = 16;
    l.maxDescriptorSetSamplers = 4;
    l.maxDescriptorSetUniformBuffers = 8;
    l.maxDescriptorSetUniformBuffersDynamic = 8;
    l.maxDescriptorSetSampledImages = 4;
    l.maxVertexInputAttributes = 16;
    l.maxVertexInputBindings = 8;
    l.maxVertexInputAttributeOffset = 2047;
    l.maxVertexInputBindingStride = 2048;
    l.maxVertexOutputComponents = 64;
    l.maxFragmentInputComponents = 64;
    l.maxFragmentOutputAttachments = 1;
    l.maxFragmentCombinedOutputResources = 1;
    l.maxComputeWorkGroupCount[0] = l.maxComputeWorkGroupCount[1] = l.maxComputeWorkGroupCount[2] = 65535;
    l.subPixelPrecisionBits = 4;  // advertised as the reference does (CPVulkanBase/Config.h:151); coverage is float
    l.subTexelPrecisionBits = 4;
    l.mipmapPrecisionBits = 4;
    l.maxDrawIndexedIndexValue = 0xFFFFFFFFu;
    l.maxDrawIndirectCount = 1;
    l.maxSamplerLodBias = 32.0f;
    l.maxSamplerAnisotropy = 1.0f;
    l.maxViewports = 1;
    l.maxViewportDimensions[0] = l.maxViewportDimensions[1] = 16384;
    l.viewportBoundsRange[0] = -32768.0f;
    l.viewportBoundsRange[1] = 32767.0f;
    l.minMemoryMapAlignment = 64;
    l.minTexelBufferOffsetAlignment = 16;
    l.minUniformBufferOffsetAlignment = 16;
    l.minStorageBufferOffsetAlignment = 16;
    l.maxFramebufferWidth = 16384;
    l.maxFramebufferHeight = 16384;
    l.maxFramebufferLayers = 1;
    l.framebufferColorSampleCounts = l.framebufferDepthSampleCounts = l.framebufferStencilSampleCounts = 1;
    l.framebufferNoAttachmentsSampleCounts = 1;
    l.maxColorAttachments = 1;
    l.sampledImageColorSampleCounts = l.sampledImageIntegerSampleCounts = l.sampledImageDepthSampleCounts = 1;
    l.sampledImageStencilSampleCounts = l.storageImageSampleCounts = 1;
    l.maxSampleMaskWords = 1;
    l.timestampPeriod = 1.0f;
    l.discreteQueuePriorities = 2;
    l.pointSizeRange[0] = l.pointSizeRange[1] = 1.0f;
    l.lineWidthRange[0] = l.lineWidthRange[1] = 1.0f;
    l.optimalBufferCopyOffsetAlignment = 16;
    l.optimalBufferCopyRowPitchAlignment = 16;
    l.nonCoherentAtomSize = 64;
}

VKAPI_ATTR void VKAPI_CALL GetPhysicalDeviceFeatures(VkPhysicalDevice, VkPhysicalDeviceFeatures* f) {
    std::memset(f, 0, sizeof(*f));
    f->fullDrawIndexUint32 = VK_TRUE;
}

VKAPI_ATTR void VKAPI_CALL GetPhysicalDeviceMemoryProperties(VkPhysicalDevice, VkPhysicalDeviceMemoryProperties* m) {
    std::memset(m, 0, sizeof(*m));
    m->memoryTypeCount = 2;
    m->memoryTypes[kMemoryTypeHostVisible].propertyFlags =
        VK_MEMORY_PROPERTY_DEVICE_LOCAL_BIT | VK_MEMORY_PROPERTY_HOST_VISIBLE_BIT | VK_MEMORY_PROPERTY_HOST_COHERENT_BIT;
    m->memoryTypes[kMemoryTypeHostVisible].heapIndex = 0;
    m->memoryTypes[kMemoryTypeDeviceOnly].propertyFlags = VK_MEMORY_PROPERTY_DEVICE_LOCAL_BIT;
    m->memoryTypes[kMemoryTypeDeviceOnly].heapIndex = 0;
    m->memoryHeapCount = 1;
    size_t free_b = 0, total_b = 0;
    if (rt::available() && cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) m->memoryHeaps[0].size = total_b;
    else m->memoryHeaps[0].size = 256ull << 30;
    m->memoryHeaps[0].flags = VK_MEMORY_HEAP_DEVICE_LOCAL_BIT;
}

VKAPI_ATTR void VKAPI_CALL GetPhysicalDeviceQueueFamilyProperties(VkPhysicalDevice, uint32_t* count, VkQueueFamilyProperties* p) {
    if (!p) {
        *count = 1;
        return;
    }
    if (*count < 1) return;
    std::memset(p, 0, sizeof(*p));
    p[0].queueFlags = VK_QUEUE_GRAPHICS_BIT | VK_QUEUE_TRANSFER_BIT;
    p[0].queueCount = kMaxQueues;
    p[0].timestampValidBits = 0;
    p[0].minImageTransferGranularity = {1, 1, 1};
    *count = 1;
}

VKAPI_ATTR void VKAPI_CALL GetPhysicalDeviceFormatProperties(VkPhysicalDevice, VkFormat f, VkFormatProperties* p) {
    std::memset(p, 0, sizeof(*p));
    const uint32_t size = format_texel_size(f);
    ColourLayout cl;
    if (f != VK_FORMAT_R8G8B8A8_UNORM && f != VK_FORMAT_B8G8R8A8_UNORM && colour_layout(f, cl)) {
        // colour attachments of the draw path (blending too: the blend is
        // computed in float and encoded to the format)
        p->linearTilingFeatures = p->optimalTilingFeatures = VK_FORMAT_FEATURE_COLOR_ATTACHMENT_BIT | VK_FORMAT_FEATURE_COLOR_ATTACHMENT_BLEND_BIT |
                                                             VK_FORMAT_FEATURE_TRANSFER_SRC_BIT | VK_FORMAT_FEATURE_TRANSFER_DST_BIT;
        if (cl.kind >= 3) {  // integer formats are not blended
            p->linearTilingFeatures &= ~VK_FORMAT_FEATURE_COLOR_ATTACHMENT_BLEND_BIT;
            p->optimalTilingFeatures &= ~VK_FORMAT_FEATURE_COLOR_ATTACHMENT_BLEND_BIT;
        }
    }
    if (f == VK_FORMAT_R8G8B8A8_UNORM || f == VK_FORMAT_B8G8R8A8_UNORM) {
        p->linearTilingFeatures = p->optimalTilingFeatures = VK_FORMAT_FEATURE_SAMPLED_IMAGE_BIT | VK_FORMAT_FEATURE_COLOR_ATTACHMENT_BIT |
                                                             VK_FORMAT_FEATURE_COLOR_ATTACHMENT_BLEND_BIT | VK_FORMAT_FEATURE_TRANSFER_SRC_BIT |
                                                             VK_FORMAT_FEATURE_TRANSFER_DST_BIT | VK_FORMAT_FEATURE_SAMPLED_IMAGE_FILTER_LINEAR_BIT;
        if (f == VK_FORMAT_B8G8R8A8_UNORM) p->linearTilingFeatures &= ~VK_FORMAT_FEATURE_SAMPLED_IMAGE_BIT;
        if (f == VK_FORMAT_B8G8R8A8_UNORM) p->optimalTilingFeatures &= ~(VK_FORMAT_FEATURE_SAMPLED_IMAGE_BIT | VK_FORMAT_FEATURE_SAMPLED_IMAGE_FILTER_LINEAR_BIT);
        if (f == VK_FORMAT_B8G8R8A8_UNORM) p->linearTilingFeatures &= ~VK_FORMAT_FEATURE_SAMPLED_IMAGE_FILTER_LINEAR_BIT;
        if (f == VK_FORMAT_R8G8B8A8_UNORM) p->bufferFeatures = VK_FORMAT_FEATURE_VERTEX_BUFFER_BIT;
    } else if (f == VK_FORMAT_D16_UNORM || f == VK_FORMAT_D32_SFLOAT || f == VK_FORMAT_D32_SFLOAT_S8_UINT) {
        p->optimalTilingFeatures = p->linearTilingFeatures =
            VK_FORMAT_FEATURE_DEPTH_STENCIL_ATTACHMENT_BIT | VK_FORMAT_FEATURE_TRANSFER_SRC_BIT | VK_FORMAT_FEATURE_TRANSFER_DST_BIT;
    } else if (size && (f == VK_FORMAT_R32_SFLOAT || f == VK_FORMAT_R32G32_SFLOAT || f == VK_FORMAT_R32G32B32_SFLOAT || f == VK_FORMAT_R32G32B32A32_SFLOAT ||
                        f == VK_FORMAT_R32_UINT || f == VK_FORMAT_R32G32_UINT || f == VK_FORMAT_R32G32B32_UINT || f == VK_FORMAT_R32G32B32A32_UINT ||
                        f == VK_FORMAT_R32_SINT || f == VK_FORMAT_R32G32_SINT || f == VK_FORMAT_R32G32B32_SINT || f == VK_FORMAT_R32G32B32A32_SINT)) {
        p->bufferFeatures = VK_FORMAT_FEATURE_VERTEX_BUFFER_BIT;
    }
}

// The device extensions (with their specification versions): the
// indirect-count draws, as the reference registers them
// (CPVulkan/Extensions.cpp:764-773, 1030-1038).
const struct {
    const char* name;
    uint32_t version;
} kDeviceExtensions[] = {{"VK_KHR_draw_indirect_count", 1}, {"VK_AMD_draw_indirect_count", 2}};

VKAPI_ATTR VkResult VKAPI_CALL EnumerateDeviceExtensionProperties(VkPhysicalDevice, const char* layer, uint32_t* count, VkExtensionProperties* props) {
    if (!count) return VK_INCOMPLETE;
    const uint32_t n = layer ? 0u : static_cast<uint32_t>(sizeof(kDeviceExtensions) / sizeof(kDeviceExtensions[0]));
    if (!props) {
        *count = n;
        return VK_SUCCESS;
    }
    const uint32_t written = std::min(*count, n);
    for (uint32_t i = 0; i < written; i++) {
        std::memset(&props[i], 0, sizeof(props[i]));
        std::strncpy(props[i].extensionName, kDeviceExtensions[i].name, VK_MAX_EXTENSION_NAME_SIZE - 1);
        props[i].specVersion = kDeviceExtensions[i].version;
    }
    *count = written;
    return written < n ? VK_INCOMPLETE : VK_SUCCESS;
}

// ------------------------------------------------------------------ device --

VKAPI_ATTR VkResult VKAPI_CALL CreateDevice(VkPhysicalDevice pd, const VkDeviceCreateInfo* ci, const VkAllocationCallbacks* alloc, VkDevice* out) {
    if (!ci || !out) return VK_ERROR_INITIALIZATION_FAILED;
    for (uint32_t i = 0; i < ci->enabledExtensionCount; i++) {
        bool known = false;
        for (const auto& e : kDeviceExtensions) known = known || (ci->ppEnabledExtensionNames[i] && std::strcmp(ci->ppEnabledExtensionNames[i], e.name) == 0);
        if (!known) return VK_ERROR_EXTENSION_NOT_PRESENT;
    }
    std::string err;
    const char* co = std::getenv("CPV_COMPILE_ONLY");
    const bool compile_only = co && co[0] == '1';
    if (rt::init(err) != rt::kOk && !compile_only) {
        rt::set_last_error("vkCreateDevice: " + err);
        return VK_ERROR_INITIALIZATION_FAILED;
    }
    // One queue family; each queue is its own CUDA stream with its own
    // binning scratch, so work submitted to different queues overlaps.
    uint32_t queues = 1;
    if (ci->queueCreateInfoCount >= 1 && ci->pQueueCreateInfos) queues = ci->pQueueCreateInfos[0].queueCount;
    if (queues < 1 || queues > kMaxQueues) return VK_ERROR_INITIALIZATION_FAILED;
    auto* dev = host_new<Device>(alloc, kScopeDevice);
    if (!dev) return VK_ERROR_OUT_OF_HOST_MEMORY;
    dev->physical = reinterpret_cast<PhysicalDevice*>(pd);
    dev->compile_only = !rt::available();
    for (uint32_t i = 0; i < queues; i++) {
        auto* q = new Queue();
        q->device = dev;
        dev->queues.push_back(q);
        if (!dev->compile_only && cudaStreamCreateWithFlags(&q->stream, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            for (Queue* x : dev->queues) {
                if (x->stream) cudaStreamDestroy(x->stream);
                delete x;
            }
            host_delete(dev, alloc);
            return VK_ERROR_INITIALIZATION_FAILED;
        }
    }
    dev->queue = dev->queues[0];
    *out = to_handle<VkDevice>(dev);
    return VK_SUCCESS;
}

VKAPI_ATTR void VKAPI_CALL DestroyDevice(VkDevice device, const VkAllocationCallbacks* alloc) {
    auto* dev = reinterpret_cast<Device*>(device);
    if (!dev) return;
    if (!dev->compile_only) {
        for (Queue* q : dev->queues) {
            cudaStreamSynchronize(q->stream);
            cudaStreamDestroy(q->stream);
        }
        for (auto& kv : dev->batch_modules) rt::unload(*kv.second);
    }
    for (Queue* q : dev->queues) delete q;
    host_delete(dev, alloc);
}

VKAPI_ATTR void VKAPI_CALL GetDeviceQueue(VkDevice device, uint32_t, uint32_t index, VkQueue* q) {
    auto* dev = reinterpret_cast<Device*>(device);
    *q = to_handle<VkQueue>(dev->queues[index < dev->queues.size() ? index : 0]);
}

// Waits for the work of every queue of the device (memory coherence points).
void sync_queues(Device* dev) {
    for (Queue* q : dev->queues) cudaStreamSynchronize(q->stream);
}

// Completion of a submission: host-visible memories the GPU wrote and that
// are mapped get their mirror refreshed (coherent memory semantics).
void complete_readback(std::vector<DeviceMemory*>& mems) {
    for (DeviceMemory* m : mems) {
        if (!m || !m->host) continue;
        m->device_dirty = true;
        if (m->mapped) {
            cudaMemcpy(m->host, m->device, m->size, cudaMemcpyDeviceToHost);
            m->device_dirty = false;
        }
    }
    mems.clear();
}

VKAPI_ATTR VkResult VKAPI_CALL DeviceWaitIdle(VkDevice device) {
    auto* dev = reinterpret_cast<Device*>(device);
    if (dev->compile_only) return VK_SUCCESS;
    for (Queue* q : dev->queues) {
        std::lock_guard<std::mutex> lock(q->mutex);
        if (cudaStreamSynchronize(q->stream) != cudaSuccess) return VK_ERROR_DEVICE_LOST;
        complete_readback(q->pending_readback);
    }
    return VK_SUCCESS;
}

VKAPI_ATTR VkResult VKAPI_CALL QueueWaitIdle(VkQueue queue) {
    auto* q = reinterpret_cast<Queue*>(queue);
    std::lock_guard<std::mutex> lock(q->mutex);
    if (cudaStreamSynchronize(q->stream) != cudaSuccess) return VK_ERROR_DEVICE_LOST;
    complete_readback(q->pending_readback);
    return VK_SUCCESS;
}

// ------------------------------------------------------------------ memory --

VKAPI_ATTR VkResult VKAPI_CALL AllocateMemory(VkDevice device, const VkMemoryAllocateInfo* ai, const VkAllocationCallbacks* alloc, VkDeviceMemory* out) {
    auto* dev = reinterpret_cast<Device*>(device);
    if (ai->memoryTypeIndex > kMemoryTypeDeviceOnly) return VK_ERROR_OUT_OF_DEVICE_MEMORY;
    auto* m = host_new<DeviceMemory>(alloc, kScopeObject);
    if (!m) return VK_ERROR_OUT_OF_HOST_MEMORY;
    m->size = ai->allocationSize;
    m->type = ai->memoryTypeIndex;
    const size_t bytes = m->size ? m->size : 1;
    if (dev->compile_only) {
        m->device = static_cast<uint8_t*>(std::calloc(bytes, 1));
        if (m->type == kMemoryTypeHostVisible) m->host = static_cast<uint8_t*>(std::calloc(bytes, 1));
        std::lock_guard<std::mutex> lock(dev->memory_mutex);
        dev->memories.insert(m);
        *out = to_handle<VkDeviceMemory>(m);
        return VK_SUCCESS;
    }
    if (cudaMalloc(reinterpret_cast<void**>(&m->device), bytes) != cudaSuccess) {
        cudaGetLastError();
        host_delete(m, alloc);
        return VK_ERROR_OUT_OF_DEVICE_MEMORY;
    }
    if (m->type == kMemoryTypeHostVisible) {
        if (cudaMallocHost(reinterpret_cast<void**>(&m->host), bytes) != cudaSuccess) {
            cudaGetLastError();
            cudaFree(m->device);
            host_delete(m, alloc);
            return VK_ERROR_OUT_OF_HOST_MEMORY;
        }
        std::memset(m->host, 0, bytes);
    }
    {
        std::lock_guard<std::mutex> lock(dev->memory_mutex);
        dev->memories.insert(m);
    }
    *out = to_handle<VkDeviceMemory>(m);
    return VK_SUCCESS;
}

VKAPI_ATTR void VKAPI_CALL FreeMemory(VkDevice device, VkDeviceMemory memory, const VkAllocationCallbacks* alloc) {
    auto* dev = reinterpret_cast<Device*>(device);
    auto* m = reinterpret_cast<DeviceMemory*>(memory);
    if (!m) return;
    if (!dev->compile_only) sync_queues(dev);
    {
        std::lock_guard<std::mutex> lock(dev->memory_mutex);
        dev->memories.erase(m);
    }
    for (Queue* q : dev->queues) {
        auto& pr = q->pending_readback;
        pr.erase(std::remove(pr.begin(), pr.end(), m), pr.end());
    }
    if (dev->compile_only) {
        std::free(m->device);
        std::free(m->host);
        host_delete(m, alloc);
        return;
    }
    cudaFree(m->device);
    if (m->host) cudaFreeHost(m->host);
    host_delete(m, alloc);
}

VKAPI_ATTR VkResult VKAPI_CALL MapMemory(VkDevice device, VkDeviceMemory memory, VkDeviceSize offset, VkDeviceSize, VkMemoryMapFlags, void** data) {
    auto* dev = reinterpret_cast<Device*>(device);
    auto* m = reinterpret_cast<DeviceMemory*>(memory);
    if (!m->host) return VK_ERROR_MEMORY_MAP_FAILED;
    if (dev->compile_only) {
        m->mapped = true;
        *data = m->host + offset;
        return VK_SUCCESS;
    }
    if (m->device_dirty) {
        sync_queues(dev);
        if (cudaMemcpy(m->host, m->device, m->size, cudaMemcpyDeviceToHost) != cudaSuccess) return VK_ERROR_MEMORY_MAP_FAILED;
        m->device_dirty = false;
    }
    m->mapped = true;
    *data = m->host + offset;
    return VK_SUCCESS;
}

VKAPI_ATTR void VKAPI_CALL UnmapMemory(VkDevice device, VkDeviceMemory memory) {
    auto* dev = reinterpret_cast<Device*>(device);
    auto* m = reinterpret_cast<DeviceMemory*>(memory);
    if (!m->host || !m->mapped) return;
    if (dev->compile_only) {
        m->mapped = false;
        return;
    }
    // The host's writes reach HBM before the call returns, copied by the SMs
    // over the chip-to-chip link (2.05 GB of mesh data: 12 ms, against 29 ms
    // for cudaMemcpy on the same machine).
    sync_queues(dev);
    cudaStream_t s = dev->queues.empty() ? nullptr : dev->queues[0]->stream;
    if (rt::copy_host_to_device(s, m->device, m->host, m->size) != rt::kOk)
        cudaMemcpy(m->device, m->host, m->size, cudaMemcpyHostToDevice);
    cudaStreamSynchronize(s);
    m->mapped = false;
}

VKAPI_ATTR VkResult VKAPI_CALL FlushMappedMemoryRanges(VkDevice device, uint32_t n, const VkMappedMemoryRange* r) {
    auto* dev = reinterpret_cast<Device*>(device);
    if (!dev->compile_only) sync_queues(dev);
    for (uint32_t i = 0; i < n; i++) {
        auto* m = reinterpret_cast<DeviceMemory*>(r[i].memory);
        if (!m->host) continue;
        const VkDeviceSize size = r[i].size == VK_WHOLE_SIZE ? m->size - r[i].offset : r[i].size;
        if (dev->compile_only || dev->queues.empty()) {
            if (cudaMemcpy(m->device + r[i].offset, m->host + r[i].offset, size, cudaMemcpyHostToDevice) != cudaSuccess) return VK_ERROR_OUT_OF_DEVICE_MEMORY;
            continue;
        }
        cudaStream_t s = dev->queues[0]->stream;
        if (rt::copy_host_to_device(s, m->device + r[i].offset, m->host + r[i].offset, size) != rt::kOk || cudaStreamSynchronize(s) != cudaSuccess)
            return VK_ERROR_OUT_OF_DEVICE_MEMORY;
    }
    return VK_SUCCESS;
}

VKAPI_ATTR VkResult VKAPI_CALL InvalidateMappedMemoryRanges(VkDevice device, uint32_t n, const VkMappedMemoryRange* r) {
    auto* dev = reinterpret_cast<Device*>(device);
    if (!dev->compile_only) sync_queues(dev);
    for (uint32_t i = 0; i < n; i++) {
        auto* m = reinterpret_cast<DeviceMemory*>(r[i].memory);
        if (!m->host) continue;
        const VkDeviceSize size = r[i].size == VK_WHOLE_SIZE ? m->size - r[i].offset : r[i].size;
        if (cudaMemcpy(m->host + r[i].offset, m->device + r[i].offset, size, cudaMemcpyDeviceToHost) != cudaSuccess) return VK_ERROR_OUT_OF_DEVICE_MEMORY;
    }
    return VK_SUCCESS;
}

// --------------------------------------------------------- buffers, images --

VKAPI_ATTR VkResult VKAPI_CALL CreateBuffer(VkDevice, const VkBufferCreateInfo* ci, const VkAllocationCallbacks* alloc, VkBuffer* out) {
    auto* b = host_new<Buffer>(alloc, kScopeObject);
    if (!b) return VK_ERROR_OUT_OF_HOST_MEMORY;
    b->size = ci->size;
    b->usage = ci->usage;
    *out = to_handle<VkBuffer>(b);
    return VK_SUCCESS;
}
VKAPI_ATTR void VKAPI_CALL DestroyBuffer(VkDevice, VkBuffer b, const VkAllocationCallbacks* alloc) { host_delete(reinterpret_cast<Buffer*>(b), alloc); }
VKAPI_ATTR void VKAPI_CALL GetBufferMemoryRequirements(VkDevice, VkBuffer buffer, VkMemoryRequirements* r) {
    auto* b = reinterpret_cast<Buffer*>(buffer);
    r->size = (b->size + 255) & ~255ull;
    r->alignment = 256;
    r->memoryTypeBits = 0x3;
}
VKAPI_ATTR VkResult VKAPI_CALL BindBufferMemory(VkDevice, VkBuffer buffer, VkDeviceMemory memory, VkDeviceSize offset) {
    auto* b = reinterpret_cast<Buffer*>(buffer);
    auto* m = reinterpret_cast<DeviceMemory*>(memory);
    if (offset + b->size > m->size) return VK_ERROR_OUT_OF_DEVICE_MEMORY;
    b->memory = m;
    b->offset = offset;
    return VK_SUCCESS;
}

VKAPI_ATTR VkResult VKAPI_CALL CreateImage(VkDevice, const VkImageCreateInfo* ci, const VkAllocationCallbacks* alloc, VkImage* out) {
    const uint32_t texel = format_texel_size(ci->format);
    if (!texel || ci->samples > 1) return VK_ERROR_FORMAT_NOT_SUPPORTED;
    auto* img = host_new<Image>(alloc, kScopeObject);
    if (!img) return VK_ERROR_OUT_OF_HOST_MEMORY;
    img->format = ci->format;
    img->texel = texel;
    img->extent = ci->extent;
    img->levels = ci->mipLevels ? ci->mipLevels : 1;
    img->layers = ci->arrayLayers ? ci->arrayLayers : 1;
    image_layout(*img);
    *out = to_handle<VkImage>(img);
    return VK_SUCCESS;
}
VKAPI_ATTR void VKAPI_CALL DestroyImage(VkDevice, VkImage i, const VkAllocationCallbacks* alloc) { host_delete(reinterpret_cast<Image*>(i), alloc); }
VKAPI_ATTR void VKAPI_CALL GetImageMemoryRequirements(VkDevice, VkImage image, VkMemoryRequirements* r) {
    auto* img = reinterpret_cast<Image*>(image);
    r->size = (img->total_size + 255) & ~255ull;
    r->alignment = 256;
    r->memoryTypeBits = 0x3;
}
VKAPI_ATTR VkResult VKAPI_CALL BindImageMemory(VkDevice, VkImage image, VkDeviceMemory memory, VkDeviceSize offset) {
    auto* img = reinterpret_cast<Image*>(image);
    auto* m = reinterpret_cast<DeviceMemory*>(memory);
    if (offset + img->total_size > m->size) return VK_ERROR_OUT_OF_DEVICE_MEMORY;
    img->memory = m;
    img->offset = offset;
    return VK_SUCCESS;
}
VKAPI_ATTR void VKAPI_CALL GetImageSubresourceLayout(VkDevice, VkImage image, const VkImageSubresource* sub, VkSubresourceLayout* out) {
    auto* img = reinterpret_cast<Image*>(image);
    const ImageLevel& L = img->level[std::min(sub->mipLevel, img->levels - 1)];
    out->offset = static_cast<uint64_t>(sub->arrayLayer) * img->layer_size + L.offset;
    out->size = L.size;
    out->rowPitch = L.stride;
    out->arrayPitch = img->layer_size;
    out->depthPitch = L.plane;
}

VKAPI_ATTR VkResult VKAPI_CALL CreateImageView(VkDevice, const VkImageViewCreateInfo* ci, const VkAllocationCallbacks* alloc, VkImageView* out) {
    auto* v = host_new<ImageView>(alloc, kScopeObject);
    if (!v) return VK_ERROR_OUT_OF_HOST_MEMORY;
    v->image = reinterpret_cast<Image*>(ci->image);
    v->format = ci->format;
    v->range = ci->subresourceRange;
    v->components = ci->components;
    if (v->range.levelCount == VK_REMAINING_MIP_LEVELS) v->range.levelCount = v->image->levels - v->range.baseMipLevel;
    if (v->range.layerCount == VK_REMAINING_ARRAY_LAYERS) v->range.layerCount = v->image->layers - v->range.baseArrayLayer;
    *out = to_handle<VkImageView>(v);
    return VK_SUCCESS;
}
VKAPI_ATTR void VKAPI_CALL DestroyImageView(VkDevice, VkImageView v, const VkAllocationCallbacks* alloc) { host_delete(reinterpret_cast<ImageView*>(v), alloc); }

VKAPI_ATTR VkResult VKAPI_CALL CreateSampler(VkDevice, const VkSamplerCreateInfo* ci, const VkAllocationCallbacks* alloc, VkSampler* out) {
    if (ci->anisotropyEnable || ci->compareEnable || ci->unnormalizedCoordinates) return VK_ERROR_FEATURE_NOT_PRESENT;
    auto* s = host_new<Sampler>(alloc, kScopeObject);
    if (!s) return VK_ERROR_OUT_OF_HOST_MEMORY;
    s->info = *ci;
    s->info.pNext = nullptr;
    *out = to_handle<VkSampler>(s);
    return VK_SUCCESS;
}
VKAPI_ATTR void VKAPI_CALL DestroySampler(VkDevice, VkSampler s, const VkAllocationCallbacks* alloc) { host_delete(reinterpret_cast<Sampler*>(s), alloc); }

// --------------------------------------------------------------- shaders --

VKAPI_ATTR VkResult VKAPI_CALL CreateShaderModule(VkDevice, const VkShaderModuleCreateInfo* ci, const VkAllocationCallbacks* alloc, VkShaderModule* out) {
    auto* sm = host_new<ShaderModule>(alloc, kScopeObject);
    if (!sm) return VK_ERROR_OUT_OF_HOST_MEMORY;
    sm->words.assign(ci->pCode, ci->pCode + ci->codeSize / 4);
    std::string err;
    if (!spirv::parse(sm->words.data(), sm->words.size(), sm->module, err)) {
        rt::set_last_error("vkCreateShaderModule: " + err);
        host_delete(sm, alloc);
        return VK_ERROR_INITIALIZATION_FAILED;
    }
    *out = to_handle<VkShaderModule>(sm);
    return VK_SUCCESS;
}
VKAPI_ATTR void VKAPI_CALL DestroyShaderModule(VkDevice, VkShaderModule s, const VkAllocationCallbacks* alloc) { host_delete(reinterpret_cast<ShaderModule*>(s), alloc); }

// Pipeline cache blob: 32-byte header {size, version 1, vendor, device,
// UUID[16]} + u32 count + {key[32], u32 size, cubin} entries — the layout of
// CPVulkan/PipelineCache.cpp:5-120 with a cubin payload.
VKAPI_ATTR VkResult VKAPI_CALL CreatePipelineCache(VkDevice, const VkPipelineCacheCreateInfo* ci, const VkAllocationCallbacks* alloc, VkPipelineCache* out) {
    auto* c = host_new<PipelineCache>(alloc, kScopeObject);
    if (!c) return VK_ERROR_OUT_OF_HOST_MEMORY;
    const uint8_t* d = static_cast<const uint8_t*>(ci->pInitialData);
    size_t n = ci->initialDataSize;
    if (d && n >= 36) {
        uint32_t count;
        std::memcpy(&count, d + 32, 4);
        size_t pos = 36;
        for (uint32_t i = 0; i < count && pos + 36 <= n; i++) {
            std::array<uint8_t, 32> key;
            std::memcpy(key.data(), d + pos, 32);
            uint32_t size;
            std::memcpy(&size, d + pos + 32, 4);
            pos += 36;
            if (pos + size > n) break;
            c->entries[key].assign(d + pos, d + pos + size);
            pos += size;
        }
    }
    *out = to_handle<VkPipelineCache>(c);
    return VK_SUCCESS;
}
VKAPI_ATTR void VKAPI_CALL DestroyPipelineCache(VkDevice, VkPipelineCache c, const VkAllocationCallbacks* alloc) { host_delete(reinterpret_cast<PipelineCache*>(c), alloc); }
VKAPI_ATTR VkResult VKAPI_CALL GetPipelineCacheData(VkDevice, VkPipelineCache cache, size_t* size, void* data) {
    auto* c = reinterpret_cast<PipelineCache*>(cache);
    std::lock_guard<std::mutex> lock(c->mutex);
    size_t need = 36;
    for (auto& kv : c->entries) need += 36 + kv.second.size();
    if (!data) {
        *size = need;
        return VK_SUCCESS;
    }
    if (*size < need) {
        *size = 0;
        return VK_INCOMPLETE;
    }
    uint8_t* o = static_cast<uint8_t*>(data);
    const uint32_t header[4] = {32u, 1u, 0x10DEu, 0x0103u};
    std::memcpy(o, header, 16);
    VkPhysicalDeviceProperties props;
    GetPhysicalDeviceProperties(nullptr, &props);
    std::memcpy(o + 16, props.pipelineCacheUUID, 16);
    const uint32_t count = static_cast<uint32_t>(c->entries.size());
    std::memcpy(o + 32, &count, 4);
    size_t pos = 36;
    for (auto& kv : c->entries) {
        std::memcpy(o + pos, kv.first.data(), 32);
        const uint32_t s = static_cast<uint32_t>(kv.second.size());
        std::memcpy(o + pos + 32, &s, 4);
        std::memcpy(o + pos + 36, kv.second.data(), s);
        pos += 36 + s;
    }
    *size = need;
    return VK_SUCCESS;
}

VKAPI_ATTR VkResult VKAPI_CALL CreateGraphicsPipelines(VkDevice device, VkPipelineCache cache, uint32_t n, const VkGraphicsPipelineCreateInfo* ci,
                                                       const VkAllocationCallbacks*, VkPipeline* out) {
    auto* dev = reinterpret_cast<Device*>(device);
    VkResult result = VK_SUCCESS;
    for (uint32_t i = 0; i < n; i++) {
        Pipeline* p = nullptr;
        const VkResult r = create_graphics_pipeline(dev, reinterpret_cast<PipelineCache*>(cache), ci[i], &p);
        out[i] = to_handle<VkPipeline>(p);
        if (r != VK_SUCCESS) result = r;
    }
    return result;
}
VKAPI_ATTR void VKAPI_CALL DestroyPipeline(VkDevice, VkPipeline pipeline, const VkAllocationCallbacks*) {
    auto* p = reinterpret_cast<Pipeline*>(pipeline);
    if (!p) return;
    rt::unload(p->module);
    delete p;
}

VKAPI_ATTR VkResult VKAPI_CALL CreatePipelineLayout(VkDevice, const VkPipelineLayoutCreateInfo* ci, const VkAllocationCallbacks* alloc, VkPipelineLayout* out) {
    auto* l = host_new<PipelineLayout>(alloc, kScopeObject);
    if (!l) return VK_ERROR_OUT_OF_HOST_MEMORY;
    for (uint32_t i = 0; i < ci->setLayoutCount; i++) l->sets.push_back(reinterpret_cast<DescriptorSetLayout*>(ci->pSetLayouts[i]));
    for (uint32_t i = 0; i < ci->pushConstantRangeCount; i++) l->push.push_back(ci->pPushConstantRanges[i]);
    *out = to_handle<VkPipelineLayout>(l);
    return VK_SUCCESS;
}
VKAPI_ATTR void VKAPI_CALL DestroyPipelineLayout(VkDevice, VkPipelineLayout l, const VkAllocationCallbacks* alloc) { host_delete(reinterpret_cast<PipelineLayout*>(l), alloc); }

// ------------------------------------------------------------ descriptors --

VKAPI_ATTR VkResult VKAPI_CALL CreateDescriptorSetLayout(VkDevice, const VkDescriptorSetLayoutCreateInfo* ci, const VkAllocationCallbacks* alloc,
                                                         VkDescriptorSetLayout* out) {
    auto* l = host_new<DescriptorSetLayout>(alloc, kScopeObject);
    if (!l) return VK_ERROR_OUT_OF_HOST_MEMORY;
    for (uint32_t i = 0; i < ci->bindingCount; i++) {
        VkDescriptorSetLayoutBinding b = ci->pBindings[i];
        std::vector<Sampler*> imm;
        if (b.pImmutableSamplers)
            for (uint32_t k = 0; k < b.descriptorCount; k++) imm.push_back(reinterpret_cast<Sampler*>(b.pImmutableSamplers[k]));
        b.pImmutableSamplers = nullptr;
        l->bindings.push_back(b);
        l->immutable.push_back(imm);
    }
    *out = to_handle<VkDescriptorSetLayout>(l);
    return VK_SUCCESS;
}
VKAPI_ATTR void VKAPI_CALL DestroyDescriptorSetLayout(VkDevice, VkDescriptorSetLayout l, const VkAllocationCallbacks* alloc) {
    host_delete(reinterpret_cast<DescriptorSetLayout*>(l), alloc);
}
VKAPI_ATTR VkResult VKAPI_CALL CreateDescriptorPool(VkDevice, const VkDescriptorPoolCreateInfo*, const VkAllocationCallbacks* alloc, VkDescriptorPool* out) {
    auto* p = host_new<DescriptorPool>(alloc, kScopeObject);
    if (!p) return VK_ERROR_OUT_OF_HOST_MEMORY;
    *out = to_handle<VkDescriptorPool>(p);
    return VK_SUCCESS;
}
VKAPI_ATTR void VKAPI_CALL DestroyDescriptorPool(VkDevice, VkDescriptorPool pool, const VkAllocationCallbacks* alloc) {
    auto* p = reinterpret_cast<DescriptorPool*>(pool);
    if (!p) return;
    for (auto* s : p->sets) delete s;
    host_delete(p, alloc);
}
VKAPI_ATTR VkResult VKAPI_CALL AllocateDescriptorSets(VkDevice, const VkDescriptorSetAllocateInfo* ai, VkDescriptorSet* out) {
    auto* pool = reinterpret_cast<DescriptorPool*>(ai->descriptorPool);
    for (uint32_t i = 0; i < ai->descriptorSetCount; i++) {
        auto* s = new DescriptorSet();
        s->layout = reinterpret_cast<DescriptorSetLayout*>(ai->pSetLayouts[i]);
        for (size_t k = 0; k < s->layout->bindings.size(); k++) {
            const auto& b = s->layout->bindings[k];
            auto& v = s->bindings[b.binding];
            v.resize(b.descriptorCount);
            for (uint32_t j = 0; j < b.descriptorCount; j++) {
                v[j].type = b.descriptorType;
                if (j < s->layout->immutable[k].size()) v[j].sampler = s->layout->immutable[k][j];
            }
        }
        pool->sets.insert(s);
        out[i] = to_handle<VkDescriptorSet>(s);
    }
    return VK_SUCCESS;
}
VKAPI_ATTR VkResult VKAPI_CALL FreeDescriptorSets(VkDevice, VkDescriptorPool pool, uint32_t n, const VkDescriptorSet* sets) {
    auto* p = reinterpret_cast<DescriptorPool*>(pool);
    for (uint32_t i = 0; i < n; i++) {
        auto* s = reinterpret_cast<DescriptorSet*>(sets[i]);
        p->sets.erase(s);
        delete s;
    }
    return VK_SUCCESS;
}
VKAPI_ATTR void VKAPI_CALL UpdateDescriptorSets(VkDevice, uint32_t nw, const VkWriteDescriptorSet* w, uint32_t nc, const VkCopyDescriptorSet* c) {
    for (uint32_t i = 0; i < nw; i++) {
        auto* s = reinterpret_cast<DescriptorSet*>(w[i].dstSet);
        auto& v = s->bindings[w[i].dstBinding];
        for (uint32_t k = 0; k < w[i].descriptorCount; k++) {
            const uint32_t e = w[i].dstArrayElement + k;
            if (e >= v.size()) v.resize(e + 1);
            Descriptor& d = v[e];
            d.type = w[i].descriptorType;
            switch (w[i].descriptorType) {
            case VK_DESCRIPTOR_TYPE_UNIFORM_BUFFER:
            case VK_DESCRIPTOR_TYPE_UNIFORM_BUFFER_DYNAMIC:
            case VK_DESCRIPTOR_TYPE_STORAGE_BUFFER:
            case VK_DESCRIPTOR_TYPE_STORAGE_BUFFER_DYNAMIC:
                d.buffer = reinterpret_cast<Buffer*>(w[i].pBufferInfo[k].buffer);
                d.offset = w[i].pBufferInfo[k].offset;
                d.range = w[i].pBufferInfo[k].range;
                break;
            case VK_DESCRIPTOR_TYPE_COMBINED_IMAGE_SAMPLER:
                d.view = reinterpret_cast<ImageView*>(w[i].pImageInfo[k].imageView);
                if (w[i].pImageInfo[k].sampler) d.sampler = reinterpret_cast<Sampler*>(w[i].pImageInfo[k].sampler);
                break;
            case VK_DESCRIPTOR_TYPE_SAMPLED_IMAGE:
            case VK_DESCRIPTOR_TYPE_STORAGE_IMAGE:
                d.view = reinterpret_cast<ImageView*>(w[i].pImageInfo[k].imageView);
                break;
            case VK_DESCRIPTOR_TYPE_SAMPLER:
                if (w[i].pImageInfo[k].sampler) d.sampler = reinterpret_cast<Sampler*>(w[i].pImageInfo[k].sampler);
                break;
            default:
                break;
            }
        }
    }
    for (uint32_t i = 0; i < nc; i++) {
        auto* src = reinterpret_cast<DescriptorSet*>(c[i].srcSet);
        auto* dst = reinterpret_cast<DescriptorSet*>(c[i].dstSet);
        for (uint32_t k = 0; k < c[i].descriptorCount; k++) {
            auto& sv = src->bindings[c[i].srcBinding];
            auto& dv = dst->bindings[c[i].dstBinding];
            if (c[i].srcArrayElement + k >= sv.size()) break;
            if (c[i].dstArrayElement + k >= dv.size()) dv.resize(c[i].dstArrayElement + k + 1);
            dv[c[i].dstArrayElement + k] = sv[c[i].srcArrayElement + k];
        }
    }
}

// ------------------------------------------------- render pass, framebuffer --

VKAPI_ATTR VkResult VKAPI_CALL CreateRenderPass(VkDevice, const VkRenderPassCreateInfo* ci, const VkAllocationCallbacks* alloc, VkRenderPass* out) {
    if (ci->subpassCount == 0 || !ci->pSubpasses) {
        rt::set_last_error("vkCreateRenderPass: a render pass needs a subpass");
        return VK_ERROR_INITIALIZATION_FAILED;
    }
    auto* rp = host_new<RenderPass>(alloc, kScopeObject);
    if (!rp) return VK_ERROR_OUT_OF_HOST_MEMORY;
    rp->attachments.assign(ci->pAttachments, ci->pAttachments + ci->attachmentCount);
    // each subpass's colour and depth references (input attachments and
    // dependencies need nothing: subpasses run in order on one stream)
    for (uint32_t k = 0; k < ci->subpassCount; k++) {
        const auto& sp = ci->pSubpasses[k];
        Subpass sub;
        // colour references keep their positions (location L of the
        // fragment shader writes reference L); trailing unused ones are
        // dropped, so a subpass whose only reference is unused has none
        for (uint32_t i = 0; i < sp.colorAttachmentCount; i++) sub.colour.push_back(sp.pColorAttachments[i].attachment);
        while (!sub.colour.empty() && sub.colour.back() == VK_ATTACHMENT_UNUSED) sub.colour.pop_back();
        if (sp.pDepthStencilAttachment) sub.depth = sp.pDepthStencilAttachment->attachment;
        rp->subpasses.push_back(sub);
    }
    *out = to_handle<VkRenderPass>(rp);
    return VK_SUCCESS;
}
VKAPI_ATTR void VKAPI_CALL DestroyRenderPass(VkDevice, VkRenderPass rp, const VkAllocationCallbacks* alloc) { host_delete(reinterpret_cast<RenderPass*>(rp), alloc); }

VKAPI_ATTR VkResult VKAPI_CALL CreateFramebuffer(VkDevice, const VkFramebufferCreateInfo* ci, const VkAllocationCallbacks* alloc, VkFramebuffer* out) {
    auto* fb = host_new<Framebuffer>(alloc, kScopeObject);
    if (!fb) return VK_ERROR_OUT_OF_HOST_MEMORY;
    fb->pass = reinterpret_cast<RenderPass*>(ci->renderPass);
    for (uint32_t i = 0; i < ci->attachmentCount; i++) fb->attachments.push_back(reinterpret_cast<ImageView*>(ci->pAttachments[i]));
    fb->width = ci->width;
    fb->height = ci->height;
    fb->layers = ci->layers;
    *out = to_handle<VkFramebuffer>(fb);
    return VK_SUCCESS;
}
VKAPI_ATTR void VKAPI_CALL DestroyFramebuffer(VkDevice, VkFramebuffer fb, const VkAllocationCallbacks* alloc) { host_delete(reinterpret_cast<Framebuffer*>(fb), alloc); }

// ------------------------------------------------------- command buffers --

VKAPI_ATTR VkResult VKAPI_CALL CreateCommandPool(VkDevice, const VkCommandPoolCreateInfo*, const VkAllocationCallbacks* alloc, VkCommandPool* out) {
    auto* p = host_new<CommandPool>(alloc, kScopeObject);
    if (!p) return VK_ERROR_OUT_OF_HOST_MEMORY;
    *out = to_handle<VkCommandPool>(p);
    return VK_SUCCESS;
}
VKAPI_ATTR void VKAPI_CALL DestroyCommandPool(VkDevice, VkCommandPool pool, const VkAllocationCallbacks* alloc) {
    auto* p = reinterpret_cast<CommandPool*>(pool);
    if (!p) return;
    for (auto* cb : p->buffers) delete cb;
    host_delete(p, alloc);
}
VKAPI_ATTR VkResult VKAPI_CALL ResetCommandPool(VkDevice, VkCommandPool pool, VkCommandPoolResetFlags) {
    for (auto* cb : reinterpret_cast<CommandPool*>(pool)->buffers) cb->reset();
    return VK_SUCCESS;
}
VKAPI_ATTR VkResult VKAPI_CALL AllocateCommandBuffers(VkDevice device, const VkCommandBufferAllocateInfo* ai, VkCommandBuffer* out) {
    auto* pool = reinterpret_cast<CommandPool*>(ai->commandPool);
    if (ai->level != VK_COMMAND_BUFFER_LEVEL_PRIMARY && ai->level != VK_COMMAND_BUFFER_LEVEL_SECONDARY) return VK_ERROR_FEATURE_NOT_PRESENT;
    for (uint32_t i = 0; i < ai->commandBufferCount; i++) {
        auto* cb = new CommandBuffer();
        cb->device = reinterpret_cast<Device*>(device);
        cb->secondary = ai->level == VK_COMMAND_BUFFER_LEVEL_SECONDARY;
        pool->buffers.insert(cb);
        out[i] = to_handle<VkCommandBuffer>(cb);
    }
    return VK_SUCCESS;
}
VKAPI_ATTR void VKAPI_CALL FreeCommandBuffers(VkDevice, VkCommandPool pool, uint32_t n, const VkCommandBuffer* cbs) {
    auto* p = reinterpret_cast<CommandPool*>(pool);
    for (uint32_t i = 0; i < n; i++) {
        auto* cb = reinterpret_cast<CommandBuffer*>(cbs[i]);
        p->buffers.erase(cb);
        delete cb;
    }
}
VKAPI_ATTR VkResult VKAPI_CALL BeginCommandBuffer(VkCommandBuffer cmd, const VkCommandBufferBeginInfo*) {
    auto* cb = reinterpret_cast<CommandBuffer*>(cmd);
    cb->reset();
    cb->recording = true;
    return VK_SUCCESS;
}
VKAPI_ATTR VkResult VKAPI_CALL EndCommandBuffer(VkCommandBuffer cmd) {
    auto* cb = reinterpret_cast<CommandBuffer*>(cmd);
    cb->recording = false;
    if (!cb->secondary) precompile_batches(cb);  // a secondary's draws are compiled with the primary that executes them
    return VK_SUCCESS;
}
VKAPI_ATTR VkResult VKAPI_CALL ResetCommandBuffer(VkCommandBuffer cmd, VkCommandBufferResetFlags) {
    reinterpret_cast<CommandBuffer*>(cmd)->reset();
    return VK_SUCCESS;
}

Cmd& push(VkCommandBuffer cmd, CmdType t) {
    auto* cb = reinterpret_cast<CommandBuffer*>(cmd);
    cb->cmds.push_back(Cmd{t});
    return cb->cmds.back();
}

VKAPI_ATTR void VKAPI_CALL CmdBindPipeline(VkCommandBuffer cmd, VkPipelineBindPoint, VkPipeline p) { push(cmd, CmdType::BindPipeline).p[0] = reinterpret_cast<void*>(p); }
VKAPI_ATTR void VKAPI_CALL CmdSetViewport(VkCommandBuffer cmd, uint32_t first, uint32_t n, const VkViewport* v) {
    if (first == 0 && n >= 1) push(cmd, CmdType::SetViewport).viewport = v[0];
}
VKAPI_ATTR void VKAPI_CALL CmdSetScissor(VkCommandBuffer cmd, uint32_t, uint32_t, const VkRect2D*) { push(cmd, CmdType::SetScissor); }
VKAPI_ATTR void VKAPI_CALL CmdSetBlendConstants(VkCommandBuffer cmd, const float c[4]) {
    auto& x = push(cmd, CmdType::SetBlendConstants);
    x.bytes.assign(reinterpret_cast<const uint8_t*>(c), reinterpret_cast<const uint8_t*>(c) + 16);
}
// Dynamic state a pipeline here never takes from the command buffer: dynamic
// line width (on line topologies), depth bounds and the stencil masks and
// reference are rejected at pipeline creation (the reference aborts on
// them: CPVulkan/CommandBuffer.h:37-43, LLVMRuntime/PipelineCompiler.cpp:
// 1137-1146, 1196-1203), and depth bias is not applied, as in the reference.
// Setting state a bound pipeline does not declare dynamic has no effect, so
// these record nothing.
VKAPI_ATTR void VKAPI_CALL CmdSetLineWidth(VkCommandBuffer, float) {}
VKAPI_ATTR void VKAPI_CALL CmdSetDepthBias(VkCommandBuffer, float, float, float) {}
VKAPI_ATTR void VKAPI_CALL CmdSetDepthBounds(VkCommandBuffer, float, float) {}
VKAPI_ATTR void VKAPI_CALL CmdSetStencilCompareMask(VkCommandBuffer, VkStencilFaceFlags, uint32_t) {}
VKAPI_ATTR void VKAPI_CALL CmdSetStencilWriteMask(VkCommandBuffer, VkStencilFaceFlags, uint32_t) {}
VKAPI_ATTR void VKAPI_CALL CmdSetStencilReference(VkCommandBuffer, VkStencilFaceFlags, uint32_t) {}
// vkCmdNextSubpass (CPVulkan/CommandBuffer.cpp:649-664, 931-935).
VKAPI_ATTR void VKAPI_CALL CmdNextSubpass(VkCommandBuffer cmd, VkSubpassContents) { push(cmd, CmdType::NextSubpass); }
VKAPI_ATTR void VKAPI_CALL CmdBindDescriptorSets(VkCommandBuffer cmd, VkPipelineBindPoint, VkPipelineLayout, uint32_t first, uint32_t n,
                                                 const VkDescriptorSet* sets, uint32_t ndyn, const uint32_t* dyn) {
    auto& c = push(cmd, CmdType::BindDescriptorSets);
    c.u[0] = first;
    c.u[1] = n;
    c.u[2] = ndyn;
    for (uint32_t i = 0; i < n; i++) c.list.push_back(reinterpret_cast<uint64_t>(sets[i]));
    for (uint32_t i = 0; i < ndyn; i++) c.list.push_back(dyn[i]);
}
VKAPI_ATTR void VKAPI_CALL CmdBindIndexBuffer(VkCommandBuffer cmd, VkBuffer b, VkDeviceSize offset, VkIndexType t) {
    auto& c = push(cmd, CmdType::BindIndexBuffer);
    c.p[0] = reinterpret_cast<void*>(b);
    c.q[0] = offset;
    c.u[0] = t;
}
// vkCmdBindVertexBuffers: records (buffer, offset) per binding
// (CPVulkan/CommandBuffer.Binding.cpp:142-178, 265-278).
VKAPI_ATTR void VKAPI_CALL CmdBindVertexBuffers(VkCommandBuffer cmd, uint32_t first, uint32_t n, const VkBuffer* b, const VkDeviceSize* off) {
    auto& c = push(cmd, CmdType::BindVertexBuffers);
    c.u[0] = first;
    c.u[1] = n;
    for (uint32_t i = 0; i < n; i++) {
        c.list.push_back(reinterpret_cast<uint64_t>(b[i]));
        c.list.push_back(off[i]);
    }
}
// vkCmdDraw / vkCmdDrawIndexed (CPVulkan/CommandBuffer.Draw.cpp:2350-2360).
VKAPI_ATTR void VKAPI_CALL CmdDraw(VkCommandBuffer cmd, uint32_t count, uint32_t instances, uint32_t first, uint32_t first_instance) {
    auto& c = push(cmd, CmdType::Draw);
    c.u[0] = count;
    c.u[1] = instances;
    c.u[2] = first;
    c.u[3] = first_instance;
}
VKAPI_ATTR void VKAPI_CALL CmdDrawIndexed(VkCommandBuffer cmd, uint32_t count, uint32_t instances, uint32_t first, int32_t vertex_offset,
                                          uint32_t first_instance) {
    auto& c = push(cmd, CmdType::DrawIndexed);
    c.u[0] = count;
    c.u[1] = instances;
    c.u[2] = first;
    c.i0 = vertex_offset;
    c.u[3] = first_instance;
}
VKAPI_ATTR void VKAPI_CALL CmdDrawIndirect(VkCommandBuffer cmd, VkBuffer b, VkDeviceSize off, uint32_t n, uint32_t stride) {
    auto& c = push(cmd, CmdType::DrawIndirect);
    c.p[0] = reinterpret_cast<void*>(b);
    c.q[0] = off;
    c.u[0] = n;
    c.u[1] = stride;
}
VKAPI_ATTR void VKAPI_CALL CmdDrawIndexedIndirect(VkCommandBuffer cmd, VkBuffer b, VkDeviceSize off, uint32_t n, uint32_t stride) {
    auto& c = push(cmd, CmdType::DrawIndexedIndirect);
    c.p[0] = reinterpret_cast<void*>(b);
    c.q[0] = off;
    c.u[0] = n;
    c.u[1] = stride;
}
// vkCmdDraw(Indexed)IndirectCountKHR / vkCmdDrawIndirectCountAMD
// (CPVulkan/CommandBuffer.Draw.cpp:2226-2348, 2421-2433): the draw count is
// min(maxDrawCount, the 32-bit word at countBufferOffset), read at replay.
VKAPI_ATTR void VKAPI_CALL CmdDrawIndirectCount(VkCommandBuffer cmd, VkBuffer b, VkDeviceSize off, VkBuffer count_buffer, VkDeviceSize count_off,
                                                uint32_t max_draws, uint32_t stride) {
    CmdDrawIndirect(cmd, b, off, max_draws, stride);
    auto& c = reinterpret_cast<CommandBuffer*>(cmd)->cmds.back();
    c.p[1] = reinterpret_cast<void*>(count_buffer);
    c.q[1] = count_off;
}
VKAPI_ATTR void VKAPI_CALL CmdDrawIndexedIndirectCount(VkCommandBuffer cmd, VkBuffer b, VkDeviceSize off, VkBuffer count_buffer, VkDeviceSize count_off,
                                                       uint32_t max_draws, uint32_t stride) {
    CmdDrawIndexedIndirect(cmd, b, off, max_draws, stride);
    auto& c = reinterpret_cast<CommandBuffer*>(cmd)->cmds.back();
    c.p[1] = reinterpret_cast<void*>(count_buffer);
    c.q[1] = count_off;
}
VKAPI_ATTR void VKAPI_CALL CmdCopyBuffer(VkCommandBuffer cmd, VkBuffer src, VkBuffer dst, uint32_t n, const VkBufferCopy* r) {
    auto& c = push(cmd, CmdType::CopyBuffer);
    c.p[0] = reinterpret_cast<void*>(src);
    c.p[1] = reinterpret_cast<void*>(dst);
    c.buffer_regions.assign(r, r + n);
}
VKAPI_ATTR void VKAPI_CALL CmdCopyBufferToImage(VkCommandBuffer cmd, VkBuffer src, VkImage dst, VkImageLayout, uint32_t n, const VkBufferImageCopy* r) {
    auto& c = push(cmd, CmdType::CopyBufferToImage);
    c.p[0] = reinterpret_cast<void*>(src);
    c.p[1] = reinterpret_cast<void*>(dst);
    c.image_regions.assign(r, r + n);
}
VKAPI_ATTR void VKAPI_CALL CmdCopyImageToBuffer(VkCommandBuffer cmd, VkImage src, VkImageLayout, VkBuffer dst, uint32_t n, const VkBufferImageCopy* r) {
    auto& c = push(cmd, CmdType::CopyImageToBuffer);
    c.p[0] = reinterpret_cast<void*>(dst);
    c.p[1] = reinterpret_cast<void*>(src);
    c.image_regions.assign(r, r + n);
}
// vkCmdBlitImage (CPVulkan/CommandBuffer.cpp:822-826).
VKAPI_ATTR void VKAPI_CALL CmdBlitImage(VkCommandBuffer cmd, VkImage src, VkImageLayout, VkImage dst, VkImageLayout, uint32_t n, const VkImageBlit* r,
                                        VkFilter filter) {
    auto& c = push(cmd, CmdType::BlitImage);
    c.p[0] = reinterpret_cast<void*>(src);
    c.p[1] = reinterpret_cast<void*>(dst);
    c.u[0] = static_cast<uint32_t>(filter);
    c.blit_regions.assign(r, r + n);
}
// vkCmdCopyImage (CPVulkan/CommandBuffer.Copy.cpp:1091-1095).
VKAPI_ATTR void VKAPI_CALL CmdCopyImage(VkCommandBuffer cmd, VkImage src, VkImageLayout, VkImage dst, VkImageLayout, uint32_t n, const VkImageCopy* r) {
    auto& c = push(cmd, CmdType::CopyImage);
    c.p[0] = reinterpret_cast<void*>(src);
    c.p[1] = reinterpret_cast<void*>(dst);
    c.image_copies.assign(r, r + n);
}
// vkCmdClearColorImage / vkCmdClearDepthStencilImage / vkCmdClearAttachments
// (CPVulkan/CommandBuffer.Draw.cpp:2380-2396).
VKAPI_ATTR void VKAPI_CALL CmdClearColorImage(VkCommandBuffer cmd, VkImage image, VkImageLayout, const VkClearColorValue* colour, uint32_t n,
                                              const VkImageSubresourceRange* ranges) {
    auto& c = push(cmd, CmdType::ClearImage);
    c.p[0] = reinterpret_cast<void*>(image);
    VkClearValue v{};
    v.color = *colour;
    c.clears.push_back(v);
    c.ranges.assign(ranges, ranges + n);
}
VKAPI_ATTR void VKAPI_CALL CmdClearDepthStencilImage(VkCommandBuffer cmd, VkImage image, VkImageLayout, const VkClearDepthStencilValue* ds, uint32_t n,
                                                     const VkImageSubresourceRange* ranges) {
    auto& c = push(cmd, CmdType::ClearImage);
    c.p[0] = reinterpret_cast<void*>(image);
    VkClearValue v{};
    v.depthStencil = *ds;
    c.clears.push_back(v);
    c.ranges.assign(ranges, ranges + n);
}
VKAPI_ATTR void VKAPI_CALL CmdClearAttachments(VkCommandBuffer cmd, uint32_t n, const VkClearAttachment* a, uint32_t rects, const VkClearRect* r) {
    auto& c = push(cmd, CmdType::ClearAttachments);
    c.clear_attachments.assign(a, a + n);
    c.clear_rects.assign(r, r + rects);
}
VKAPI_ATTR void VKAPI_CALL CmdFillBuffer(VkCommandBuffer cmd, VkBuffer dst, VkDeviceSize off, VkDeviceSize size, uint32_t data) {
    auto& c = push(cmd, CmdType::FillBuffer);
    c.p[0] = reinterpret_cast<void*>(dst);
    c.q[0] = off;
    c.q[1] = size;
    c.u[0] = data;
}
VKAPI_ATTR void VKAPI_CALL CmdUpdateBuffer(VkCommandBuffer cmd, VkBuffer dst, VkDeviceSize off, VkDeviceSize size, const void* data) {
    auto& c = push(cmd, CmdType::UpdateBuffer);
    c.p[0] = reinterpret_cast<void*>(dst);
    c.q[0] = off;
    c.bytes.assign(static_cast<const uint8_t*>(data), static_cast<const uint8_t*>(data) + size);
}
VKAPI_ATTR void VKAPI_CALL CmdPipelineBarrier(VkCommandBuffer cmd, VkPipelineStageFlags, VkPipelineStageFlags, VkDependencyFlags, uint32_t,
                                              const VkMemoryBarrier*, uint32_t, const VkBufferMemoryBarrier*, uint32_t, const VkImageMemoryBarrier*) {
    push(cmd, CmdType::Barrier);
}
VKAPI_ATTR void VKAPI_CALL CmdPushConstants(VkCommandBuffer cmd, VkPipelineLayout, VkShaderStageFlags, uint32_t off, uint32_t size, const void* v) {
    auto& c = push(cmd, CmdType::PushConstants);
    c.u[0] = off;
    c.bytes.assign(static_cast<const uint8_t*>(v), static_cast<const uint8_t*>(v) + size);
}
VKAPI_ATTR void VKAPI_CALL CmdBeginRenderPass(VkCommandBuffer cmd, const VkRenderPassBeginInfo* bi, VkSubpassContents) {
    auto& c = push(cmd, CmdType::BeginRenderPass);
    c.p[0] = reinterpret_cast<void*>(bi->renderPass);
    c.p[1] = reinterpret_cast<void*>(bi->framebuffer);
    c.clears.assign(bi->pClearValues, bi->pClearValues + bi->clearValueCount);
}
VKAPI_ATTR void VKAPI_CALL CmdEndRenderPass(VkCommandBuffer cmd) { push(cmd, CmdType::EndRenderPass); }

// vkCmdExecuteCommands (CPVulkan/CommandBuffer.cpp:704-730): the reference
// replays each secondary's commands in place, with the primary's state. A
// secondary re-recorded after this call invalidates the primary (Vulkan's
// rule), so its commands are copied into the primary now; the primary then
// batches, captures and replays them like its own.
VKAPI_ATTR void VKAPI_CALL CmdExecuteCommands(VkCommandBuffer cmd, uint32_t n, const VkCommandBuffer* cbs) {
    auto* primary = reinterpret_cast<CommandBuffer*>(cmd);
    for (uint32_t i = 0; i < n; i++) {
        const auto* sec = reinterpret_cast<const CommandBuffer*>(cbs[i]);
        if (sec && sec != primary) primary->cmds.insert(primary->cmds.end(), sec->cmds.begin(), sec->cmds.end());
    }
}

// ------------------------------------------------------ sync and submit --

VKAPI_ATTR VkResult VKAPI_CALL CreateFence(VkDevice, const VkFenceCreateInfo* ci, const VkAllocationCallbacks* alloc, VkFence* out) {
    auto* f = host_new<Fence>(alloc, kScopeObject);
    if (!f) return VK_ERROR_OUT_OF_HOST_MEMORY;
    if (rt::available() && cudaEventCreateWithFlags(&f->event, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        host_delete(f, alloc);
        return VK_ERROR_OUT_OF_DEVICE_MEMORY;
    }
    f->signalled = (ci->flags & VK_FENCE_CREATE_SIGNALED_BIT) != 0;
    *out = to_handle<VkFence>(f);
    return VK_SUCCESS;
}
VKAPI_ATTR void VKAPI_CALL DestroyFence(VkDevice, VkFence fence, const VkAllocationCallbacks* alloc) {
    auto* f = reinterpret_cast<Fence*>(fence);
    if (!f) return;
    if (f->event) cudaEventDestroy(f->event);
    host_delete(f, alloc);
}
VKAPI_ATTR VkResult VKAPI_CALL ResetFences(VkDevice, uint32_t n, const VkFence* fences) {
    for (uint32_t i = 0; i < n; i++) {
        auto* f = reinterpret_cast<Fence*>(fences[i]);
        f->signalled = false;
        f->pending = false;
    }
    return VK_SUCCESS;
}

// Queries a fence without blocking; on completion runs the coherence
// readback of its submission.
VkResult poll_fence(Device* dev, Fence* f) {
    if (f->signalled) return VK_SUCCESS;
    if (!f->pending) return VK_NOT_READY;
    const cudaError_t e = cudaEventQuery(f->event);
    if (e == cudaErrorNotReady) return VK_NOT_READY;
    if (e != cudaSuccess) {
        cudaGetLastError();
        return VK_ERROR_DEVICE_LOST;
    }
    {
        std::lock_guard<std::mutex> lock(dev->queue->mutex);
        complete_readback(f->readback);
    }
    f->pending = false;
    f->signalled = true;
    return VK_SUCCESS;
}

VKAPI_ATTR VkResult VKAPI_CALL GetFenceStatus(VkDevice device, VkFence fence) {
    return poll_fence(reinterpret_cast<Device*>(device), reinterpret_cast<Fence*>(fence));
}

// vkWaitForFences with a timeout in nanoseconds (CPVulkan/Fence.cpp:46-56,
// 192-198): polls the CUDA events; VK_TIMEOUT when the limit passes.
VKAPI_ATTR VkResult VKAPI_CALL WaitForFences(VkDevice device, uint32_t n, const VkFence* fences, VkBool32 all, uint64_t timeout) {
    auto* dev = reinterpret_cast<Device*>(device);
    const auto start = std::chrono::steady_clock::now();
    while (true) {
        uint32_t done = 0;
        for (uint32_t i = 0; i < n; i++) {
            const VkResult r = poll_fence(dev, reinterpret_cast<Fence*>(fences[i]));
            if (r == VK_ERROR_DEVICE_LOST) return r;
            if (r == VK_SUCCESS) done++;
        }
        if ((all && done == n) || (!all && done > 0)) return VK_SUCCESS;
        const auto elapsed = std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - start).count();
        if (timeout == 0 || static_cast<uint64_t>(elapsed) >= timeout) return VK_TIMEOUT;
        if (n == 1 && all && timeout == ~0ull) {
            auto* f = reinterpret_cast<Fence*>(fences[0]);
            if (f->pending && cudaEventSynchronize(f->event) != cudaSuccess) {
                cudaGetLastError();
                return VK_ERROR_DEVICE_LOST;
            }
            continue;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

VKAPI_ATTR VkResult VKAPI_CALL CreateSemaphore(VkDevice, const VkSemaphoreCreateInfo*, const VkAllocationCallbacks* alloc, VkSemaphore* out) {
    auto* s = host_new<Semaphore>(alloc, kScopeObject);
    if (!s) return VK_ERROR_OUT_OF_HOST_MEMORY;
    if (rt::available() && cudaEventCreateWithFlags(&s->event, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        host_delete(s, alloc);
        return VK_ERROR_OUT_OF_DEVICE_MEMORY;
    }
    *out = to_handle<VkSemaphore>(s);
    return VK_SUCCESS;
}
VKAPI_ATTR void VKAPI_CALL DestroySemaphore(VkDevice, VkSemaphore sem, const VkAllocationCallbacks* alloc) {
    auto* s = reinterpret_cast<Semaphore*>(sem);
    if (!s) return;
    if (s->event) cudaEventDestroy(s->event);
    host_delete(s, alloc);
}

// vkQueueSubmit (CPVulkan/Queue.cpp:11-77): waits, replays each command
// buffer onto the queue's stream, signals semaphores and the fence. Returns
// once the work is enqueued. no_alloc selects the fixed binning scratch.
VkResult submit(VkQueue queue, uint32_t n, const VkSubmitInfo* si, VkFence fence, bool no_alloc) {
    auto* q = reinterpret_cast<Queue*>(queue);
    Device* dev = q->device;
    if (dev->compile_only) {
        rt::set_last_error("vkQueueSubmit: compile-only device (no CUDA device)");
        return VK_ERROR_DEVICE_LOST;
    }
    std::vector<DeviceMemory*> written;
    {
        // Coherent host-visible memory: host writes made while mapped are
        // visible to the device at submission.
        std::lock_guard<std::mutex> lock(dev->memory_mutex);
        for (DeviceMemory* m : dev->memories)
            if (m->mapped && m->host) rt::copy_host_to_device(q->stream, m->device, m->host, m->size);
    }
    for (uint32_t i = 0; i < n; i++) {
        for (uint32_t k = 0; k < si[i].waitSemaphoreCount; k++) {
            auto* s = reinterpret_cast<Semaphore*>(si[i].pWaitSemaphores[k]);
            if (s->signalled) cudaStreamWaitEvent(q->stream, s->event, 0);
            s->signalled = false;
        }
        for (uint32_t k = 0; k < si[i].commandBufferCount; k++) {
            const VkResult r = run_command_buffer(q, reinterpret_cast<CommandBuffer*>(si[i].pCommandBuffers[k]), written, no_alloc);
            if (r != VK_SUCCESS) return r;
        }
        for (uint32_t k = 0; k < si[i].signalSemaphoreCount; k++) {
            auto* s = reinterpret_cast<Semaphore*>(si[i].pSignalSemaphores[k]);
            cudaEventRecord(s->event, q->stream);
            s->signalled = true;
        }
    }
    std::vector<DeviceMemory*> host_visible;
    for (DeviceMemory* m : written)
        if (m && m->host && std::find(host_visible.begin(), host_visible.end(), m) == host_visible.end()) host_visible.push_back(m);
    if (fence) {
        auto* f = reinterpret_cast<Fence*>(fence);
        if (cudaEventRecord(f->event, q->stream) != cudaSuccess) return VK_ERROR_DEVICE_LOST;
        f->pending = true;
        f->signalled = false;
        f->readback = host_visible;
    }
    {
        std::lock_guard<std::mutex> lock(q->mutex);
        for (DeviceMemory* m : host_visible) q->pending_readback.push_back(m);
    }
    if (cudaGetLastError() != cudaSuccess) return VK_ERROR_DEVICE_LOST;
    return VK_SUCCESS;
}

VKAPI_ATTR VkResult VKAPI_CALL QueueSubmit(VkQueue queue, uint32_t n, const VkSubmitInfo* si, VkFence fence) { return submit(queue, n, si, fence, false); }

// ------------------------------------------------------- dispatch tables --

struct Entry {
    const char* name;
    PFN_vkVoidFunction fn;
};

#define E(name) {"vk" #name, reinterpret_cast<PFN_vkVoidFunction>(name)}
const Entry kGlobal[] = {E(CreateInstance), E(EnumerateInstanceExtensionProperties), E(EnumerateInstanceVersion)};
const Entry kInstance[] = {
    E(DestroyInstance), E(EnumeratePhysicalDevices), E(GetPhysicalDeviceProperties), E(GetPhysicalDeviceFeatures),
    E(GetPhysicalDeviceMemoryProperties), E(GetPhysicalDeviceQueueFamilyProperties), E(GetPhysicalDeviceFormatProperties),
    E(EnumerateDeviceExtensionProperties), E(CreateDevice),
};
const Entry kDevice[] = {
    E(DestroyDevice), E(GetDeviceQueue), E(DeviceWaitIdle), E(QueueWaitIdle), E(AllocateMemory), E(FreeMemory), E(MapMemory), E(UnmapMemory),
    E(FlushMappedMemoryRanges), E(InvalidateMappedMemoryRanges), E(CreateBuffer), E(DestroyBuffer), E(GetBufferMemoryRequirements),
    E(BindBufferMemory), E(CreateImage), E(DestroyImage), E(GetImageMemoryRequirements), E(BindImageMemory), E(GetImageSubresourceLayout),
    E(CreateImageView), E(DestroyImageView), E(CreateSampler), E(DestroySampler), E(CreateShaderModule), E(DestroyShaderModule),
    E(CreatePipelineCache), E(DestroyPipelineCache), E(GetPipelineCacheData), E(CreateGraphicsPipelines), E(DestroyPipeline),
    E(CreatePipelineLayout), E(DestroyPipelineLayout), E(CreateDescriptorSetLayout), E(DestroyDescriptorSetLayout), E(CreateDescriptorPool),
    E(DestroyDescriptorPool), E(AllocateDescriptorSets), E(FreeDescriptorSets), E(UpdateDescriptorSets), E(CreateRenderPass),
    E(DestroyRenderPass), E(CreateFramebuffer), E(DestroyFramebuffer), E(CreateCommandPool), E(DestroyCommandPool), E(ResetCommandPool),
    E(AllocateCommandBuffers), E(FreeCommandBuffers), E(BeginCommandBuffer), E(EndCommandBuffer), E(ResetCommandBuffer), E(CmdBindPipeline),
    E(CmdSetViewport), E(CmdSetScissor), E(CmdSetBlendConstants), E(CmdSetLineWidth), E(CmdSetDepthBias), E(CmdSetDepthBounds),
    E(CmdSetStencilCompareMask), E(CmdSetStencilWriteMask), E(CmdSetStencilReference), E(CmdBindDescriptorSets), E(CmdBindIndexBuffer), E(CmdBindVertexBuffers),
    E(CmdDraw), E(CmdDrawIndexed), E(CmdDrawIndirect), E(CmdDrawIndexedIndirect),
    {"vkCmdDrawIndirectCountKHR", reinterpret_cast<PFN_vkVoidFunction>(CmdDrawIndirectCount)},
    {"vkCmdDrawIndexedIndirectCountKHR", reinterpret_cast<PFN_vkVoidFunction>(CmdDrawIndexedIndirectCount)},
    {"vkCmdDrawIndirectCountAMD", reinterpret_cast<PFN_vkVoidFunction>(CmdDrawIndirectCount)}, E(CmdCopyBuffer), E(CmdCopyImage),
    E(CmdClearColorImage), E(CmdClearDepthStencilImage), E(CmdClearAttachments), E(CmdCopyBufferToImage), E(CmdBlitImage),
    E(CmdCopyImageToBuffer), E(CmdFillBuffer), E(CmdUpdateBuffer), E(CmdPipelineBarrier), E(CmdPushConstants), E(CmdBeginRenderPass),
    E(CmdNextSubpass), E(CmdEndRenderPass), E(CmdExecuteCommands), E(QueueSubmit), E(CreateFence), E(DestroyFence), E(ResetFences), E(GetFenceStatus), E(WaitForFences),
    E(CreateSemaphore), E(DestroySemaphore),
};
#undef E

PFN_vkVoidFunction lookup(const Entry* t, size_t n, const char* name) {
    for (size_t i = 0; i < n; i++)
        if (std::strcmp(t[i].name, name) == 0) return t[i].fn;
    return nullptr;
}

VKAPI_ATTR PFN_vkVoidFunction VKAPI_CALL GetDeviceProcAddr(VkDevice, const char* name) {
    if (std::strcmp(name, "vkGetDeviceProcAddr") == 0) return reinterpret_cast<PFN_vkVoidFunction>(GetDeviceProcAddr);
    return lookup(kDevice, sizeof(kDevice) / sizeof(kDevice[0]), name);
}

VKAPI_ATTR PFN_vkVoidFunction VKAPI_CALL GetInstanceProcAddr(VkInstance instance, const char* name) {
    if (!name) return nullptr;
    if (std::strcmp(name, "vkGetInstanceProcAddr") == 0) return reinterpret_cast<PFN_vkVoidFunction>(GetInstanceProcAddr);
    if (std::strcmp(name, "vkGetDeviceProcAddr") == 0) return reinterpret_cast<PFN_vkVoidFunction>(GetDeviceProcAddr);
    if (auto f = lookup(kGlobal, sizeof(kGlobal) / sizeof(kGlobal[0]), name)) return f;
    if (!instance) return nullptr;
    if (auto f = lookup(kInstance, sizeof(kInstance) / sizeof(kInstance[0]), name)) return f;
    return lookup(kDevice, sizeof(kDevice) / sizeof(kDevice[0]), name);
}

}  // namespace
}  // namespace cpv::icd

// ----------------------------------------------------------- loader ABI --

extern "C" {

CPV_EXPORT VkResult VKAPI_CALL vk_icdNegotiateLoaderICDInterfaceVersion(uint32_t* version) {
    if (!version) return VK_ERROR_INCOMPATIBLE_DRIVER;
    if (*version > 5) *version = 5;
    return VK_SUCCESS;
}

CPV_EXPORT PFN_vkVoidFunction VKAPI_CALL vk_icdGetInstanceProcAddr(VkInstance instance, const char* name) {
    return cpv::icd::GetInstanceProcAddr(instance, name);
}

CPV_EXPORT PFN_vkVoidFunction VKAPI_CALL vk_icdGetPhysicalDeviceProcAddr(VkInstance, const char*) { return nullptr; }

CPV_EXPORT const char* cpv_last_error(void) { return cpv::rt::last_error(); }

CPV_EXPORT uint64_t cpv_kernel_launches(void) { return cpv::rt::launches(); }

CPV_EXPORT const char* cpv_batch_tuning(void) { return cpv::icd::last_tuning(); }
CPV_EXPORT void cpv_batch_stats(uint64_t out[3]) { cpv::rt::batch_stats(out); }

CPV_EXPORT int cpv_queue_record(VkQueue queue, uint32_t slot) {
    auto* q = reinterpret_cast<cpv::icd::Queue*>(queue);
    if (!q || slot >= 16) return -1;
    if (!q->timing[slot] && cudaEventCreate(&q->timing[slot]) != cudaSuccess) return -1;
    return cudaEventRecord(q->timing[slot], q->stream) == cudaSuccess ? 0 : -1;
}

CPV_EXPORT double cpv_queue_elapsed_ms(VkQueue queue, uint32_t a, uint32_t b) {
    auto* q = reinterpret_cast<cpv::icd::Queue*>(queue);
    if (!q || a >= 16 || b >= 16 || !q->timing[a] || !q->timing[b]) return -1.0;
    if (cudaEventSynchronize(q->timing[b]) != cudaSuccess) return -1.0;
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, q->timing[a], q->timing[b]) != cudaSuccess) return -1.0;
    return ms;
}

CPV_EXPORT uint64_t cpv_queue_scratch_generation(VkQueue queue) {
    auto* q = reinterpret_cast<cpv::icd::Queue*>(queue);
    return q ? q->scratch.generation() : 0;
}

CPV_EXPORT void cpv_profile_enable(int on) { cpv::rt::profile_enable(on != 0); }

CPV_EXPORT int cpv_profile_get(const char* kernel, uint64_t* launches, double* total_ms) { return cpv::rt::profile_get(kernel, launches, total_ms); }

CPV_EXPORT void cpv_profile_reset(void) { cpv::rt::profile_reset(); }

CPV_EXPORT VkResult VKAPI_CALL cpv_queue_submit_no_alloc(VkQueue queue, uint32_t submitCount, const VkSubmitInfo* pSubmits, VkFence fence) {
    using namespace cpv::icd;
    if (!queue || (submitCount && !pSubmits)) {
        cpv::rt::set_last_error("cpv_queue_submit_no_alloc: null queue or submit array");
        return VK_ERROR_INITIALIZATION_FAILED;
    }
    auto* q = reinterpret_cast<Queue*>(queue);
    if (q->device->compile_only) {
        cpv::rt::set_last_error("cpv_queue_submit_no_alloc: compile-only device (no CUDA device)");
        return VK_ERROR_DEVICE_LOST;
    }
    std::string err;
    if (cpv::rt::static_scratch_setup(err) != cpv::rt::kOk) {
        cpv::rt::set_last_error("cpv_queue_submit_no_alloc: " + err);
        return VK_ERROR_INITIALIZATION_FAILED;
    }
    // Reject an oversized draw before any work of the submission is enqueued.
    for (uint32_t i = 0; i < submitCount; i++)
        for (uint32_t k = 0; k < pSubmits[i].commandBufferCount; k++) {
            const VkResult r = check_no_alloc(q, reinterpret_cast<CommandBuffer*>(pSubmits[i].pCommandBuffers[k]));
            if (r != VK_SUCCESS) return r;
        }
    return submit(queue, submitCount, pSubmits, fence, true);
}

CPV_EXPORT int cpv_device_available(void) {
    std::string err;
    return cpv::rt::init(err) == cpv::rt::kOk ? 1 : 0;
}

}  // extern "C"
